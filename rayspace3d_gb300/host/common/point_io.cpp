// point_io.cpp -- WKT / "x y z" point files (query/src/runtime/PointIO.cpp:12-72), parsed
// in parallel with the reference's exact per-line semantics.  No CUDA dependency, so the
// tests can compile it alone.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <thread>
#include <vector>

#include "rs_cli.h"

namespace rscli {

// One fgets() segment of PointIO.cpp:33-62: up to 1023 characters, or through the newline.
static void parsePointSegment(char* line, std::vector<float>& pts) {
    char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (*p == '\0' || *p == '\r' || *p == '\n' || *p == '#') return;
    if (std::strncmp(p, "POINT", 5) == 0) {
        char* s = std::strchr(p, '(');
        if (s) {
            ++s;
            char* e;
            const float x = std::strtof(s, &e);
            const float y = std::strtof(e, &e);
            const float z = std::strtof(e, &e);
            pts.push_back(x);
            pts.push_back(y);
            pts.push_back(z);
        }
    } else if ((*p >= '0' && *p <= '9') || *p == '-') {
        char* e;
        const float x = std::strtof(p, &e);
        const float y = std::strtof(e, &e);
        const float z = std::strtof(e, &e);
        if (p != e) {
            pts.push_back(x);
            pts.push_back(y);
            pts.push_back(z);
        }
    }
}

// Parses text[begin, end) (whole lines) exactly as the reference's fgets loop would.
static void parsePointRange(const char* text, size_t begin, size_t end, std::vector<float>& pts) {
    char seg[1024];
    size_t i = begin;
    while (i < end) {
        size_t n = 0;
        while (i < end && n < 1023) {
            const char c = text[i++];
            seg[n++] = c;
            if (c == '\n') break;
        }
        seg[n] = '\0';
        parsePointSegment(seg, pts);
    }
}

std::vector<float> loadPointDataset(const std::string& path) {
    std::vector<float> pts;
    if (path.empty()) {
        std::cout << "No point dataset provided, using default test points" << std::endl;
        return {0.0f, 0.0f, -1.0f, 0.5f, 0.5f, -1.0f, 1.0f, 1.0f, -1.0f};
    }
    std::cout << "=== Loading Point Dataset ===" << std::endl;
    std::cout << "Loading points from: " << path << std::endl;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::cerr << "Error: Could not open point dataset file: " << path << std::endl;
        return pts;
    }
    std::vector<char> text;
    {
        std::fseek(f, 0, SEEK_END);
        const long size = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        text.resize(size > 0 ? (size_t)size : 0);
        if (size > 0 && std::fread(text.data(), 1, text.size(), f) != text.size()) text.clear();
    }
    std::fclose(f);
    // Chunks end at newlines (where every fgets segment sequence restarts) and are parsed
    // in parallel, then concatenated in file order.
    const size_t nthreads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const size_t parts = text.size() < (1u << 20) ? 1 : nthreads;
    std::vector<size_t> cut(parts + 1, text.size());
    cut[0] = 0;
    for (size_t k = 1; k < parts; ++k) {
        size_t c = std::max(cut[k - 1], text.size() * k / parts);
        while (c < text.size() && text[c - 1] != '\n') ++c;
        cut[k] = c;
    }
    std::vector<std::vector<float>> out(parts);
    std::vector<std::thread> th;
    for (size_t k = 0; k < parts; ++k)
        th.emplace_back([&, k]() {
            out[k].reserve((cut[k + 1] - cut[k]) / 8);
            parsePointRange(text.data(), cut[k], cut[k + 1], out[k]);
        });
    for (auto& t : th) t.join();
    size_t total = 0;
    for (auto& v : out) total += v.size();
    pts.reserve(total);
    for (auto& v : out) pts.insert(pts.end(), v.begin(), v.end());
    std::cout << "Found " << pts.size() / 3 << " points." << std::endl;
    return pts;
}

}  // namespace rscli
