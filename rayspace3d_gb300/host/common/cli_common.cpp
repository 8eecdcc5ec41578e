// cli_common.cpp -- shared host code of the drop-in executables (see rs_cli.h).
#include <algorithm>
#include <cmath>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <set>
#include <sstream>
#include <unordered_map>

#include <cuda_runtime.h>

#include "rs_cli.h"

namespace rscli {

namespace {
constexpr uint32_t kMagic = 0x52334442;  // "R3DB"

template <class T>
bool readArray(std::ifstream& in, std::vector<T>& v, uint64_t count) {
    v.resize(count);
    if (count == 0) return true;
    in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(count * sizeof(T)));
    return static_cast<bool>(in);
}
}  // namespace

Geometry loadGeometryFromFile(const std::string& path) {
    std::cout << "=== Loading Preprocessed Geometry (Binary) ===" << std::endl;
    Geometry g;
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        std::cerr << "Error: Could not open file for reading: " << path << std::endl;
        return g;
    }
    uint32_t magic = 0, version = 0;
    in.read(reinterpret_cast<char*>(&magic), 4);
    in.read(reinterpret_cast<char*>(&version), 4);
    if (!in || magic != kMagic) {
        std::cerr << "Error: Invalid file format (Magic mismatch). File: " << path << std::endl;
        return g;
    }
    uint64_t nV = 0, nI = 0, nM = 0, nE = 0, nES = 0, total = 0;
    uint8_t hasGrid = 0, hasEdges = 0;
    if (version == 2) {
        uint64_t h[6];
        uint8_t flags[8];
        in.read(reinterpret_cast<char*>(h), sizeof(h));
        in.read(reinterpret_cast<char*>(flags), sizeof(flags));
        nV = h[0], nI = h[1], nM = h[2], nE = h[3], nES = h[4], total = h[5];
        hasGrid = flags[0];
        hasEdges = flags[1];
    } else if (version == 1) {
        uint64_t h[4];
        uint8_t flags[8];
        in.read(reinterpret_cast<char*>(h), sizeof(h));
        in.read(reinterpret_cast<char*>(flags), sizeof(flags));
        nV = h[0], nI = h[1], nM = h[2], total = h[3];
        hasGrid = flags[0];
    } else {
        std::cerr << "Error: Unsupported binary geometry version " << version << " in file: " << path
                  << ". Expected version 2. Re-run preprocessing." << std::endl;
        return g;
    }
    Geometry out;
    out.totalTriangles = total;
    bool ok = in && readArray(in, out.V, 3 * nV) && readArray(in, out.I, 3 * nI) && readArray(in, out.T, nM);
    if (ok && hasEdges) {
        ok = readArray(in, out.starts, 3 * nE) && readArray(in, out.ends, 3 * nE) && readArray(in, out.offsets, nE) &&
             readArray(in, out.counts, nE) && readArray(in, out.sources, nES);
    }
    if (ok && hasGrid) {
        float b[6];
        uint32_t r[4];
        in.read(reinterpret_cast<char*>(b), sizeof(b));
        in.read(reinterpret_cast<char*>(r), sizeof(r));
        ok = static_cast<bool>(in);
        if (ok) {
            out.hasGrid = true;
            for (int k = 0; k < 3; ++k) {
                out.gmin[k] = b[k];
                out.gmax[k] = b[3 + k];
                out.res[k] = r[k];
            }
            ok = readArray(in, out.cells, (uint64_t)r[0] * r[1] * r[2]);
        }
    }
    if (!ok) {
        std::cerr << "Error: Truncated geometry file: " << path << std::endl;
        return g;
    }
    return out;
}

bool requirePrecomputedEdges(const Geometry& g, const std::string& path, const char* label) {
    if (g.hasEdges()) return true;
    std::cerr << "Error: " << label << " loaded from '" << path << "' does not contain precomputed edges."
              << std::endl;
    std::cerr << "Re-run preprocess_dataset to regenerate the .pre file with embedded edge payload." << std::endl;
    return false;
}

bool writeBinaryFile(const std::string& path, const Geometry& g) {
    std::ofstream out(path, std::ios::binary);
    if (!out) {
        std::cerr << "Error: Could not open file for writing: " << path << std::endl;
        return false;
    }
    const bool edges = g.hasEdges();
    uint32_t head[2] = {kMagic, 2};
    uint64_t h[6] = {g.numVertices(), g.numTriangles(), (uint64_t)g.T.size(), edges ? g.numEdges() : 0,
                     edges ? (uint64_t)g.sources.size() : 0, g.totalTriangles};
    uint8_t flags[8] = {(uint8_t)(g.hasGrid ? 1 : 0), (uint8_t)(edges ? 1 : 0), 0, 0, 0, 0, 0, 0};
    out.write(reinterpret_cast<const char*>(head), sizeof(head));
    out.write(reinterpret_cast<const char*>(h), sizeof(h));
    out.write(reinterpret_cast<const char*>(flags), sizeof(flags));
    auto put = [&](const void* p, size_t bytes) {
        if (bytes) out.write(reinterpret_cast<const char*>(p), (std::streamsize)bytes);
    };
    put(g.V.data(), g.V.size() * sizeof(float));
    put(g.I.data(), g.I.size() * sizeof(uint32_t));
    put(g.T.data(), g.T.size() * sizeof(int32_t));
    if (edges) {
        put(g.starts.data(), g.starts.size() * sizeof(float));
        put(g.ends.data(), g.ends.size() * sizeof(float));
        put(g.offsets.data(), g.offsets.size() * sizeof(int32_t));
        put(g.counts.data(), g.counts.size() * sizeof(int32_t));
        put(g.sources.data(), g.sources.size() * sizeof(int32_t));
    }
    if (g.hasGrid) {
        float b[6] = {g.gmin[0], g.gmin[1], g.gmin[2], g.gmax[0], g.gmax[1], g.gmax[2]};
        uint32_t r[4] = {g.res[0], g.res[1], g.res[2], 0};
        put(b, sizeof(b));
        put(r, sizeof(r));
        if (g.cells.size() != (size_t)g.res[0] * g.res[1] * g.res[2])
            std::cerr << "Warning: Grid cell count mismatch in write!" << std::endl;
        put(g.cells.data(), g.cells.size() * sizeof(GridCellH));
    }
    out.close();
    return static_cast<bool>(out);
}

std::vector<std::string> splitPaths(const std::string& input) {
    std::vector<std::string> out;
    std::stringstream ss(input);
    std::string item;
    while (std::getline(ss, item, ',')) {
        const size_t a = item.find_first_not_of(" \t");
        const size_t b = item.find_last_not_of(" \t");
        if (a != std::string::npos) out.push_back(item.substr(a, b - a + 1));
    }
    return out;
}

int countDistinctObjects(const std::vector<int32_t>& t2o) {
    std::set<int32_t> s(t2o.begin(), t2o.end());
    return (int)s.size();
}

// ---------------------------------------------------------------------------
// PerformanceTimer (query/src/timer.cpp): phase list + manual measurements + counters.
// ---------------------------------------------------------------------------
void PerformanceTimer::start(const std::string& phase) {
    phases_.clear();
    manual_.clear();
    counters_.clear();
    total_start_ = clock::now();
    running_ = true;
    finished_ = false;
    Phase p;
    p.name = phase;
    p.start = total_start_;
    phases_.push_back(p);
}

void PerformanceTimer::endCurrent() {
    if (!phases_.empty() && !phases_.back().ended) {
        phases_.back().end = clock::now();
        phases_.back().us =
            std::chrono::duration_cast<std::chrono::microseconds>(phases_.back().end - phases_.back().start).count();
        phases_.back().ended = true;
    }
}

void PerformanceTimer::next(const std::string& phase) {
    if (!running_) {
        std::cerr << "Timer not started! Call start() first." << std::endl;
        return;
    }
    endCurrent();
    Phase p;
    p.name = phase;
    p.start = clock::now();
    phases_.push_back(p);
}

void PerformanceTimer::addMeasurement(const std::string& phase, long long us) {
    Phase p;
    p.name = phase;
    p.us = us;
    p.ended = true;
    manual_.push_back(p);
}

void PerformanceTimer::addCounter(const std::string& name, unsigned long long value) {
    counters_.emplace_back(name, value);
}

long long PerformanceTimer::getTotalDuration() const {
    if (!finished_) return -1;
    return std::chrono::duration_cast<std::chrono::microseconds>(total_end_ - total_start_).count();
}

void PerformanceTimer::finish(const std::string& filename) {
    if (!running_) {
        std::cerr << "Timer not started! Call start() first." << std::endl;
        return;
    }
    endCurrent();
    total_end_ = clock::now();
    running_ = false;
    finished_ = true;
    std::cout << "\n=== Detailed Performance Summary ===" << std::endl;
    for (const auto* list : {&phases_, &manual_})
        for (const auto& p : *list)
            std::cout << std::left << std::setw(30) << (p.name + ":") << std::right << std::setw(20) << p.us
                      << " microseconds (" << std::fixed << std::setprecision(2) << (double)p.us / 1000.0 << " ms)"
                      << std::endl;
    if (!counters_.empty()) {
        std::cout << "\n=== Profiling Counters ===" << std::endl;
        for (const auto& c : counters_)
            std::cout << std::left << std::setw(30) << (c.first + ":") << std::right << std::setw(20) << c.second
                      << std::endl;
    }
    const long long total = getTotalDuration();
    if (total > 0)
        std::cout << std::left << std::setw(25) << "Total Execution Time:" << std::right << std::setw(10) << total
                  << " microseconds (" << std::fixed << std::setprecision(2) << (double)total / 1000.0 << " ms)"
                  << std::endl;
    std::cout.unsetf(std::ios::floatfield);
    writeResults(filename);
}

static std::string lower(const std::string& s) {
    std::string out;
    out.reserve(s.size());
    for (char c : s) out.push_back((char)std::tolower((unsigned char)c));
    return out;
}

void PerformanceTimer::writeResults(const std::string& filename) const {
    std::ofstream f(filename);
    if (!f) {
        std::cerr << "Warning: Could not write timing results to file." << std::endl;
        return;
    }
    f << "{\n  \"phases\": {\n";
    std::unordered_map<std::string, int> seen;
    std::vector<const Phase*> all;
    for (const auto& p : phases_) all.push_back(&p);
    for (const auto& p : manual_) all.push_back(&p);
    for (size_t i = 0; i < all.size(); ++i) {
        const std::string ln = lower(all[i]->name);
        const int k = ++seen[ln];
        f << "    \"" << ln << "_" << k << "\": {\n";
        f << "      \"duration_us\": " << all[i]->us << ",\n";
        f << "      \"duration_ms\": " << std::fixed << std::setprecision(2) << (double)all[i]->us / 1000.0 << "\n";
        f << "    }" << (i + 1 < all.size() ? "," : "") << "\n";
    }
    f << "  },\n";
    if (writeCounters) {
        f << "  \"counters\": {\n";
        for (size_t i = 0; i < counters_.size(); ++i)
            f << "    \"" << lower(counters_[i].first) << "\": " << counters_[i].second
              << (i + 1 < counters_.size() ? "," : "") << "\n";
        f << "  },\n";
    }
    const long long total = getTotalDuration();
    if (total > 0) {
        f << "  \"total\": {\n    \"duration_us\": " << total << ",\n    \"duration_ms\": " << std::fixed
          << std::setprecision(2) << (double)total / 1000.0 << "\n  }\n";
    } else {
        f << "  \"total\": null\n";
    }
    f << "}\n";
    std::cout << "Performance timing written to " << filename << std::endl;
}

// ---------------------------------------------------------------------------
void checkCuda(int err, const char* what) {
    if (err != cudaSuccess) {
        std::cerr << "CUDA error in " << what << ": " << cudaGetErrorString((cudaError_t)err) << std::endl;
        std::exit(EXIT_FAILURE);
    }
}

void check(int status, const char* what) {
    if (status != RS_OK) {
        std::cerr << "Engine error in " << what << ": " << rs_status_string(status) << " (" << status << ")"
                  << std::endl;
        std::exit(EXIT_FAILURE);
    }
}

template <class T>
static T* upload(const std::vector<T>& v) {
    T* d = nullptr;
    if (v.empty()) return nullptr;
    checkCuda(cudaMalloc((void**)&d, v.size() * sizeof(T)), "cudaMalloc");
    checkCuda(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
    return d;
}

void DeviceGeometry::uploadMesh(const Geometry& g) {
    V = upload(g.V);
    I = upload(g.I);
    T = upload(g.T);
    nV = g.numVertices();
    nF = g.numTriangles();
}

void DeviceGeometry::uploadEdges(const Geometry& g) {
    starts = upload(g.starts);
    ends = upload(g.ends);
    offsets = upload(g.offsets);
    counts = upload(g.counts);
    sources = upload(g.sources);
    nE = g.numEdges();
    nS = g.sources.size();
}

void DeviceGeometry::uploadGrid(const Geometry& g) {
    if (!g.hasGrid) return;
    cells = upload(g.cells);
    nCells = g.cells.size();
}

void DeviceGeometry::release() {
    for (void* p : {(void*)V, (void*)I, (void*)T, (void*)starts, (void*)ends, (void*)offsets, (void*)counts,
                    (void*)sources, cells})
        if (p) cudaFree(p);
    *this = DeviceGeometry();
}

Estimate estimatePairs(const Geometry& g1, const Geometry& g2, const DeviceGeometry& d1, const DeviceGeometry& d2,
                       float epsilon, float gamma, bool alphaCorrection) {
    Estimate est;
    if (!g1.hasGrid || !g2.hasGrid) return est;
    // Cell volume from mesh1's grid (raytracer_overlap_estimated_main.cpp:256-262).
    const float w = g1.gmax[0] - g1.gmin[0], h = g1.gmax[1] - g1.gmin[1], dpt = g1.gmax[2] - g1.gmin[2];
    const float csX = w / g1.res[0], csY = h / g1.res[1], csZ = dpt / g1.res[2];
    const float cellVolume = csX * csY * csZ;
    const uint64_t numCells = (uint64_t)g1.res[0] * g1.res[1] * g1.res[2];
    if (g1.cells.size() != numCells || g2.cells.size() != numCells || !d1.cells || !d2.cells) return est;
    double raw = 0.0;
    float means[4];
    check(rs_estimate_grid(d1.cells, d2.cells, numCells, cellVolume, epsilon, gamma, &raw, means, nullptr),
          "rs_estimate_grid");
    est.ok = true;
    est.raw = (float)raw;
    est.avgSize1 = means[0];
    est.volRatio1 = means[1];
    est.avgSize2 = means[2];
    est.volRatio2 = means[3];
    est.eff1 = est.avgSize1 * std::cbrt(est.volRatio1);
    est.eff2 = est.avgSize2 * std::cbrt(est.volRatio2);
    if (alphaCorrection) {
        const float cs = est.eff1 + est.eff2;
        const float mv = cs * cs * cs;
        const float cv = cellVolume < 1e-9f ? 1e-9f : cellVolume;
        est.alpha = mv / cv;
        if (est.alpha < 1.0f) est.alpha = 1.0f;
    }
    est.pairs = rs_estimate_pairs_from_raw(raw, means, cellVolume, alphaCorrection ? 1 : 0);
    return est;
}

long long microsSince(std::chrono::high_resolution_clock::time_point t0) {
    return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::high_resolution_clock::now() - t0)
        .count();
}

void MeshPairOptions::parse(int argc, char** argv, const std::vector<std::string>& valued,
                            const std::vector<std::string>& plain) {
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--help" || a == "-h") {
            helpRequested = true;
        } else if (a == "--mesh1" && i + 1 < argc) {
            mesh1 = argv[++i];
        } else if (a == "--mesh2" && i + 1 < argc) {
            mesh2 = argv[++i];
        } else if (a == "--output" && i + 1 < argc) {
            output = argv[++i];
        } else if (a == "--ptx" && i + 1 < argc) {
            ptx = argv[++i];  // accepted for compatibility; the engine loads no PTX
        } else if (allowRuns && a == "--runs" && i + 1 < argc) {
            runs = std::atoi(argv[++i]);
        } else if (allowRuns && a == "--warmup-runs" && i + 1 < argc) {
            warmupRuns = std::atoi(argv[++i]);
        } else if (allowNoExport && a == "--no-export") {
            exportResults = false;
        } else if (std::find(valued.begin(), valued.end(), a) != valued.end() && i + 1 < argc) {
            extra.emplace_back(a, argv[++i]);
        } else if (std::find(plain.begin(), plain.end(), a) != plain.end()) {
            extra.emplace_back(a, "");
        }
    }
}

bool MeshPairOptions::has(const std::string& flag) const {
    for (const auto& kv : extra)
        if (kv.first == flag) return true;
    return false;
}

std::string MeshPairOptions::get(const std::string& flag, const std::string& def) const {
    std::string v = def;
    for (const auto& kv : extra)
        if (kv.first == flag) v = kv.second;  // last occurrence wins, like the reference parsers
    return v;
}

void MeshPairOptions::sanitizeRunCounts() {
    if (runs < 1) runs = 1;
    if (warmupRuns < 0) warmupRuns = 0;
}

void printHelp(const char* exe, const std::string& usage, const std::string& description,
               const std::vector<std::pair<std::string, std::string>>& options) {
    std::cout << "Usage: " << exe << " " << usage << std::endl;
    if (!description.empty()) std::cout << description << std::endl;
    std::cout << "Options:" << std::endl;
    for (const auto& o : options) std::cout << "  " << std::left << std::setw(34) << o.first << o.second << std::endl;
}

}  // namespace rscli
