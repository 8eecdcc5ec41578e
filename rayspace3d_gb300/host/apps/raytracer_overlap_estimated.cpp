// raytracer_overlap_estimated -- grid-estimated hash overlap join, drop-in for the
// reference's `raytracer_overlap_estimated`
// (query/src/applications/raytracer_overlap_estimated_main.cpp:160-488).  Compiled with
// RS_DIRECT it is `raytracer_overlap_direct_estimation`
// (raytracer_overlap_direct_estimation_main.cpp:221-690): --query-direction,
// --pairs-output, --track-hash-contention, --no-alpha-correction, --hash-table-size,
// --hash-table-free-mem-fraction and odd (non power of two) table sizes.
// Differences by design: a table that fills up grows and the query reruns instead of
// dropping keys, and exported pairs are sorted by (object_id_mesh1, object_id_mesh2).
#include <cuda_runtime.h>

#include <chrono>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "rs_cli.h"

#ifndef RS_DIRECT
#define RS_DIRECT 0
#endif

using namespace rscli;
using clk = std::chrono::high_resolution_clock;

int main(int argc, char* argv[]) {
    PerformanceTimer timer;
    MeshPairOptions opt("estimated_overlap_timing.json");
    std::vector<std::string> valued = {"--gamma", "--epsilon"};
    std::vector<std::string> plain = {"--estimate-only"};
    if (RS_DIRECT) {
        valued.insert(valued.end(), {"--query-direction", "--pairs-output", "--hash-table-size",
                                     "--hash-table-free-mem-fraction"});
        plain.insert(plain.end(), {"--track-hash-contention", "--no-alpha-correction"});
    }
    opt.parse(argc, argv, valued, plain);
    if (opt.helpRequested) {
        std::vector<std::pair<std::string, std::string>> o = {
            {"--mesh1 <path>", "Path to first mesh dataset (geometry file)"},
            {"--mesh2 <path>", "Path to second mesh dataset (geometry file)"},
            {"--output <path>", "Path to JSON file for performance timing output"},
            {"--ptx <path>", "Accepted for compatibility (the engine loads no PTX)"},
            {"--runs <number>", "Number of measured query runs (default: 1)"},
            {"--warmup-runs <number>", "Number of warmup iterations (default: 2)"},
            {"--gamma <float>", "Gamma parameter for estimation (default: 0.8)"},
            {"--epsilon <float>", "Epsilon parameter for estimation (default: 0.001)"}};
        if (RS_DIRECT) {
            o.push_back({"--query-direction <d>", "Query direction: both|mesh1_to_mesh2|mesh2_to_mesh1 (default: both)"});
            o.push_back({"--pairs-output <path>", "Optional CSV export path for unique result pairs"});
            o.push_back({"--track-hash-contention", "Track hash accesses and contention rate"});
            o.push_back({"--no-alpha-correction", "Disable replication-factor alpha correction for estimated pairs"});
            o.push_back({"--hash-table-size <ull>", "Override hash table size (slots); 0 = auto-compute"});
            o.push_back({"--hash-table-free-mem-fraction <f>", "Use f in (0,1] of free GPU memory for hash table sizing"});
        }
        o.push_back({"--estimate-only", "Only run selectivity estimation, skip actual query"});
        o.push_back({"--help, -h", "Show this help message"});
        printHelp(argv[0], "--mesh1 <path> --mesh2 <path> [options]",
                  RS_DIRECT ? "Overlap direct-estimation query with optional pair export and hash contention diagnostics."
                            : "Overlap estimated query using selectivity estimation plus hash-based refinement.",
                  o);
        return 0;
    }
    opt.sanitizeRunCounts();
    const float gamma = std::stof(opt.get("--gamma", "0.8"));
    const float epsilon = std::stof(opt.get("--epsilon", "0.001"));
    const bool estimateOnly = opt.has("--estimate-only");
    const std::string dirArg = opt.get("--query-direction", "both");
    int direction = 0;
    if (dirArg == "mesh1_to_mesh2") direction = 1;
    else if (dirArg == "mesh2_to_mesh1") direction = 2;
    else if (dirArg != "both") {
        std::cerr << "Error: Invalid --query-direction value: " << dirArg
                  << ". Expected one of: both, mesh1_to_mesh2, mesh2_to_mesh1" << std::endl;
        return 1;
    }
    const std::string pairsOutput = opt.get("--pairs-output", "");
    const bool trackContention = opt.has("--track-hash-contention");
    const bool alphaCorrection = !opt.has("--no-alpha-correction");
    const unsigned long long manualSize = std::stoull(opt.get("--hash-table-size", "0"));
    const float freeMemFraction = std::stof(opt.get("--hash-table-free-mem-fraction", "0"));
    if (!opt.mesh1.size() || !opt.mesh2.size()) {
        std::cerr << "Usage: " << argv[0] << " --mesh1 <path> --mesh2 <path> [options]" << std::endl;
        return 1;
    }
    if (RS_DIRECT && (freeMemFraction < 0.0f || freeMemFraction > 1.0f)) {
        std::cerr << "Error: --hash-table-free-mem-fraction must be in [0, 1]." << std::endl;
        return 1;
    }

    timer.start("Load Mesh1");
    Geometry g1 = loadGeometryFromFile(opt.mesh1);
    if (g1.V.empty()) {
        std::cerr << "Error loading mesh1." << std::endl;
        return 1;
    }
    if (!requirePrecomputedEdges(g1, opt.mesh1, "Mesh1")) return 1;
    timer.next("Load Mesh2");
    Geometry g2 = loadGeometryFromFile(opt.mesh2);
    if (g2.V.empty()) {
        std::cerr << "Error loading mesh2." << std::endl;
        return 1;
    }
    if (!requirePrecomputedEdges(g2, opt.mesh2, "Mesh2")) return 1;

    DeviceGeometry d1, d2;
    auto estimate = [&](bool verbose) -> long long {
        if (!g1.hasGrid || !g2.hasGrid) {
            if (verbose) std::cout << "Skipping estimation: Grid data not found." << std::endl;
            return 0;
        }
        if (!d1.cells) d1.uploadGrid(g1);
        if (!d2.cells) d2.uploadGrid(g2);
        const Estimate e = estimatePairs(g1, g2, d1, d2, epsilon, gamma, alphaCorrection);
        if (!e.ok) {
            if (verbose) std::cerr << "Error: Grid mismatch. Skipping estimation." << std::endl;
            return 0;
        }
        if (verbose) {
            std::cout << (RS_DIRECT ? "\n=== Selectivity Estimation (Overlap - Direct) ===" : "\n=== Selectivity Estimation (Overlap) ===")
                      << std::endl;
            std::cout << "Raw Potential Pairs:       " << (long long)e.raw << std::endl;
            std::cout << "Avg Object Size (Mesh1):   " << e.avgSize1 << std::endl;
            std::cout << "Avg Object Size (Mesh2):   " << e.avgSize2 << std::endl;
            std::cout << "Avg VolRatio (Mesh1):      " << e.volRatio1 << std::endl;
            std::cout << "Avg VolRatio (Mesh2):      " << e.volRatio2 << std::endl;
            std::cout << "Effective Size (Mesh1):    " << e.eff1 << std::endl;
            std::cout << "Effective Size (Mesh2):    " << e.eff2 << std::endl;
            if (RS_DIRECT) std::cout << "Alpha Correction Enabled:  " << (alphaCorrection ? "yes" : "no") << std::endl;
            std::cout << "Replication Factor (alpha):" << e.alpha << std::endl;
            std::cout << "Final Estimated Pairs:     " << e.pairs << std::endl;
            std::cout << "==============================\n" << std::endl;
        }
        return e.pairs;
    };
    // Table size: raytracer_overlap_estimated_main.cpp:316-325 (power of two) or
    // raytracer_overlap_direct_estimation_main.cpp:438-466 (manual, free-memory fraction, odd).
    auto tableSize = [&](long long est, bool& pow2) -> unsigned long long {
        pow2 = !RS_DIRECT;
        if (!RS_DIRECT) return rs_hash_size_pow2(est);
        if (manualSize > 0) return manualSize;
        if (freeMemFraction > 0.0f) {
            size_t freeB = 0, totalB = 0;
            if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess && freeB > 0) {
                unsigned long long slots = (unsigned long long)(freeMemFraction * (double)freeB) / 8ull;
                if (slots < 1024ull) slots = 1024ull;
                if (slots % 2ull == 0ull) slots += 1ull;
                return slots;
            }
            std::cerr << "Warning: cudaMemGetInfo failed for free-memory hash sizing. Falling back to estimate-based sizing."
                      << std::endl;
        }
        unsigned long long size = 16777216ull;
        if (est > 0) {
            unsigned long long target = (unsigned long long)(est / 0.5);
            if (target < 1024) target = 1024;
            if (target > 2147483648ull) target = 2147483648ull;
            size = target;
            if (size % 2 == 0) size++;
        }
        return size;
    };

    if (estimateOnly) {
        timer.next("Selectivity Estimation");
        (void)estimate(true);
        timer.finish(opt.output);
        return 0;
    }
    timer.next("Init OptiX");
    checkCuda(cudaFree(0), "context creation");
    timer.next("Upload Mesh1");
    d1.uploadMesh(g1);
    timer.next("Upload Mesh2");
    d2.uploadMesh(g2);
    rs_bvh *b1 = nullptr, *b2 = nullptr;
    timer.next("Build Mesh1 Index");
    check(rs_bvh_build(d1.V, d1.nV, d1.I, d1.nF, d1.T, 0, &b1, nullptr), "rs_bvh_build");
    timer.next("Build Mesh2 Index");
    check(rs_bvh_build(d2.V, d2.nV, d2.I, d2.nF, d2.T, 0, &b2, nullptr), "rs_bvh_build");
    if (RS_DIRECT) {
        timer.next("Upload Mesh1 Edges");
        d1.uploadEdges(g1);
        std::cout << "Mesh1 edges uploaded: " << d1.nE << " unique edges" << std::endl;
        timer.next("Upload Mesh2 Edges");
        d2.uploadEdges(g2);
        std::cout << "Mesh2 edges uploaded: " << d2.nE << " unique edges" << std::endl;
        timer.next("Create Edge Launcher");
    }
    timer.next("Prepare Kernel Parameters");
    if (!RS_DIRECT) {
        d1.uploadEdges(g1);
        d2.uploadEdges(g2);
    }
    rs_pairset* ps = nullptr;
    unsigned long long psSize = 0;
    bool psPow2 = true;
    uint64_t* dKeys = nullptr;
    uint64_t dCap = 0;
    std::vector<uint64_t> hostKeys;
    unsigned long long accesses = 0, contentions = 0;

    auto hashQuery = [&](long long est, bool verbose, bool timed) {
        bool pow2 = true;
        const unsigned long long size = tableSize(est, pow2);
        if (verbose) {
            if (!RS_DIRECT) std::cout << "Using Power-of-Two Hash Table Size (bitwise opt): " << size << std::endl;
            else if (manualSize > 0) std::cout << "Using Manual Hash Table Size: " << size << std::endl;
            else if (freeMemFraction > 0.0f) std::cout << "Using Free GPU Memory Hash Table Size: " << size << std::endl;
            else std::cout << "Using Direct Estimated Hash Table Size: " << size << std::endl;
        }
        if (!ps || size != psSize || pow2 != psPow2) {
            if (ps) rs_pairset_destroy(ps);
            check(rs_pairset_create(size, pow2 ? 1 : 0, &ps, nullptr), "rs_pairset_create");
            psSize = size;
            psPow2 = pow2;
        }
        rs_pairset_set_tracking(ps, trackContention ? 1 : 0);
        check(rs_pairset_clear(ps, nullptr), "rs_pairset_clear");
        int st = RS_OK;
        if (direction == 0 || direction == 1) {
            const auto t0 = clk::now();
            st = rs_edge_join(b2, d1.starts, d1.ends, d1.offsets, d1.counts, d1.sources, d1.nE, 0, ps, nullptr);
            if (timed) timer.addMeasurement("Raytrace_Hash_Mesh1ToMesh2", microsSince(t0));
        }
        if (st == RS_OK && (direction == 0 || direction == 2)) {
            const auto t0 = clk::now();
            st = rs_edge_join(b1, d2.starts, d2.ends, d2.offsets, d2.counts, d2.sources, d2.nE, 1, ps, nullptr);
            if (timed) timer.addMeasurement("Raytrace_Hash_Mesh2ToMesh1", microsSince(t0));
        }
        if (st == RS_ERR_TABLE_FULL) {
            if (verbose) std::cout << "Pair table full: growing it and rerunning the query" << std::endl;
            check(rs_overlap_join(b1, d1.starts, d1.ends, d1.offsets, d1.counts, d1.sources, d1.nE, b2, d2.starts,
                                  d2.ends, d2.offsets, d2.counts, d2.sources, d2.nE, direction, 0, ps, nullptr),
                  "rs_overlap_join");
        } else {
            check(st, "rs_edge_join");
        }
        const auto t0 = clk::now();
        uint64_t cap = 0, cnt = 0;
        check(rs_pairset_info(ps, &cap, &cnt, nullptr), "rs_pairset_info");
        if (cnt > dCap) {
            if (dKeys) cudaFree(dKeys);
            checkCuda(cudaMalloc((void**)&dKeys, cnt * sizeof(uint64_t)), "cudaMalloc");
            dCap = cnt;
        }
        uint64_t n = 0;
        check(rs_pairset_finalize(ps, 0, dKeys, dCap, &n, nullptr), "rs_pairset_finalize");
        if (timed) timer.addMeasurement("compact_hash_table_pairs", microsSince(t0));
        if (trackContention) {
            uint64_t c[8];
            check(rs_pairset_counters(ps, c, nullptr), "rs_pairset_counters");
            accesses = c[0];
            contentions = c[1];
        }
        if (verbose) std::cout << "Hash Table Query found " << n << " unique pairs." << std::endl;
        return n;
    };

    timer.next("Warmup");
    if (opt.warmupRuns > 0) {
        std::cout << "Running " << opt.warmupRuns << " warmup iterations (estimation + hash query)..." << std::endl;
        for (int w = 0; w < opt.warmupRuns; ++w) hashQuery(estimate(false), false, false);
    }
    uint64_t finalUnique = 0;
    for (int run = 0; run < opt.runs; ++run) {
        const bool verbose = run == 0;
        timer.next("Selectivity Estimation");
        const long long est = estimate(verbose);
        timer.next("Execute Hash Query");
        const uint64_t n = hashQuery(est, verbose, true);
        timer.next("Download Results");
        hostKeys.resize(n);
        if (n) checkCuda(cudaMemcpy(hostKeys.data(), dKeys, n * sizeof(uint64_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
        finalUnique = n;
        if (trackContention) {
            const double pct = accesses ? 100.0 * (double)contentions / (double)accesses : 0.0;
            std::cout << std::fixed << std::setprecision(2) << "Hash contention (run " << (run + 1)
                      << "): " << contentions << "/" << accesses << " accesses (" << pct << "%)" << std::endl;
            std::cout.unsetf(std::ios::floatfield);
        }
    }
    timer.next("Cleanup");
    if (dKeys) cudaFree(dKeys);
    if (ps) rs_pairset_destroy(ps);
    rs_bvh_destroy(b1);
    rs_bvh_destroy(b2);
    d1.release();
    d2.release();
    std::cout << "\n=== Mesh Overlap Join Summary ===" << std::endl;
    if (RS_DIRECT) {
        std::cout << "Query direction: " << dirArg << std::endl;
        std::cout << "Hash contention tracking: " << (trackContention ? "enabled" : "disabled") << std::endl;
    }
    std::cout << "Mesh1 triangles: " << g1.numTriangles() << std::endl;
    std::cout << "Mesh1 objects: " << countDistinctObjects(g1.T) << std::endl;
    std::cout << "Mesh2 triangles: " << g2.numTriangles() << std::endl;
    std::cout << "Mesh2 objects: " << countDistinctObjects(g2.T) << std::endl;
    std::cout << "Mesh1 Universe Min: [" << g1.gmin[0] << ", " << g1.gmin[1] << ", " << g1.gmin[2] << "]" << std::endl;
    std::cout << "Mesh1 Universe Max: [" << g1.gmax[0] << ", " << g1.gmax[1] << ", " << g1.gmax[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Min: [" << g2.gmin[0] << ", " << g2.gmin[1] << ", " << g2.gmin[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Max: [" << g2.gmax[0] << ", " << g2.gmax[1] << ", " << g2.gmax[2] << "]" << std::endl;
    std::cout << "Unique object pairs: " << finalUnique << std::endl;
    if (RS_DIRECT && !pairsOutput.empty()) {
        std::ofstream csv(pairsOutput);
        if (!csv.is_open()) {
            std::cerr << "Warning: Failed to open pairs output file: " << pairsOutput << std::endl;
        } else {
            csv << "object_id_mesh1,object_id_mesh2\n";
            for (uint64_t k : hostKeys) csv << (int32_t)(k >> 32) << "," << (int32_t)(k & 0xffffffffu) << "\n";
            std::cout << "Pair results written to: " << pairsOutput << std::endl;
        }
    }
    timer.finish(opt.output);
    std::cout << "\nQuery completed in " << (double)timer.getTotalDuration() / 1000.0 << " ms." << std::endl;
    std::cout << "Results saved to: " << opt.output << std::endl;
    return 0;
}
