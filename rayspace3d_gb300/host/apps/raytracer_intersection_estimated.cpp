// raytracer_intersection_estimated -- full intersection (edge-ray overlap plus containment
// fallback) with grid-estimated hash sizing, drop-in for the reference's
// `raytracer_intersection_estimated` (query/src/applications/raytracer_intersection_estimated_main.cpp:212-760):
// same flags, phases, manual measurements, counters, intersection_pairs.csv
// (a_object_id,b_object_id; here sorted by (a, b)), intersection_pair_hits.csv and
// intersection_containment_tracking.csv.  --overlap-max-iterations caps the hits each
// edge ray takes (rs_pairset_set_edge_rule), as in trace_edge_multi_hits
// (mesh_intersection.cu:16-91).  --containment-max-iterations and --use-anyhit-containment
// are accepted: the reference always runs the any-hit containment path
// (useAnyhitContainment is never false, raytracer_intersection_estimated_main.cpp:227,280),
// which ignores the iteration cap, and the engine's containment ray likewise collects every
// crossing in one traversal, so the tracking CSV reports one iteration per ray.
#include <cuda_runtime.h>

#include <chrono>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rs_cli.h"

using namespace rscli;
using clk = std::chrono::high_resolution_clock;

int main(int argc, char* argv[]) {
    PerformanceTimer timer;
    MeshPairOptions opt("estimated_intersection_timing.json");
    opt.allowRuns = false;  // this executable takes no --runs / --warmup-runs / --no-export
    opt.parse(argc, argv,
              {"--gamma", "--epsilon", "--query-direction", "--overlap-max-iterations", "--containment-max-iterations",
               "--hash-load-factor", "--pairs-output", "--pair-hits-output", "--containment-tracking-output"},
              {"--estimate-only", "--use-anyhit-containment", "--enable-profiling-stats"});
    if (opt.helpRequested) {
        printHelp(argv[0], "--mesh1 <path> --mesh2 <path> [options]",
                  "Intersection estimated query: overlap plus containment passes with hash-based deduplication.",
                  {{"--mesh1 <path>", "Path to first mesh dataset (geometry file)"},
                   {"--mesh2 <path>", "Path to second mesh dataset (geometry file)"},
                   {"--output <path>", "Path to JSON file for performance timing output"},
                   {"--ptx <path>", "Accepted for compatibility (the engine loads no PTX)"},
                   {"--gamma <float>", "Estimation gamma (default: 0.8)"},
                   {"--epsilon <float>", "Estimation epsilon (default: 0.001)"},
                   {"--estimate-only", "Run only selectivity estimation"},
                   {"--query-direction <both|mesh1_to_mesh2|mesh2_to_mesh1>", "Control query direction (default: both)"},
                   {"--overlap-max-iterations <int>", "Overlap ray iteration cap (default: 100)"},
                   {"--containment-max-iterations <int>",
                    "Accepted (the any-hit containment path, always on, has no iteration cap)"},
                   {"--use-anyhit-containment", "Accepted (the engine's containment is the any-hit path)"},
                   {"--hash-load-factor <float>", "Hash load factor in (0,1] (default: 0.5)"},
                   {"--enable-profiling-stats", "Enable device-side profiling counters"},
                   {"--pairs-output <path>", "Intersection pairs CSV path (default: intersection_pairs.csv)"},
                   {"--pair-hits-output <path>", "Pair hit tracking CSV path (default: intersection_pair_hits.csv)"},
                   {"--containment-tracking-output <path>",
                    "Containment tracking CSV path (default: intersection_containment_tracking.csv)"},
                   {"--help, -h", "Show this help message"}});
        return 0;
    }
    const float gamma = std::stof(opt.get("--gamma", "0.8"));
    const float epsilon = std::stof(opt.get("--epsilon", "0.001"));
    const bool estimateOnly = opt.has("--estimate-only");
    const bool profiling = opt.has("--enable-profiling-stats");
    const float loadFactor = std::stof(opt.get("--hash-load-factor", "0.5"));
    const int overlapMax = std::stoi(opt.get("--overlap-max-iterations", "100"));
    const int containmentMax = std::stoi(opt.get("--containment-max-iterations", "1024"));
    std::string pairsPath = opt.get("--pairs-output", "");
    std::string hitsPath = opt.get("--pair-hits-output", "");
    std::string trackPath = opt.get("--containment-tracking-output", "");
    if (pairsPath.empty()) pairsPath = "intersection_pairs.csv";
    if (hitsPath.empty()) hitsPath = "intersection_pair_hits.csv";
    if (trackPath.empty()) trackPath = "intersection_containment_tracking.csv";
    const std::string dirArg = opt.get("--query-direction", "both");
    int direction = 0;
    if (dirArg == "mesh1_to_mesh2") direction = 1;
    else if (dirArg == "mesh2_to_mesh1") direction = 2;
    else if (dirArg != "both") {
        std::cerr << "Invalid query direction: " << dirArg << std::endl;
        std::cerr << "Valid values for --query-direction are: both, mesh1_to_mesh2, mesh2_to_mesh1" << std::endl;
        return 1;
    }
    if (loadFactor <= 0.0f || loadFactor > 1.0f) {
        std::cerr << "Invalid --hash-load-factor. Expected value in (0, 1]." << std::endl;
        return 1;
    }
    if (overlapMax <= 0 || containmentMax <= 0) {
        std::cerr << "Iteration limits must be > 0." << std::endl;
        return 1;
    }
    if (opt.mesh1.empty() || opt.mesh2.empty()) {
        std::cerr << "Usage: " << argv[0] << " --mesh1 <path> --mesh2 <path> [options]" << std::endl;
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

    timer.next("Selectivity Estimation");
    DeviceGeometry d1, d2;
    long long estimated = 0;
    if (g1.hasGrid && g2.hasGrid) {
        if (g1.res[0] != g2.res[0] || g1.gmin[0] != g2.gmin[0] || g1.gmax[0] != g2.gmax[0])
            std::cerr << "Warning: Grid parameters (resolution/bounds) mismatch. Estimation may be invalid." << std::endl;
        d1.uploadGrid(g1);
        d2.uploadGrid(g2);
        const Estimate e = estimatePairs(g1, g2, d1, d2, epsilon, gamma, true);
        if (e.ok) {
            estimated = e.pairs;
            std::cout << "\n=== Selectivity Estimation ===" << std::endl;
            std::cout << "Raw Potential Pairs:       " << (long long)e.raw << std::endl;
            std::cout << "Avg Object Size (Mesh1):   " << e.avgSize1 << std::endl;
            std::cout << "Avg Object Size (Mesh2):   " << e.avgSize2 << std::endl;
            std::cout << "Avg VolRatio (Mesh1):      " << e.volRatio1 << std::endl;
            std::cout << "Avg VolRatio (Mesh2):      " << e.volRatio2 << std::endl;
            std::cout << "Effective Size (Mesh1):    " << e.eff1 << std::endl;
            std::cout << "Effective Size (Mesh2):    " << e.eff2 << std::endl;
            std::cout << "Replication Factor (alpha):" << e.alpha << std::endl;
            std::cout << "Final Estimated Pairs:     " << e.pairs << std::endl;
            std::cout << "==============================\n" << std::endl;
        } else {
            std::cerr << "Error: Grid has " << g1.cells.size() << "/" << g2.cells.size() << " cells, expected "
                      << (uint64_t)g1.res[0] * g1.res[1] * g1.res[2] << ". Skipping estimation." << std::endl;
        }
    } else {
        std::cout << "Skipping estimation: Grid data not found in one or both datasets." << std::endl;
        std::cout << "Run preprocess_dataset with --generate-grid to enable estimation." << std::endl;
    }
    if (estimateOnly) {
        timer.finish(opt.output);
        return 0;
    }
    const unsigned long long tableSize = rs_hash_size_odd(estimated, loadFactor);
    std::cout << "\n=== Query Configuration ===" << std::endl;
    std::cout << "Estimated Pairs:    " << estimated << std::endl;
    std::cout << "Hash Table Size:    " << tableSize << " (Load Factor ~" << loadFactor << ")" << std::endl;
    std::cout << "Query Direction:    " << dirArg << std::endl;
    std::cout << "Overlap Max Iter:   " << overlapMax << std::endl;
    std::cout << "Contain Max Iter:   " << containmentMax << std::endl;
    std::cout << "Profiling Stats:    " << (profiling ? "enabled" : "disabled") << std::endl;
    std::cout << "===========================\n" << std::endl;

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
    timer.next("Prepare Kernel Parameters");
    d1.uploadEdges(g1);
    d2.uploadEdges(g2);
    rs_pairset* ps = nullptr;
    check(rs_pairset_create(tableSize, 0, &ps, nullptr), "rs_pairset_create");
    rs_pairset_set_tracking(ps, profiling ? 1 : 0);
    check(rs_pairset_set_edge_rule(ps, overlapMax, 0), "rs_pairset_set_edge_rule");
    // Per-source tracking buffers (PairHitTracking.h: 256 targets per source).
    constexpr int kMaxTargets = 256;
    int32_t maxObj1 = -1, maxObj2 = -1;
    for (int32_t o : g1.T) maxObj1 = std::max(maxObj1, o);
    for (int32_t o : g2.T) maxObj2 = std::max(maxObj2, o);
    const uint64_t n1 = (uint64_t)(maxObj1 + 1), n2 = (uint64_t)(maxObj2 + 1);
    int32_t *tid1 = nullptr, *tid2 = nullptr;
    uint32_t *thit1 = nullptr, *thit2 = nullptr, *cand1 = nullptr, *cand2 = nullptr;
    checkCuda(cudaMalloc(&tid1, std::max<uint64_t>(n1, 1) * kMaxTargets * 4), "cudaMalloc");
    checkCuda(cudaMalloc(&thit1, std::max<uint64_t>(n1, 1) * kMaxTargets * 4), "cudaMalloc");
    checkCuda(cudaMalloc(&cand1, std::max<uint64_t>(n1, 1) * 4), "cudaMalloc");
    checkCuda(cudaMalloc(&tid2, std::max<uint64_t>(n2, 1) * kMaxTargets * 4), "cudaMalloc");
    checkCuda(cudaMalloc(&thit2, std::max<uint64_t>(n2, 1) * kMaxTargets * 4), "cudaMalloc");
    checkCuda(cudaMalloc(&cand2, std::max<uint64_t>(n2, 1) * 4), "cudaMalloc");
    checkCuda(cudaMemset(tid1, 0xff, std::max<uint64_t>(n1, 1) * kMaxTargets * 4), "cudaMemset");
    checkCuda(cudaMemset(tid2, 0xff, std::max<uint64_t>(n2, 1) * kMaxTargets * 4), "cudaMemset");
    checkCuda(cudaMemset(thit1, 0, std::max<uint64_t>(n1, 1) * kMaxTargets * 4), "cudaMemset");
    checkCuda(cudaMemset(thit2, 0, std::max<uint64_t>(n2, 1) * kMaxTargets * 4), "cudaMemset");
    checkCuda(cudaMemset(cand1, 0, std::max<uint64_t>(n1, 1) * 4), "cudaMemset");
    checkCuda(cudaMemset(cand2, 0, std::max<uint64_t>(n2, 1) * 4), "cudaMemset");

    timer.next("Query");
    std::cout << "Running Intersection Query..." << std::endl;
    const bool a2b = direction == 0 || direction == 1, b2a = direction == 0 || direction == 2;
    uint64_t numUnique = 0;
    uint64_t* dKeys = nullptr;
    for (int attempt = 0; attempt < 8; ++attempt) {
        check(rs_pairset_clear(ps, nullptr), "rs_pairset_clear");
        int st = RS_OK;
        auto t0 = clk::now();
        if (a2b) {
            st = rs_edge_join(b2, d1.starts, d1.ends, d1.offsets, d1.counts, d1.sources, d1.nE, 0, ps, nullptr);
            timer.addMeasurement("Raytrace_Overlap_Hash_Mesh1ToMesh2", microsSince(t0));
        }
        if (st == RS_OK && b2a) {
            t0 = clk::now();
            st = rs_edge_join(b1, d2.starts, d2.ends, d2.offsets, d2.counts, d2.sources, d2.nE, 1, ps, nullptr);
            timer.addMeasurement("Raytrace_Overlap_Hash_Mesh2ToMesh1", microsSince(t0));
        }
        if (st == RS_OK && a2b) {
            t0 = clk::now();
            st = rs_containment_tracked(b2, d1.V, d1.nV, d1.I, d1.nF, d1.T, 0, ps, kMaxTargets, tid1, thit1, cand1,
                                        n1, nullptr);
            timer.addMeasurement("Raytrace_Containment_Hash_Mesh1ToMesh2", microsSince(t0));
        }
        if (st == RS_OK && b2a) {
            t0 = clk::now();
            st = rs_containment_tracked(b1, d2.V, d2.nV, d2.I, d2.nF, d2.T, 1, ps, kMaxTargets, tid2, thit2, cand2,
                                        n2, nullptr);
            timer.addMeasurement("Raytrace_Containment_Hash_Mesh2ToMesh1", microsSince(t0));
        }
        if (st == RS_ERR_TABLE_FULL) {
            // The reference drops keys here; the engine grows the table and reruns the query.
            uint64_t cap = 0, cnt = 0;
            rs_pairset_info(ps, &cap, &cnt, nullptr);
            rs_pairset_destroy(ps);
            check(rs_pairset_create(cap * 4 + 1, 0, &ps, nullptr), "rs_pairset_create");
            rs_pairset_set_tracking(ps, profiling ? 1 : 0);
            check(rs_pairset_set_edge_rule(ps, overlapMax, 0), "rs_pairset_set_edge_rule");
            std::cout << "Pair table full: growing it to " << (cap * 4 + 1) << " slots and rerunning" << std::endl;
            continue;
        }
        check(st, "query");
        t0 = clk::now();
        uint64_t cap = 0, cnt = 0;
        check(rs_pairset_info(ps, &cap, &cnt, nullptr), "rs_pairset_info");
        checkCuda(cudaMalloc((void**)&dKeys, std::max<uint64_t>(cnt, 1) * sizeof(uint64_t)), "cudaMalloc");
        check(rs_pairset_finalize(ps, 0, dKeys, cnt, &numUnique, nullptr), "rs_pairset_finalize");
        timer.addMeasurement("compact_hash_table_pairs", microsSince(t0));
        break;
    }
    std::cout << "Hash Table Query found " << numUnique << " unique pairs." << std::endl;
    std::cout << "Actual Intersection Pairs: " << numUnique << std::endl;
    timer.addCounter("Profile_Actual_Intersection_Pairs", numUnique);
    std::cout << "Mesh1 Universe Min: [" << g1.gmin[0] << ", " << g1.gmin[1] << ", " << g1.gmin[2] << "]" << std::endl;
    std::cout << "Mesh1 Universe Max: [" << g1.gmax[0] << ", " << g1.gmax[1] << ", " << g1.gmax[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Min: [" << g2.gmin[0] << ", " << g2.gmin[1] << ", " << g2.gmin[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Max: [" << g2.gmax[0] << ", " << g2.gmax[1] << ", " << g2.gmax[2] << "]" << std::endl;

    std::vector<uint64_t> keys(numUnique);
    if (numUnique) checkCuda(cudaMemcpy(keys.data(), dKeys, numUnique * 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
    {
        std::ofstream out(pairsPath);
        if (!out.is_open()) {
            std::cerr << "Failed to open intersection pairs output: " << pairsPath << std::endl;
            return 1;
        }
        out << "a_object_id,b_object_id\n";
        for (uint64_t k : keys) out << (int32_t)(k >> 32) << ',' << (int32_t)(k & 0xffffffffu) << "\n";
    }
    auto fetch = [](const void* d, uint64_t n) {
        std::vector<uint32_t> h(n);
        if (n) checkCuda(cudaMemcpy(h.data(), d, n * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
        return h;
    };
    const std::vector<uint32_t> ht1 = fetch(tid1, n1 * kMaxTargets), hh1 = fetch(thit1, n1 * kMaxTargets),
                                hc1 = fetch(cand1, n1), ht2 = fetch(tid2, n2 * kMaxTargets),
                                hh2 = fetch(thit2, n2 * kMaxTargets), hc2 = fetch(cand2, n2);
    {
        std::ofstream out(hitsPath);
        if (!out.is_open()) {
            std::cerr << "Failed to open pair hit tracking output: " << hitsPath << std::endl;
            return 1;
        }
        out << "direction,source_object_id,target_object_id,target_ray_hits\n";
        for (uint64_t s = 0; a2b && s < n1; ++s)
            for (int j = 0; j < kMaxTargets; ++j) {
                const int32_t t = (int32_t)ht1[s * kMaxTargets + j];
                if (t >= 0) out << "mesh1_to_mesh2," << s << ',' << t << ',' << hh1[s * kMaxTargets + j] << "\n";
            }
        for (uint64_t s = 0; b2a && s < n2; ++s)
            for (int j = 0; j < kMaxTargets; ++j) {
                const int32_t t = (int32_t)ht2[s * kMaxTargets + j];
                if (t >= 0) out << "mesh2_to_mesh1," << s << ',' << t << ',' << hh2[s * kMaxTargets + j] << "\n";
            }
    }
    {
        std::ofstream out(trackPath);
        if (!out.is_open()) {
            std::cerr << "Failed to open containment tracking output: " << trackPath << std::endl;
            return 1;
        }
        out << "direction,source_object_id,iterations,candidate_count,candidate_overflow_events\n";
        for (uint64_t s = 0; s < n1; ++s) out << "mesh1_to_mesh2," << s << ',' << (a2b ? 1 : 0) << ',' << hc1[s] << ",0\n";
        for (uint64_t s = 0; s < n2; ++s) out << "mesh2_to_mesh1," << s << ',' << (b2a ? 1 : 0) << ',' << hc2[s] << ",0\n";
    }
    std::cout << "Intersection pairs CSV: " << pairsPath << std::endl;
    std::cout << "Pair hit tracking CSV: " << hitsPath << std::endl;
    std::cout << "Containment tracking CSV: " << trackPath << std::endl;
    if (profiling) {
        uint64_t c[8];
        check(rs_pairset_counters(ps, c, nullptr), "rs_pairset_counters");
        timer.addCounter("Profile_Overlap_Trace_Calls", c[2]);
        timer.addCounter("Profile_Overlap_Iterations_Total", c[2]);
        timer.addCounter("Profile_Overlap_Hits_Total", c[3]);
        timer.addCounter("Profile_Containment_Rays_Total", c[4]);
        timer.addCounter("Profile_Containment_Iterations_Total", c[4]);
        timer.addCounter("Profile_Containment_Hits_Total", c[5]);
        timer.addCounter("Profile_Containment_Candidate_Additions", c[6]);
        timer.addCounter("Profile_Containment_Candidate_Overflow", 0);
        timer.addCounter("Profile_Overlap_Avg_Iterations_x1000", c[2] ? 1000ull : 0ull);
        timer.addCounter("Profile_Containment_Avg_Iterations_x1000", c[4] ? 1000ull : 0ull);
    }
    timer.next("Cleanup");
    for (void* p : {(void*)tid1, (void*)tid2, (void*)thit1, (void*)thit2, (void*)cand1, (void*)cand2, (void*)dKeys})
        if (p) cudaFree(p);
    rs_pairset_destroy(ps);
    rs_bvh_destroy(b1);
    rs_bvh_destroy(b2);
    d1.release();
    d2.release();
    timer.finish(opt.output);
    return 0;
}
