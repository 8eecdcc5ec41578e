// raytracer_containment -- strict containment join, drop-in for the reference's
// `raytracer_containment` (query/src/applications/raytracer_containment_main.cpp:96-438,
// query/src/cuda/mesh_containment.cu:76-377): the B objects whose first vertex lies inside
// an A object (odd parity of a +Z ray, t in [1e-4, 1e10]) while no edge of either object
// crosses the other.  Same flags, phases, summary, mesh_containment_results.csv
// (a_object_id,b_object_id[,pair_type]; here containment pairs sorted by (a, b), then the
// overlap pairs sorted when --include-overlap-pairs) and timing JSON.  The reference
// collects both phases in hash tables; the engine runs the overlap join (both edge
// directions into one pair table), the B->A containment rays into another, and removes
// the overlap pairs from the sorted containment list.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include "rs_cli.h"

using namespace rscli;

struct ContainResult {
    std::vector<uint64_t> contained;  // (a << 32 | b), sorted
    std::vector<uint64_t> overlap;    // sorted
};

static std::vector<uint64_t> finalizeKeys(rs_pairset* ps) {
    uint64_t cap = 0, cnt = 0;
    check(rs_pairset_info(ps, &cap, &cnt, nullptr), "rs_pairset_info");
    std::vector<uint64_t> keys;
    if (!cnt) return keys;
    uint64_t* d = nullptr;
    checkCuda(cudaMalloc((void**)&d, cnt * sizeof(uint64_t)), "cudaMalloc");
    uint64_t n = 0;
    check(rs_pairset_finalize(ps, 0, d, cnt, &n, nullptr), "rs_pairset_finalize");
    keys.resize(n);
    if (n) checkCuda(cudaMemcpy(keys.data(), d, n * sizeof(uint64_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
    cudaFree(d);
    return keys;
}

static ContainResult runOnce(rs_bvh* bA, rs_bvh* bB, const DeviceGeometry& dA, const DeviceGeometry& dB,
                             rs_pairset* psO, rs_pairset* psC) {
    ContainResult r;
    // Phase 1 (mesh_containment.cu:76-171): edges of B into A and of A into B, as (a, b).
    check(rs_pairset_clear(psO, nullptr), "rs_pairset_clear");
    check(rs_overlap_join(bA, dA.starts, dA.ends, dA.offsets, dA.counts, dA.sources, dA.nE, bB, dB.starts, dB.ends,
                          dB.offsets, dB.counts, dB.sources, dB.nE, 0, 0, psO, nullptr),
          "rs_overlap_join");
    // Phase 2 (:236-377): one +Z ray per B object against A, parity per A object, as (a, b).
    check(rs_pairset_clear(psC, nullptr), "rs_pairset_clear");
    int st = rs_containment(bA, dB.V, dB.nV, dB.I, dB.nF, dB.T, 1, psC, nullptr);
    if (st == RS_ERR_TABLE_FULL) {
        uint64_t cap = 0, cnt = 0;
        check(rs_pairset_info(psC, &cap, &cnt, nullptr), "rs_pairset_info");
        while (st == RS_ERR_TABLE_FULL) {
            check(rs_pairset_destroy(psC), "rs_pairset_destroy");
            cap *= 4;
            check(rs_pairset_create(cap, 1, &psC, nullptr), "rs_pairset_create");
            st = rs_containment(bA, dB.V, dB.nV, dB.I, dB.nF, dB.T, 1, psC, nullptr);
        }
    }
    check(st, "rs_containment");
    r.overlap = finalizeKeys(psO);
    const std::vector<uint64_t> inside = finalizeKeys(psC);
    std::set_difference(inside.begin(), inside.end(), r.overlap.begin(), r.overlap.end(),
                        std::back_inserter(r.contained));
    return r;
}

int main(int argc, char* argv[]) {
    PerformanceTimer timer;
    timer.start("Data Reading");
    MeshPairOptions opt("containment_timing.json");
    opt.allowNoExport = true;
    opt.parse(argc, argv, {}, {"--use-anyhit-point-in-mesh", "--include-overlap-pairs"});
    if (opt.helpRequested) {
        printHelp(argv[0], "--mesh1 <A_dataset> --mesh2 <B_dataset> [options]",
                  "Containment query: finds pairs where B objects are fully contained in A objects.",
                  {{"--mesh1 <path>", "Dataset A (container meshes)"},
                   {"--mesh2 <path>", "Dataset B (objects tested for containment)"},
                   {"--output <path>", "Path to JSON file for performance timing output"},
                   {"--ptx <path>", "Accepted for compatibility (the engine loads no PTX)"},
                   {"--runs <number>", "Number of measured query runs (default: 1)"},
                   {"--warmup-runs <number>", "Number of warmup iterations (default: 2)"},
                   {"--use-anyhit-point-in-mesh", "Accepted (the engine always collects every crossing in one traversal)"},
                   {"--include-overlap-pairs", "Include overlap/touch pairs in output (union of overlap + strict containment)"},
                   {"--no-export", "Do not export results to CSV"},
                   {"--help, -h", "Show this help message"}});
        return 0;
    }
    opt.sanitizeRunCounts();
    const bool includeOverlap = opt.has("--include-overlap-pairs");
    std::cout << "=== Mesh Containment Query ===" << std::endl;
    std::cout << "(checks which B-objects are fully contained inside A-objects)" << std::endl;
    std::cout << "Point-in-mesh mode: anyhit" << std::endl;
    std::cout << "Include overlap pairs: " << (includeOverlap ? "yes" : "no") << std::endl;
    if (opt.mesh1.empty()) {
        std::cerr << "Error: Mesh1 file path is required. Use --mesh1 <path_to_mesh1_file>" << std::endl;
        return 1;
    }
    if (opt.mesh2.empty()) {
        std::cerr << "Error: Mesh2 file path is required. Use --mesh2 <path_to_mesh2_file>" << std::endl;
        return 1;
    }
    timer.next("Application Creation");
    checkCuda(cudaFree(0), "context creation");
    timer.next("Load Mesh A");
    std::cout << "Loading dataset A from: " << opt.mesh1 << std::endl;
    Geometry gA = loadGeometryFromFile(opt.mesh1);
    if (gA.V.empty() || !requirePrecomputedEdges(gA, opt.mesh1, "Mesh1")) return 1;
    std::cout << "  A: " << gA.numVertices() << " vertices, " << gA.numTriangles() << " triangles" << std::endl;
    timer.next("Load Mesh B");
    std::cout << "Loading dataset B from: " << opt.mesh2 << std::endl;
    Geometry gB = loadGeometryFromFile(opt.mesh2);
    if (gB.V.empty() || !requirePrecomputedEdges(gB, opt.mesh2, "Mesh2")) return 1;
    std::cout << "  B: " << gB.numVertices() << " vertices, " << gB.numTriangles() << " triangles" << std::endl;
    const size_t nA = countDistinctObjects(gA.T), nB = countDistinctObjects(gB.T);
    std::cout << "  A objects: " << nA << "   B objects: " << nB << std::endl;
    DeviceGeometry dA, dB;
    timer.next("Upload Mesh A");
    dA.uploadMesh(gA);
    timer.next("Upload Mesh B");
    dB.uploadMesh(gB);
    rs_bvh *bA = nullptr, *bB = nullptr;
    timer.next("Build A Index");
    check(rs_bvh_build(dA.V, dA.nV, dA.I, dA.nF, dA.T, 0, &bA, nullptr), "rs_bvh_build");
    timer.next("Build B Index");
    check(rs_bvh_build(dB.V, dB.nV, dB.I, dB.nF, dB.T, 0, &bB, nullptr), "rs_bvh_build");
    timer.next("Prepare Kernel Parameters");
    dA.uploadEdges(gA);
    dB.uploadEdges(gB);
    rs_pairset *psO = nullptr, *psC = nullptr;
    check(rs_pairset_create(1 << 20, 1, &psO, nullptr), "rs_pairset_create");
    // __raygen__check_edges (mesh_containment.cu:99-170): t_min moves to the next float after
    // each hit, at most 256 traces per edge.
    check(rs_pairset_set_edge_rule(psO, 256, 1), "rs_pairset_set_edge_rule");
    check(rs_pairset_create(1 << 20, 1, &psC, nullptr), "rs_pairset_create");
    timer.next("Warmup");
    if (opt.warmupRuns > 0) {
        std::cout << "Running " << opt.warmupRuns << " warmup iterations..." << std::endl;
        for (int w = 0; w < opt.warmupRuns; ++w) runOnce(bA, bB, dA, dB, psO, psC);
    }
    timer.next("Query");
    std::cout << "\n=== Executing containment query ===" << std::endl;
    ContainResult res;
    for (int run = 0; run < opt.runs; ++run) {
        res = runOnce(bA, bB, dA, dB, psO, psC);
        if (run == opt.runs - 1) {
            std::cout << "Containment pairs found: " << res.contained.size() << std::endl;
            if (includeOverlap) std::cout << "Overlap/touch pairs found: " << res.overlap.size() << std::endl;
        }
    }
    timer.next("Download Results");
    timer.next("Output");
    std::cout << "\n=== Containment Query Summary ===" << std::endl;
    std::cout << "A triangles: " << gA.numTriangles() << "  objects: " << nA << std::endl;
    std::cout << "B triangles: " << gB.numTriangles() << "  objects: " << nB << std::endl;
    std::cout << "Containment pairs (B in A): " << res.contained.size() << std::endl;
    if (includeOverlap) {
        std::cout << "Overlap/Touch pairs (A vs B): " << res.overlap.size() << std::endl;
        std::cout << "Reported pairs: " << (res.contained.size() + res.overlap.size()) << std::endl;
    }
    if (opt.exportResults) {
        const std::string csvFile = "mesh_containment_results.csv";
        std::cout << "Exporting results to " << csvFile << std::endl;
        std::ofstream csv(csvFile);
        auto row = [&](uint64_t k) { csv << (int32_t)(k >> 32) << "," << (int32_t)(k & 0xffffffffu); };
        if (includeOverlap) {
            csv << "a_object_id,b_object_id,pair_type\n";
            for (uint64_t k : res.contained) {
                row(k);
                csv << ",containment\n";
            }
            for (uint64_t k : res.overlap) {
                row(k);
                csv << ",overlap\n";
            }
        } else {
            csv << "a_object_id,b_object_id\n";
            for (uint64_t k : res.contained) {
                row(k);
                csv << "\n";
            }
        }
    }
    timer.next("Cleanup");
    rs_pairset_destroy(psO);
    rs_pairset_destroy(psC);
    rs_bvh_destroy(bA);
    rs_bvh_destroy(bB);
    dA.release();
    dB.release();
    timer.finish(opt.output);
    std::cout << "\nContainment query completed successfully." << std::endl;
    return 0;
}
