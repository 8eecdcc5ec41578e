// raytracer_mesh_overlap -- edge-ray overlap join, drop-in for the reference's
// `raytracer_mesh_overlap` (query/src/applications/rayspace_mesh_overlap_main.cpp:252-495):
// same flags, phases, summary, mesh_overlap_results.csv (object_id_mesh1,object_id_mesh2,
// sorted by (object_id_mesh2, object_id_mesh1) like the reference's u64 sort of
// MeshQueryResult) and timing JSON.  The reference counts, scans, writes and sorts in two
// passes per direction; the engine traces each edge once into a pair table, so its manual
// measurements are Raytrace_Mesh1ToMesh2, Raytrace_Mesh2ToMesh1 and Deduplication.
#include <cuda_runtime.h>

#include <chrono>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rs_cli.h"

using namespace rscli;
using clk = std::chrono::high_resolution_clock;

struct JoinResult {
    std::vector<uint64_t> keys;
    long long a2b_us = 0, b2a_us = 0, dedup_us = 0;
};

static JoinResult runJoin(rs_bvh* b1, rs_bvh* b2, const DeviceGeometry& d1, const DeviceGeometry& d2,
                          rs_pairset* ps, uint64_t** dKeys, uint64_t* dCap) {
    JoinResult r;
    check(rs_pairset_clear(ps, nullptr), "rs_pairset_clear");
    auto t0 = clk::now();
    int st = rs_edge_join(b2, d1.starts, d1.ends, d1.offsets, d1.counts, d1.sources, d1.nE, 0, ps, nullptr);
    r.a2b_us = microsSince(t0);
    if (st == RS_OK) {
        t0 = clk::now();
        st = rs_edge_join(b1, d2.starts, d2.ends, d2.offsets, d2.counts, d2.sources, d2.nE, 1, ps, nullptr);
        r.b2a_us = microsSince(t0);
    }
    if (st == RS_ERR_TABLE_FULL) {  // grow the table and rerun both directions
        check(rs_overlap_join(b1, d1.starts, d1.ends, d1.offsets, d1.counts, d1.sources, d1.nE, b2, d2.starts,
                              d2.ends, d2.offsets, d2.counts, d2.sources, d2.nE, 0, 0, ps, nullptr),
              "rs_overlap_join");
    } else {
        check(st, "rs_edge_join");
    }
    t0 = clk::now();
    uint64_t cap = 0, cnt = 0;
    check(rs_pairset_info(ps, &cap, &cnt, nullptr), "rs_pairset_info");
    if (cnt > *dCap) {
        if (*dKeys) cudaFree(*dKeys);
        checkCuda(cudaMalloc((void**)dKeys, cnt * sizeof(uint64_t)), "cudaMalloc");
        *dCap = cnt;
    }
    uint64_t n = 0;
    check(rs_pairset_finalize(ps, 1, *dKeys, *dCap, &n, nullptr), "rs_pairset_finalize");
    r.dedup_us = microsSince(t0);
    r.keys.resize(n);
    if (n) checkCuda(cudaMemcpy(r.keys.data(), *dKeys, n * sizeof(uint64_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
    return r;
}

int main(int argc, char* argv[]) {
    PerformanceTimer timer;
    timer.start("Data Reading");
    MeshPairOptions opt("mesh_overlap_timing.json");
    opt.allowNoExport = true;
    opt.parse(argc, argv, {}, {});
    if (opt.helpRequested) {
        printHelp(argv[0], "[--mesh1 <path>] [--mesh2 <path>] [--output <json_output_file>] [--runs <number>] [--ptx <ptx_file>]",
                  "Mesh overlap join query for reporting overlapping object pairs between two datasets.",
                  {{"--mesh1 <path>", "Path to first mesh dataset (geometry file)"},
                   {"--mesh2 <path>", "Path to second mesh dataset (geometry file)"},
                   {"--output <path>", "Path to JSON file for performance timing output"},
                   {"--ptx <path>", "Accepted for compatibility (the engine loads no PTX)"},
                   {"--runs <number>", "Number of measured query runs (default: 1)"},
                   {"--warmup-runs <number>", "Number of warmup iterations (default: 2)"},
                   {"--no-export", "Do not export results to CSV"},
                   {"--help, -h", "Show this help message"}});
        return 0;
    }
    opt.sanitizeRunCounts();
    std::cout << "Mesh-to-Mesh Overlap Join" << std::endl;
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
    timer.next("Load Mesh1");
    std::cout << "Loading Mesh1 from: " << opt.mesh1 << std::endl;
    Geometry g1 = loadGeometryFromFile(opt.mesh1);
    if (g1.V.empty()) {
        std::cerr << "Error: Failed to load Mesh1 from " << opt.mesh1 << std::endl;
        return 1;
    }
    if (!requirePrecomputedEdges(g1, opt.mesh1, "Mesh1")) return 1;
    std::cout << "Mesh1 loaded: " << g1.numVertices() << " vertices, " << g1.numTriangles() << " triangles" << std::endl;
    timer.next("Load Mesh2");
    std::cout << "Loading Mesh2 from: " << opt.mesh2 << std::endl;
    Geometry g2 = loadGeometryFromFile(opt.mesh2);
    if (g2.V.empty()) {
        std::cerr << "Error: Failed to load Mesh2 from " << opt.mesh2 << std::endl;
        return 1;
    }
    if (!requirePrecomputedEdges(g2, opt.mesh2, "Mesh2")) return 1;
    std::cout << "Mesh2 loaded: " << g2.numVertices() << " vertices, " << g2.numTriangles() << " triangles" << std::endl;
    DeviceGeometry d1, d2;
    timer.next("Upload Mesh1");
    d1.uploadMesh(g1);
    std::cout << "Mesh1 uploaded to GPU" << std::endl;
    timer.next("Upload Mesh2");
    d2.uploadMesh(g2);
    std::cout << "Mesh2 uploaded to GPU" << std::endl;
    rs_bvh *b1 = nullptr, *b2 = nullptr;
    timer.next("Build Mesh1 Index");
    check(rs_bvh_build(d1.V, d1.nV, d1.I, d1.nF, d1.T, 0, &b1, nullptr), "rs_bvh_build");
    std::cout << "Mesh1 acceleration structure built" << std::endl;
    timer.next("Build Mesh2 Index");
    check(rs_bvh_build(d2.V, d2.nV, d2.I, d2.nF, d2.T, 0, &b2, nullptr), "rs_bvh_build");
    std::cout << "Mesh2 acceleration structure built" << std::endl;
    timer.next("Upload Mesh1");
    d1.uploadEdges(g1);
    std::cout << "Mesh1 edges uploaded: " << d1.nE << " unique edges" << std::endl;
    timer.next("Upload Mesh2");
    d2.uploadEdges(g2);
    std::cout << "Mesh2 edges uploaded: " << d2.nE << " unique edges" << std::endl;
    timer.next("Create Launcher");
    rs_pairset* ps = nullptr;
    check(rs_pairset_create(1 << 20, 1, &ps, nullptr), "rs_pairset_create");
    timer.next("Prepare Kernel Parameters");
    uint64_t* dKeys = nullptr;
    uint64_t dCap = 0;
    timer.next("Warmup");
    if (opt.warmupRuns > 0) {
        std::cout << "Running " << opt.warmupRuns << " warmup iterations (edge rays)..." << std::endl;
        for (int w = 0; w < opt.warmupRuns; ++w) runJoin(b1, b2, d1, d2, ps, &dKeys, &dCap);
    }
    timer.next("Query");
    std::cout << "\n=== Executing mesh overlap detection (edge rays) ===" << std::endl;
    JoinResult res = runJoin(b1, b2, d1, d2, ps, &dKeys, &dCap);
    timer.addMeasurement("Raytrace_Mesh1ToMesh2", res.a2b_us);
    timer.addMeasurement("Raytrace_Mesh2ToMesh1", res.b2a_us);
    timer.addMeasurement("Deduplication", res.dedup_us);
    std::cout << "Deduplication: Found " << res.keys.size() << " unique object pairs." << std::endl;
    timer.next("Download Results");
    timer.next("Output");
    std::cout << "\n=== Mesh Overlap Join Summary ===" << std::endl;
    std::cout << "Mesh1 triangles: " << g1.numTriangles() << std::endl;
    std::cout << "Mesh1 objects: " << countDistinctObjects(g1.T) << std::endl;
    std::cout << "Mesh2 triangles: " << g2.numTriangles() << std::endl;
    std::cout << "Mesh2 objects: " << countDistinctObjects(g2.T) << std::endl;
    std::cout << "Mesh1 Universe Min: [" << g1.gmin[0] << ", " << g1.gmin[1] << ", " << g1.gmin[2] << "]" << std::endl;
    std::cout << "Mesh1 Universe Max: [" << g1.gmax[0] << ", " << g1.gmax[1] << ", " << g1.gmax[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Min: [" << g2.gmin[0] << ", " << g2.gmin[1] << ", " << g2.gmin[2] << "]" << std::endl;
    std::cout << "Mesh2 Universe Max: [" << g2.gmax[0] << ", " << g2.gmax[1] << ", " << g2.gmax[2] << "]" << std::endl;
    std::cout << "Unique object pairs: " << res.keys.size() << std::endl;
    if (opt.exportResults) {
        std::cout << "Exporting results to mesh_overlap_results.csv" << std::endl;
        std::ofstream csv("mesh_overlap_results.csv");
        csv << "object_id_mesh1,object_id_mesh2\n";
        for (uint64_t k : res.keys) csv << (int32_t)(k >> 32) << "," << (int32_t)(k & 0xffffffffu) << "\n";
    }
    timer.next("Cleanup");
    if (dKeys) cudaFree(dKeys);
    rs_pairset_destroy(ps);
    rs_bvh_destroy(b1);
    rs_bvh_destroy(b2);
    d1.release();
    d2.release();
    timer.finish(opt.output);
    return 0;
}
