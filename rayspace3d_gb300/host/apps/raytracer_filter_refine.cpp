// raytracer_filter_refine -- bounding-box filter + point-in-mesh refine, drop-in for the
// reference's `raytracer_filter_refine` (query/src/applications/rayspace_filter_refine_main.cpp:20-170):
// same flags, phases, summary, ray_results.csv (original point id, polygon id; refine
// hits, here in ascending point order) and timing JSON.  The filter (parity against the
// 12-triangle box of all vertices) and the refine run fused in one launch.
#include <cuda_runtime.h>

#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rs_cli.h"

using namespace rscli;

int main(int argc, char* argv[]) {
    PerformanceTimer timer;
    timer.start("Data Reading");
    std::string geometryPath, pointsPath, outputJson = "performance_timing_filter_refine.json", ptx;
    int runs = 1, warmupRuns = 2;
    bool exportResults = true;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--geometry" && i + 1 < argc) geometryPath = argv[++i];
        else if (a == "--points" && i + 1 < argc) pointsPath = argv[++i];
        else if (a == "--output" && i + 1 < argc) outputJson = argv[++i];
        else if (a == "--ptx" && i + 1 < argc) ptx = argv[++i];
        else if (a == "--runs" && i + 1 < argc) runs = std::atoi(argv[++i]);
        else if (a == "--warmup-runs" && i + 1 < argc) warmupRuns = std::atoi(argv[++i]);
        else if (a == "--no-export") exportResults = false;
        else if (a == "--help" || a == "-h") {
            std::cout << "Usage: " << argv[0] << " --geometry <path> --points <path> [options]" << std::endl;
            std::cout << "Options:" << std::endl;
            std::cout << "  --geometry <path>     Path to preprocessed geometry file" << std::endl;
            std::cout << "  --points <path>       Path to WKT file containing POINT geometries." << std::endl;
            std::cout << "  --output <path>       Path to JSON file for performance timing output" << std::endl;
            std::cout << "  --runs <number>       Number of times to run the query (for performance testing)" << std::endl;
            std::cout << "  --warmup-runs <num>   Number of warmup runs (default: 2)" << std::endl;
            std::cout << "  --no-export           Disable CSV export of results" << std::endl;
            std::cout << "  --ptx <ptx_file>      Accepted for compatibility (the engine loads no PTX)" << std::endl;
            std::cout << "  --help, -h            Show this help message" << std::endl;
            return 0;
        }
    }
    (void)runs;
    (void)warmupRuns;
    std::cout << "RaySpace3D GB300 engine: filter-refine point-in-mesh" << std::endl;
    if (geometryPath.empty()) {
        std::cerr << "Error: Geometry file path is required. Use --geometry <path_to_geometry_file>" << std::endl;
        return 1;
    }
    if (pointsPath.empty()) {
        std::cerr << "Error: Points file path is required. Use --points <path_to_point_file>" << std::endl;
        return 1;
    }
    std::cout << "Loading geometry from: " << geometryPath << std::endl;
    Geometry geometry = loadGeometryFromFile(geometryPath);
    if (geometry.V.empty()) {
        std::cerr << "Error: Failed to load geometry from " << geometryPath << std::endl;
        return 1;
    }
    std::cout << "Geometry loaded: " << geometry.numVertices() << " vertices, " << geometry.numTriangles()
              << " triangles" << std::endl;
    std::cout << "Loading points from: " << pointsPath << std::endl;
    std::vector<float> points = loadPointDataset(pointsPath);
    const uint64_t n = points.size() / 3;
    if (n == 0) {
        std::cerr << "Error: Failed to load points from " << pointsPath << std::endl;
        return 1;
    }
    std::cout << "Points loaded: " << n << std::endl;

    timer.next("Application Creation");
    checkCuda(cudaFree(0), "context creation");
    float mn[3] = {3.40282347e38f, 3.40282347e38f, 3.40282347e38f}, mx[3] = {-3.40282347e38f, -3.40282347e38f, -3.40282347e38f};
    for (uint64_t v = 0; v < geometry.numVertices(); ++v)
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::min(mn[k], geometry.V[3 * v + k]);
            mx[k] = std::max(mx[k], geometry.V[3 * v + k]);
        }
    std::cout << "\nQuery bounding box computed:" << std::endl;
    std::cout << "  Min: (" << mn[0] << ", " << mn[1] << ", " << mn[2] << ")" << std::endl;
    std::cout << "  Max: (" << mx[0] << ", " << mx[1] << ", " << mx[2] << ")" << std::endl;

    timer.next("Filter-Refine Execution");
    DeviceGeometry dg;
    dg.uploadMesh(geometry);
    rs_bvh* bvh = nullptr;
    check(rs_bvh_build(dg.V, dg.nV, dg.I, dg.nF, dg.T, 0, &bvh, nullptr), "rs_bvh_build");
    float* dPoints = nullptr;
    int32_t *dObj = nullptr, *dIds = nullptr, *dHitObj = nullptr;
    checkCuda(cudaMalloc(&dPoints, points.size() * sizeof(float)), "cudaMalloc");
    checkCuda(cudaMemcpy(dPoints, points.data(), points.size() * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
    checkCuda(cudaMalloc(&dObj, n * sizeof(int32_t)), "cudaMalloc");
    checkCuda(cudaMalloc(&dIds, n * sizeof(int32_t)), "cudaMalloc");
    checkCuda(cudaMalloc(&dHitObj, n * sizeof(int32_t)), "cudaMalloc");
    check(rs_pim_filtered(bvh, dPoints, n, 0.0f, 0.0f, 1.0f, dObj, nullptr, nullptr), "rs_pim_filtered");
    uint64_t inside = 0;
    check(rs_compact_hits(dObj, n, dIds, dHitObj, n, &inside, nullptr), "rs_compact_hits");
    std::vector<int32_t> ids(inside), objs(inside);
    if (inside) {
        checkCuda(cudaMemcpy(ids.data(), dIds, inside * sizeof(int32_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
        checkCuda(cudaMemcpy(objs.data(), dHitObj, inside * sizeof(int32_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }

    timer.next("Output");
    // Candidates of the filter alone (for the summary): parity against the box mesh.
    uint64_t candidates = 0;
    {
        const float bv[24] = {mn[0], mn[1], mn[2], mx[0], mn[1], mn[2], mx[0], mx[1], mn[2], mn[0], mx[1], mn[2],
                              mn[0], mn[1], mx[2], mx[0], mn[1], mx[2], mx[0], mx[1], mx[2], mn[0], mx[1], mx[2]};
        const uint32_t bi[36] = {0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4,
                                 3, 6, 2, 3, 7, 6, 0, 4, 7, 0, 7, 3, 1, 2, 6, 1, 6, 5};
        Geometry box;
        box.V.assign(bv, bv + 24);
        box.I.assign(bi, bi + 36);
        box.T.assign(12, 0);
        DeviceGeometry db;
        db.uploadMesh(box);
        rs_bvh* bb = nullptr;
        check(rs_bvh_build(db.V, db.nV, db.I, db.nF, db.T, 0, &bb, nullptr), "rs_bvh_build");
        // The refine results are already on the host, so the device buffers are reused.
        check(rs_pim(bb, dPoints, n, 0.0f, 0.0f, 1.0f, dObj, nullptr, nullptr), "rs_pim");
        check(rs_compact_hits(dObj, n, dIds, dHitObj, n, &candidates, nullptr), "rs_compact_hits");
        rs_bvh_destroy(bb);
        db.release();
    }
    const uint64_t filtered = n - candidates;
    std::cout << "\n=== FINAL RESULTS ===" << std::endl;
    std::cout << "Total points:            " << n << std::endl;
    std::cout << "Filtered by bbox:        " << filtered << " (" << (filtered * 100.0 / n) << "%)" << std::endl;
    std::cout << "Candidates tested:       " << candidates << " (" << (candidates * 100.0 / n) << "%)" << std::endl;
    std::cout << "Points INSIDE polygons:  " << inside << " (" << (inside * 100.0 / n) << "%)" << std::endl;
    std::cout << "Points OUTSIDE polygons: " << (n - inside) << " (" << ((n - inside) * 100.0 / n) << "%)" << std::endl;
    if (exportResults) {
        std::cout << "Exporting results (hits only)" << std::endl;
        std::ofstream csv("ray_results.csv");
        csv << "pointId,polygonId\n";
        for (uint64_t k = 0; k < inside; ++k) csv << ids[k] << "," << objs[k] << "\n";
        std::cout << "Exported " << inside << " hit points" << std::endl;
    }

    timer.next("Cleanup");
    rs_bvh_destroy(bvh);
    dg.release();
    for (void* p : {(void*)dPoints, (void*)dObj, (void*)dIds, (void*)dHitObj}) cudaFree(p);
    timer.finish(outputJson);
    std::cout << std::endl << "Filter-Refine processing complete!" << std::endl;
    return 0;
}
