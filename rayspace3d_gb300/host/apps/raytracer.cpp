// raytracer -- point-in-mesh parity, drop-in for the reference's `raytracer`
// (query/src/applications/rayspace_main.cpp:39-260): same flags, phases, stdout summary,
// ray_results.csv (pointId,polygonId; hits only, here in ascending point order) and
// timing JSON.  Engine flag (ignored by the reference): --rs-direction x|y|z (default z).
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
    std::string geometryPath, pointsPath, outputJson = "performance_timing.json", ptx, direction = "z";
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
        else if (a == "--rs-direction" && i + 1 < argc) direction = argv[++i];
        else if (a == "--help" || a == "-h") {
            std::cout << "Usage: " << argv[0]
                      << " [--geometry <path(s)>] [--points <path(s)>] [--output <json_output_file>] [--runs <number>]"
                         " [--ptx <ptx_file>]" << std::endl;
            std::cout << "Options:" << std::endl;
            std::cout << "  --geometry <path(s)>  Path(s) to preprocessed geometry file(s). Use commas to separate multiple files." << std::endl;
            std::cout << "  --points <path(s)>    Path(s) to WKT file(s) containing POINT geometries. Use commas to separate multiple files." << std::endl;
            std::cout << "  --output <path>       Path to JSON file for performance timing output" << std::endl;
            std::cout << "  --runs <number>       Number of times to run the query (for performance testing)" << std::endl;
            std::cout << "  --warmup-runs <num>   Number of warmup runs (default: 2)" << std::endl;
            std::cout << "  --no-export           Disable CSV export of results" << std::endl;
            std::cout << "  --ptx <ptx_file>      Accepted for compatibility (the engine loads no PTX)" << std::endl;
            std::cout << "  --rs-direction <x|y|z> Ray direction (default: z, the reference's +Z)" << std::endl;
            std::cout << "  --help, -h            Show this help message" << std::endl;
            return 0;
        }
    }
    std::cout << "RaySpace3D GB300 engine: point-in-mesh parity" << std::endl;
    const float dx = direction == "x" ? 1.0f : 0.0f, dy = direction == "y" ? 1.0f : 0.0f,
                dz = (direction != "x" && direction != "y") ? 1.0f : 0.0f;
    const std::vector<std::string> geometryFiles = splitPaths(geometryPath);
    const std::vector<std::string> pointFiles = splitPaths(pointsPath);
    if (geometryFiles.empty()) {
        std::cerr << "Error: Geometry file path is required. Use --geometry <path_to_geometry_file>" << std::endl;
        return 1;
    }
    if (pointFiles.empty()) {
        std::cerr << "Error: Points file path is required. Use --points <path_to_point_file>" << std::endl;
        return 1;
    }
    const size_t numTasks = std::max(geometryFiles.size(), pointFiles.size());
    if (geometryFiles.size() > 1 && pointFiles.size() > 1 && geometryFiles.size() != pointFiles.size()) {
        std::cerr << "Error: When both --geometry and --points are lists, they must have the same length." << std::endl;
        return 1;
    }
    std::cout << "Processing " << numTasks << " task(s)" << std::endl;

    timer.next("Application Creation");
    checkCuda(cudaFree(0), "context creation");

    std::string cachedGeometryPath, cachedPointsPath;
    Geometry geometry;
    DeviceGeometry dgeom;
    rs_bvh* bvh = nullptr;
    std::vector<float> points;
    float* dPoints = nullptr;
    int32_t* dObj = nullptr;
    int32_t* dIds = nullptr;
    int32_t* dHitObj = nullptr;
    uint64_t numPoints = 0;

    for (size_t task = 0; task < numTasks; ++task) {
        const std::string gpath = geometryFiles[geometryFiles.size() == 1 ? 0 : task];
        const std::string ppath = pointFiles[pointFiles.size() == 1 ? 0 : task];
        std::cout << "\n=== Task " << (task + 1) << "/" << numTasks << " ===" << std::endl;
        std::cout << "Geometry: " << gpath << std::endl;
        std::cout << "Points: " << ppath << std::endl;
        if (gpath != cachedGeometryPath) {
            timer.next("Load Geometry");
            std::cout << "Loading new geometry..." << std::endl;
            geometry = loadGeometryFromFile(gpath);
            if (geometry.V.empty()) {
                std::cerr << "Error: Failed to load geometry from " << gpath << std::endl;
                continue;
            }
            cachedGeometryPath = gpath;
            timer.next("Upload Geometry");
            if (bvh) rs_bvh_destroy(bvh);
            bvh = nullptr;
            dgeom.release();
            dgeom.uploadMesh(geometry);
            timer.next("Build Index");
            check(rs_bvh_build(dgeom.V, dgeom.nV, dgeom.I, dgeom.nF, dgeom.T, 0, &bvh, nullptr), "rs_bvh_build");
            std::cout << "Acceleration structure built" << std::endl;
        } else {
            std::cout << "Using cached geometry" << std::endl;
        }
        if (ppath != cachedPointsPath) {
            timer.next("Load Points");
            std::cout << "Loading new points..." << std::endl;
            points = loadPointDataset(ppath);
            if (points.empty()) {
                std::cerr << "Error: Failed to load points from " << ppath << std::endl;
                continue;
            }
            cachedPointsPath = ppath;
            numPoints = points.size() / 3;
            std::cout << "Points loaded: " << numPoints << std::endl;
            timer.next("Upload Points");
            for (void* p : {(void*)dPoints, (void*)dObj, (void*)dIds, (void*)dHitObj})
                if (p) cudaFree(p);
            checkCuda(cudaMalloc(&dPoints, points.size() * sizeof(float)), "cudaMalloc");
            checkCuda(cudaMemcpy(dPoints, points.data(), points.size() * sizeof(float), cudaMemcpyHostToDevice),
                      "cudaMemcpy");
            checkCuda(cudaMalloc(&dObj, numPoints * sizeof(int32_t)), "cudaMalloc");
            checkCuda(cudaMalloc(&dIds, numPoints * sizeof(int32_t)), "cudaMalloc");
            checkCuda(cudaMalloc(&dHitObj, numPoints * sizeof(int32_t)), "cudaMalloc");
            std::cout << "Points uploaded to GPU" << std::endl;
        } else {
            std::cout << "Using cached points" << std::endl;
        }
        if (!bvh || numPoints == 0) continue;

        timer.next("Warmup");
        for (int w = 0; w < warmupRuns; ++w)
            check(rs_pim(bvh, dPoints, numPoints, dx, dy, dz, dObj, nullptr, nullptr), "rs_pim");

        timer.next("Query");
        if (runs > 1) {
            std::cout << "\n=== Running " << runs << " iterations for performance measurement ===" << std::endl;
            for (int r = 0; r < runs; ++r) {
                std::cout << "Run " << (r + 1) << "/" << runs << std::endl;
                check(rs_pim(bvh, dPoints, numPoints, dx, dy, dz, dObj, nullptr, nullptr), "rs_pim");
            }
        } else {
            std::cout << "\n=== Tracing " << numPoints << " rays in a single GPU launch ===" << std::endl;
            check(rs_pim(bvh, dPoints, numPoints, dx, dy, dz, dObj, nullptr, nullptr), "rs_pim");
        }

        timer.next("Download Results");
        uint64_t numHit = 0;
        check(rs_compact_hits(dObj, numPoints, dIds, dHitObj, numPoints, &numHit, nullptr), "rs_compact_hits");
        std::vector<int32_t> ids(numHit), objs(numHit);
        if (numHit) {
            checkCuda(cudaMemcpy(ids.data(), dIds, numHit * sizeof(int32_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
            checkCuda(cudaMemcpy(objs.data(), dHitObj, numHit * sizeof(int32_t), cudaMemcpyDeviceToHost), "cudaMemcpy");
        }

        timer.next("Output");
        std::cout << "\n=== Point-in-Polygon Summary ===" << std::endl;
        std::cout << "Total rays: " << numPoints << std::endl;
        std::cout << "Points INSIDE polygons:  " << numHit << std::endl;
        std::cout << "Points OUTSIDE polygons: " << (numPoints - numHit) << std::endl;
        std::cout << "Inside ratio: " << (numPoints ? (double)numHit / numPoints * 100.0 : 0.0) << " %" << std::endl;
        if (exportResults) {
            std::cout << "Exporting results (hits only)" << std::endl;
            std::ofstream csv("ray_results.csv");
            csv << "pointId,polygonId\n";
            for (uint64_t k = 0; k < numHit; ++k) csv << ids[k] << "," << objs[k] << "\n";
        }
    }

    timer.next("Cleanup");
    if (bvh) rs_bvh_destroy(bvh);
    dgeom.release();
    for (void* p : {(void*)dPoints, (void*)dObj, (void*)dIds, (void*)dHitObj})
        if (p) cudaFree(p);
    timer.finish(outputJson);
    std::cout << std::endl << "Total tasks processed: " << numTasks << std::endl;
    return 0;
}
