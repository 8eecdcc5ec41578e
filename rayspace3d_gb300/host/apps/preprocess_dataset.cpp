// preprocess_dataset -- the preprocessing step (preprocess/src/preprocess_dataset.cpp:183-385)
// with its two compute stages on the GPU: grid statistics (rs_grid_stats, generateGridStats
// :37-179) and the unique-edge payload (rs_extract_edges, EdgePreprocessor::extractEdges,
// preprocess/src/EdgePreprocessor.cpp:41-119).  Both are bit-identical to the reference's, so
// the written .pre v2 file is byte-identical to the one the reference writes for the same
// geometry (struct padding aside, written here as zeros).
//
// Flags, phase names, stdout summary and timing JSON follow the reference.  The dataset
// loaders (OBJ through tinyobjloader, .dt through tdbase, WKT polygons through CGAL
// triangulation) are not part of the engine: --dataset takes a .pre file of version 1 or 2
// whose geometry (vertices, triangles, triangle-to-object map) is re-preprocessed; other
// inputs are refused with an error.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <filesystem>
#include <iomanip>
#include <iostream>
#include <random>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "rs_cli.h"

using namespace rscli;

namespace {

void usage(const char* exe) {
    std::cout << "Usage: " << exe
              << " [--mode <wkt|mesh|dt>] [--dataset <path>] [--output-geometry <geometry_output_file>]"
                 " [--output-timing <timing_output_file>]"
              << std::endl;
    std::cout << "Options:" << std::endl;
    std::cout << "  --mode <wkt|mesh|dt>       Dataset loading mode (default: mesh)" << std::endl;
    std::cout << "  --dataset <path>           Path to dataset (a .pre file: its geometry is preprocessed again)" << std::endl;
    std::cout << "  --output-geometry <path>   Path to text file for geometry data output" << std::endl;
    std::cout << "  --output-timing <path>     Path to JSON file for preprocessing timing output" << std::endl;
    std::cout << "  --shuffle                  Randomly translate each loaded object" << std::endl;
    std::cout << "  --generate-grid            Generate grid statistics for selectivity estimation" << std::endl;
    std::cout << "  --grid-resolution <N>      Grid resolution (default: 128)" << std::endl;
    std::cout << "  --world-size <S>           World size (default: auto-detected)" << std::endl;
}

std::string lowerExt(const std::string& path) {
    std::string ext = std::filesystem::path(path).extension().string();
    for (auto& c : ext) c = (char)std::tolower((unsigned char)c);
    return ext;
}

// --shuffle (:293-334): one uniform(-15, 15) translation per object applied to the vertices
// its triangles use.  The reference seeds from std::random_device, so its output is not
// reproducible; this does the same.
void shuffleObjects(Geometry& g) {
    if (g.numTriangles() != g.T.size()) {
        std::cerr << "Warning: indices and triangleToObject size mismatch; skipping shuffle." << std::endl;
        return;
    }
    std::unordered_map<int, std::unordered_set<unsigned int>> objVerts;
    for (uint64_t t = 0; t < g.numTriangles(); ++t) {
        auto& s = objVerts[g.T[t]];
        for (int k = 0; k < 3; ++k) s.insert(g.I[3 * t + k]);
    }
    std::random_device rd;
    std::mt19937 rng(rd());
    std::uniform_real_distribution<float> dist(-15.0f, 15.0f);
    std::cout << "Applying random translations to " << objVerts.size() << " objects..." << std::endl;
    size_t processed = 0;
    for (auto& kv : objVerts) {
        const float tx = dist(rng), ty = dist(rng), tz = dist(rng);
        for (unsigned int v : kv.second)
            if (v < g.numVertices()) {
                g.V[3 * (uint64_t)v] += tx;
                g.V[3 * (uint64_t)v + 1] += ty;
                g.V[3 * (uint64_t)v + 2] += tz;
            }
        if (++processed <= 3)
            std::cout << "  Object " << kv.first << " translated by (" << std::fixed << std::setprecision(2) << tx
                      << ", " << ty << ", " << tz << ")" << std::endl;
    }
    std::cout.unsetf(std::ios::floatfield);
}

template <class T>
T* toDevice(const std::vector<T>& v) {
    T* d = nullptr;
    checkCuda(cudaMalloc((void**)&d, std::max<size_t>(v.size(), 1) * sizeof(T)), "cudaMalloc");
    if (!v.empty()) checkCuda(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
    return d;
}

template <class T>
void toHost(std::vector<T>& v, const T* d, size_t n) {
    v.resize(n);
    if (n) checkCuda(cudaMemcpy(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy");
}

}  // namespace

int main(int argc, char** argv) {
    std::string datasetPath, outputGeometryPath = "geometry_data.txt", outputTimingPath = "preprocessing_timing.json";
    std::string modeStr = "mesh";
    bool shuffle = false, generateGrid = false;
    int gridResolution = 128;
    float worldSize = -1.0f;

    std::cout << "Arguments received:" << std::endl;
    for (int i = 0; i < argc; ++i) std::cout << "  [" << i << "] " << argv[i] << std::endl;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--dataset" && i + 1 < argc) datasetPath = argv[++i];
        else if (a == "--mode" && i + 1 < argc) modeStr = argv[++i];
        else if (a == "--output-geometry" && i + 1 < argc) outputGeometryPath = argv[++i];
        else if (a == "--output-timing" && i + 1 < argc) outputTimingPath = argv[++i];
        else if (a == "--shuffle" || a == "shuffle") shuffle = true;
        else if (a == "--generate-grid") generateGrid = true;
        else if ((a == "--grid-resolution" || a == "--euler-grid-size") && i + 1 < argc) gridResolution = std::stoi(argv[++i]);
        else if (a == "--world-size" && i + 1 < argc) worldSize = std::stof(argv[++i]);
        else if (a == "--gamma" && i + 1 < argc) ++i;
        else if (a == "--help" || a == "-h") {
            usage(argv[0]);
            return 0;
        } else std::cout << "Warning: Unknown argument '" << a << "'" << std::endl;
    }
    if (modeStr != "mesh" && modeStr != "wkt" && modeStr != "dt") {
        std::cerr << "Error: Unknown mode '" << modeStr << "'. Valid modes: wkt, mesh, dt" << std::endl;
        return 1;
    }
    if (datasetPath.empty()) {
        std::cerr << "Error: Dataset path is required. Use --dataset <path>" << std::endl;
        return 1;
    }
    std::cout << "Dataset Preprocessing Tool" << std::endl;
    std::cout << "Mode: " << modeStr << std::endl;
    std::cout << "Input dataset: " << datasetPath << std::endl;
    std::cout << "Output geometry: " << outputGeometryPath << std::endl;
    std::cout << "Output timing: " << outputTimingPath << std::endl;

    PerformanceTimer timer;
    timer.writeCounters = false;
    timer.start(modeStr == "wkt" ? "Loading WKT Dataset" : "Loading Dataset");
    if (lowerExt(datasetPath) != ".pre") {
        std::cerr << "Error: Could not determine loader for path: " << datasetPath
                  << " (preprocess_dataset on the GPU reads .pre geometry; OBJ, DT and WKT loaders are not included)"
                  << std::endl;
        return 1;
    }
    Geometry g = loadGeometryFromFile(datasetPath);
    if (g.V.empty()) {
        std::cerr << "Error: Failed to load dataset or dataset is empty." << std::endl;
        return 1;
    }
    // Only the geometry is kept; grid and edges are derived again.
    g.hasGrid = false;
    g.cells.clear();
    g.starts.clear();
    g.ends.clear();
    g.offsets.clear();
    g.counts.clear();
    g.sources.clear();
    if (g.totalTriangles == 0) g.totalTriangles = g.numTriangles();

    if (shuffle) {
        timer.next("Shuffling Objects (Random Translation)");
        shuffleObjects(g);
    }

    const uint64_t nV = g.numVertices(), nF = g.numTriangles();
    float* dV = toDevice(g.V);
    uint32_t* dI = toDevice(g.I);
    int32_t* dT = toDevice(g.T);

    if (generateGrid) {
        timer.next("Generating Grid Statistics");
        int32_t maxObj = -1;
        for (int32_t o : g.T) maxObj = std::max(maxObj, o);
        const uint64_t ncell = (uint64_t)gridResolution * gridResolution * gridResolution;
        void* dCells = nullptr;
        checkCuda(cudaMalloc(&dCells, ncell * sizeof(GridCellH)), "cudaMalloc");
        float b[6];
        check(rs_grid_stats(dV, nV, dI, nF, dT, (uint64_t)(maxObj + 1), gridResolution, worldSize, dCells, b, nullptr),
              "rs_grid_stats");
        toHost(g.cells, reinterpret_cast<const GridCellH*>(dCells), ncell);
        cudaFree(dCells);
        g.hasGrid = true;
        for (int k = 0; k < 3; ++k) {
            g.gmin[k] = b[k];
            g.gmax[k] = b[3 + k];
            g.res[k] = (uint32_t)gridResolution;
        }
        std::cout << "Grid statistics generated. Resolution: " << gridResolution << ", WorldSize: " << worldSize
                  << std::endl;
    }

    timer.next("Extracting Edges");
    {
        const uint64_t cap = std::max<uint64_t>(3 * nF, 1);
        float *dS = nullptr, *dE = nullptr;
        int32_t *dOff = nullptr, *dCnt = nullptr, *dSrc = nullptr;
        checkCuda(cudaMalloc((void**)&dS, cap * 3 * sizeof(float)), "cudaMalloc");
        checkCuda(cudaMalloc((void**)&dE, cap * 3 * sizeof(float)), "cudaMalloc");
        checkCuda(cudaMalloc((void**)&dOff, cap * sizeof(int32_t)), "cudaMalloc");
        checkCuda(cudaMalloc((void**)&dCnt, cap * sizeof(int32_t)), "cudaMalloc");
        checkCuda(cudaMalloc((void**)&dSrc, cap * sizeof(int32_t)), "cudaMalloc");
        uint64_t nE = 0, nS = 0;
        check(rs_extract_edges(dV, nV, dI, nF, dT, dS, dE, dOff, dCnt, dSrc, cap, &nE, &nS, nullptr),
              "rs_extract_edges");
        toHost(g.starts, dS, 3 * nE);
        toHost(g.ends, dE, 3 * nE);
        toHost(g.offsets, dOff, nE);
        toHost(g.counts, dCnt, nE);
        toHost(g.sources, dSrc, nS);
        for (void* p : {(void*)dS, (void*)dE, (void*)dOff, (void*)dCnt, (void*)dSrc}) cudaFree(p);
    }
    cudaFree(dV);
    cudaFree(dI);
    cudaFree(dT);
    if (!g.hasEdges()) {
        std::cerr << "Error: Edge extraction failed. No valid edge payload generated." << std::endl;
        return 1;
    }
    std::cout << "Extracted " << g.numEdges() << " unique edges with " << g.sources.size()
              << " flattened source-object entries" << std::endl;

    timer.next("Writing Geometry Data");
    if (writeBinaryFile(outputGeometryPath, g))
        std::cout << "Geometry data written to: " << outputGeometryPath << " (Binary)" << std::endl;
    timer.finish(outputTimingPath);

    std::cout << "\n=== Preprocessing Complete ===" << std::endl;
    std::cout << "Mode: " << modeStr << std::endl;
    std::cout << "Processed dataset: " << datasetPath << std::endl;
    std::cout << "Total objects (triangles): " << g.totalTriangles << std::endl;
    std::cout << "Total vertices: " << nV << std::endl;
    std::cout << "Total triangles: " << nF << std::endl;
    std::cout << "Total extracted edges: " << g.numEdges() << std::endl;
    std::cout << "Universe Extents: [" << (g.gmax[0] - g.gmin[0]) << ", " << (g.gmax[1] - g.gmin[1]) << ", "
              << (g.gmax[2] - g.gmin[2]) << "]" << std::endl;
    std::cout << "Universe Min: [" << g.gmin[0] << ", " << g.gmin[1] << ", " << g.gmin[2] << "]" << std::endl;
    std::cout << "Universe Max: [" << g.gmax[0] << ", " << g.gmax[1] << ", " << g.gmax[2] << "]" << std::endl;
    std::cout << "Geometry data saved to: " << outputGeometryPath << std::endl;
    std::cout << "Timing data saved to: " << outputTimingPath << std::endl;
    return 0;
}
