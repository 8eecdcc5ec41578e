// rs_cli.h -- host layer of the drop-in executables (raytracer, raytracer_filter_refine,
// raytracer_mesh_overlap, raytracer_overlap_estimated, raytracer_overlap_direct_estimation,
// raytracer_intersection_estimated).
//
// Restates the reference's host-side formats and helpers in C++ over librs.so:
//   .pre v2 / v1 reading        common/include/BinaryIO.h:14-180
//   .pre v2 writing             common/include/BinaryIO.h:35-102
//   point files                 query/src/runtime/PointIO.cpp:32-92
//   phase timer + timing JSON   query/src/timer.cpp:1-192
//   flag parsing                query/src/applications/app_cli_options.h:10-163
//   selectivity estimate        query/src/applications/raytracer_overlap_estimated_main.cpp:129-158,252-325
#pragma once

#include <chrono>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "rayspace3d.h"

namespace rscli {

struct GridCellH {
    uint32_t centerCount, touchCount;
    float avgSizeMean, volRatio;
};

struct Geometry {
    std::vector<float> V;        // xyz per vertex
    std::vector<uint32_t> I;     // 3 per triangle
    std::vector<int32_t> T;      // object per triangle
    uint64_t totalTriangles = 0;
    std::vector<float> starts, ends;  // xyz per edge
    std::vector<int32_t> offsets, counts, sources;
    bool hasGrid = false;
    float gmin[3] = {0, 0, 0}, gmax[3] = {0, 0, 0};
    uint32_t res[3] = {0, 0, 0};
    std::vector<GridCellH> cells;

    uint64_t numVertices() const { return V.size() / 3; }
    uint64_t numTriangles() const { return I.size() / 3; }
    uint64_t numEdges() const { return starts.size() / 3; }
    bool hasEdges() const {
        return !starts.empty() && starts.size() == ends.size() && offsets.size() == numEdges() &&
               counts.size() == numEdges();
    }
};

// RaySpace::IO::readBinaryFile semantics: prints the reference's messages and returns an
// empty geometry on a missing file, a magic mismatch or an unsupported version.
// Version 1 files (48-byte header, no edges) are read as well.
Geometry loadGeometryFromFile(const std::string& path);
bool requirePrecomputedEdges(const Geometry& g, const std::string& path, const char* label);
// RaySpace::IO::writeBinaryFile: version-2 layout, edge section when the payload is
// present, grid section when hasGrid; struct padding is written as zeros.
bool writeBinaryFile(const std::string& path, const Geometry& g);
// Flat xyz floats; an empty path yields the reference's three default points.
std::vector<float> loadPointDataset(const std::string& path);
std::vector<std::string> splitPaths(const std::string& input);
int countDistinctObjects(const std::vector<int32_t>& t2o);

class PerformanceTimer {
public:
    void start(const std::string& phase);
    void next(const std::string& phase);
    void finish(const std::string& filename);
    void addMeasurement(const std::string& phase, long long us);
    void addCounter(const std::string& name, unsigned long long value);
    long long getTotalDuration() const;
    // The preprocessing timer (common/src/timer.cpp:96-137) writes no "counters" object.
    bool writeCounters = true;

private:
    using clock = std::chrono::high_resolution_clock;
    struct Phase {
        std::string name;
        clock::time_point start, end;
        long long us = 0;
        bool ended = false;
    };
    std::vector<Phase> phases_, manual_;
    std::vector<std::pair<std::string, unsigned long long>> counters_;
    clock::time_point total_start_, total_end_;
    bool running_ = false, finished_ = false;
    void endCurrent();
    void writeResults(const std::string& filename) const;
};

// Device copies of one geometry set (caller owns; release() frees).
struct DeviceGeometry {
    float* V = nullptr;
    uint32_t* I = nullptr;
    int32_t* T = nullptr;
    float* starts = nullptr;
    float* ends = nullptr;
    int32_t* offsets = nullptr;
    int32_t* counts = nullptr;
    int32_t* sources = nullptr;
    void* cells = nullptr;
    uint64_t nV = 0, nF = 0, nE = 0, nS = 0, nCells = 0;
    void uploadMesh(const Geometry& g);
    void uploadEdges(const Geometry& g);
    void uploadGrid(const Geometry& g);
    void release();
};

// Aborts with the reference's fail-fast behaviour (EXIT_FAILURE) on an engine error.
void check(int status, const char* what);
void checkCuda(int cuda_error, const char* what);

struct Estimate {
    bool ok = false;
    long long pairs = 0;
    float raw = 0.0f;
    float avgSize1 = 0, avgSize2 = 0, volRatio1 = 1, volRatio2 = 1, eff1 = 0, eff2 = 0, alpha = 1;
};
// Grid estimate exactly as the estimated mains compute it; needs both grids on the device.
Estimate estimatePairs(const Geometry& g1, const Geometry& g2, const DeviceGeometry& d1, const DeviceGeometry& d2,
                       float epsilon, float gamma, bool alphaCorrection);

long long microsSince(std::chrono::high_resolution_clock::time_point t0);

// Flag parsing shared by the mesh-pair executables (app_cli_options.h:10-163): unknown
// flags are ignored; --help/-h only sets a flag.
struct MeshPairOptions {
    std::string mesh1, mesh2, output, ptx;
    int runs = 1, warmupRuns = 2;
    bool exportResults = true, helpRequested = false;
    bool allowNoExport = false, allowRuns = true;
    std::vector<std::pair<std::string, std::string>> extra;  // app-specific flags seen (name, value)
    explicit MeshPairOptions(std::string defaultOutput) : output(std::move(defaultOutput)) {}
    // `valued` lists app flags that take a value; `plain` those that do not.
    void parse(int argc, char** argv, const std::vector<std::string>& valued, const std::vector<std::string>& plain);
    bool has(const std::string& flag) const;
    std::string get(const std::string& flag, const std::string& def) const;
    void sanitizeRunCounts();
};

void printHelp(const char* exe, const std::string& usage, const std::string& description,
               const std::vector<std::pair<std::string, std::string>>& options);

}  // namespace rscli
