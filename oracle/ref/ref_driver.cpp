// Driver that runs pieces of the reference's own host code on fixed inputs, to pin the
// engine's restatements (test infrastructure; built by oracle/ref_build.py into
// oracle/_ref/ref_driver).  Modes:
//   edges   <in.bin> <out.bin>   EdgePreprocessor::extractEdges (preprocess/src/EdgePreprocessor.cpp:41-119)
//   prewrite <in.bin> <out.pre>  RaySpace::IO::writeBinaryFile (common/include/BinaryIO.h:35-102)
//   preread <in.pre> <out.bin>   RaySpace::IO::readBinaryFile  (common/include/BinaryIO.h:104-180)
//   points  <in.txt> <out.bin>   loadPointDataset (query/src/runtime/PointIO.cpp:32-92)
//   box     <in.bin> <out.bin>   BoundingBox::computeFromGeometry + createBoxMesh (geometry/BoundingBox.cpp:4-50)
//   timer   <out.json>           PerformanceTimer::writeResultsToFile (query/src/timer.cpp:124-192)
//   grid    <in.bin> <out.bin> <resolution> <worldSize>
//                                generateGridStats (preprocess/src/preprocess_dataset.cpp:37-181)
// in.bin layout: u64 nV, u64 nF, float V[nV*3], u32 I[nF*3], i32 T[nF], u8 hasGrid,
//   [grid: f32 min[3], f32 max[3], u32 res[3], cells 16 B each].
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "BinaryIO.h"
#include "BoundingBox.h"
#include "EdgePreprocessor.h"
#include "PointIO.h"
#include "timer.h"

void generateGridStats(GeometryData& geometry, GridData& grid, int resolution, float worldSize);

static std::vector<char> slurp(const char* p) {
    std::ifstream f(p, std::ios::binary);
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

static GeometryData read_in(const char* path) {
    std::vector<char> b = slurp(path);
    size_t pos = 0;
    auto take = [&](void* dst, size_t n) { std::memcpy(dst, b.data() + pos, n); pos += n; };
    uint64_t nV, nF;
    take(&nV, 8);
    take(&nF, 8);
    GeometryData g;
    g.vertices.resize(nV);
    g.indices.resize(nF);
    g.triangleToObject.resize(nF);
    take(g.vertices.data(), nV * 12);
    take(g.indices.data(), nF * 12);
    take(g.triangleToObject.data(), nF * 4);
    g.totalTriangles = nF;
    uint8_t hasGrid = 0;
    if (pos < b.size()) take(&hasGrid, 1);
    if (hasGrid) {
        float mn[3], mx[3];
        uint32_t res[3];
        take(mn, 12);
        take(mx, 12);
        take(res, 12);
        g.grid.hasGrid = true;
        g.grid.minBound = {mn[0], mn[1], mn[2]};
        g.grid.maxBound = {mx[0], mx[1], mx[2]};
        g.grid.resolution = {res[0], res[1], res[2]};
        size_t nc = (size_t)res[0] * res[1] * res[2];
        g.grid.cells.resize(nc);
        take(g.grid.cells.data(), nc * 16);
    }
    return g;
}

template <class V>
static void put(std::ofstream& o, const V& v) {
    uint64_t n = v.size();
    o.write((const char*)&n, 8);
    if (n) o.write((const char*)v.data(), n * sizeof(v[0]));
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    std::string mode = argv[1];
    if (mode == "edges" && argc == 4) {
        GeometryData g = read_in(argv[2]);
        EdgeData e = EdgePreprocessor::extractEdges(g.indices, g.triangleToObject, g.vertices);
        std::ofstream o(argv[3], std::ios::binary);
        put(o, e.edgeStarts);
        put(o, e.edgeEnds);
        put(o, e.sourceObjectOffsets);
        put(o, e.sourceObjectCounts);
        put(o, e.sourceObjects);
        return 0;
    }
    if (mode == "prewrite" && argc == 4) {
        GeometryData g = read_in(argv[2]);
        g.edges = EdgePreprocessor::extractEdges(g.indices, g.triangleToObject, g.vertices);
        return RaySpace::IO::writeBinaryFile(argv[3], g) ? 0 : 1;
    }
    if (mode == "preread" && argc == 4) {
        GeometryData g = RaySpace::IO::readBinaryFile(argv[2]);
        std::ofstream o(argv[3], std::ios::binary);
        put(o, g.vertices);
        put(o, g.indices);
        put(o, g.triangleToObject);
        put(o, g.edges.edgeStarts);
        put(o, g.edges.edgeEnds);
        put(o, g.edges.sourceObjectOffsets);
        put(o, g.edges.sourceObjectCounts);
        put(o, g.edges.sourceObjects);
        put(o, g.grid.cells);
        return 0;
    }
    if (mode == "points" && argc == 4) {
        PointData p = loadPointDataset(argv[2]);
        std::ofstream o(argv[3], std::ios::binary);
        put(o, p.positions);
        return 0;
    }
    if (mode == "box" && argc == 4) {
        GeometryData g = read_in(argv[2]);
        BoundingBox bb = BoundingBox::computeFromGeometry(g);
        BoundingBox::BoxMesh m = bb.createBoxMesh();
        std::ofstream o(argv[3], std::ios::binary);
        put(o, m.vertices);
        put(o, m.indices);
        put(o, m.triangleToObject);
        return 0;
    }
    if (mode == "grid" && argc == 6) {
        GeometryData g = read_in(argv[2]);
        generateGridStats(g, g.grid, std::atoi(argv[4]), (float)std::atof(argv[5]));
        std::ofstream o(argv[3], std::ios::binary);
        const float b[6] = {g.grid.minBound.x, g.grid.minBound.y, g.grid.minBound.z,
                            g.grid.maxBound.x, g.grid.maxBound.y, g.grid.maxBound.z};
        const uint32_t r[3] = {g.grid.resolution.x, g.grid.resolution.y, g.grid.resolution.z};
        o.write((const char*)b, sizeof b);
        o.write((const char*)r, sizeof r);
        put(o, g.grid.cells);
        return 0;
    }
    if (mode == "timer" && argc == 3) {
        PerformanceTimer t;
        t.start("Data Reading");
        t.next("Query");
        t.addMeasurement("Raytrace_Mesh1ToMesh2_Pass1", 1234);
        t.addMeasurement("Raytrace_Mesh1ToMesh2_Pass1", 5);
        t.addMeasurement("compact_hash_table_pairs", 987654);
        t.addCounter("Profile_Actual_Intersection_Pairs", 42);
        t.addCounter("Profile_Overlap_Hits_Total", 18446744073709551615ull);
        t.finish(argv[2]);
        return 0;
    }
    return 2;
}
