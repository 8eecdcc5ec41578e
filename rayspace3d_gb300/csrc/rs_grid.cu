// rs_grid.cu -- per-cell grid statistics on the GPU (generateGridStats,
// preprocess/src/preprocess_dataset.cpp:37-181), bit for bit.
//
// The reference keeps its objects in a std::unordered_map<int, ObjectStats> filled in
// triangle order (:69-86), sums each object's signed volume in FP64 in triangle order
// (:88-114), then visits the map in its iteration order and adds every object's mean extent
// and volume ratio into the float sums of the cells it touches (:116-168).  Float sums
// depend on their order, so the engine reproduces every order:
//   * object boxes: atomic min/max (order-free), plus each object's first and last valid
//     triangle;
//   * volumes: one thread per object adds its triangles' float terms into an FP64 sum in
//     triangle order -- straight over [first, last] when tri2obj never decreases, else over
//     a stable radix sort of the triangles by object;
//   * visit order: the host inserts the objects in order of first appearance into a
//     std::unordered_map<int, ...> of the same library and reads its iteration order;
//   * cell sums: each object, in visit order, emits one (cell, rank) record per touched
//     cell; a stable radix sort by cell leaves each cell's records in visit order, and one
//     thread per cell adds them in that order and divides by the count (:170-177).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kGT = 256;
constexpr uint32_t kNone = 0xffffffffu;

__device__ __forceinline__ int g_f2ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float g_ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct ObjStats {
    int box[6];      // ordered-int min xyz, max xyz
    uint32_t first;  // first valid triangle
    uint32_t last;   // last valid triangle
    double volume;   // signed volume sum
};

// Per visited object (rank order): the quantities its cells receive and its cell range.
struct ObjCells {
    float avg, ratio;
    int lo[3], hi[3];
};

__global__ void k_gs_init(ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_obj) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        o[i].box[c] = g_f2ord(1e30f);
        o[i].box[3 + c] = g_f2ord(-1e30f);
    }
    o[i].first = kNone;
    o[i].last = 0;
    o[i].volume = 0.0;
}

__device__ __forceinline__ bool tri_valid(const uint32_t* __restrict__ I, uint64_t nV, uint64_t t) {
    return I[3 * t] < nV && I[3 * t + 1] < nV && I[3 * t + 2] < nV;
}

// Pass 1 (preprocess_dataset.cpp:69-86): object boxes and valid-triangle span.  flags[0]
// is set when a valid triangle's object is outside [0, n_obj); flags[1] when tri2obj
// decreases somewhere (objects not stored contiguously).
__global__ void k_gs_boxes(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t nF,
                           const int32_t* __restrict__ T, ObjStats* __restrict__ o, uint64_t n_obj,
                           uint32_t* __restrict__ flags) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    if (t > 0 && T[t] < T[t - 1]) flags[1] = 1;
    if (!tri_valid(I, nV, t)) return;
    const int32_t obj = T[t];
    if (obj < 0 || (uint64_t)obj >= n_obj) {
        flags[0] = 1;
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a = V[3 * (uint64_t)I[3 * t] + c], b = V[3 * (uint64_t)I[3 * t + 1] + c],
                    d = V[3 * (uint64_t)I[3 * t + 2] + c];
        atomicMin(&o[obj].box[c], g_f2ord(fminf(fminf(a, b), d)));
        atomicMax(&o[obj].box[3 + c], g_f2ord(fmaxf(fmaxf(a, b), d)));
    }
    atomicMin(&o[obj].first, (uint32_t)t);
    atomicMax(&o[obj].last, (uint32_t)t);
}

// The float term of one triangle (:100-113): translate by the box centre, dot(cross(t0,t1), t2),
// every operation rounded as written.
__device__ __forceinline__ float volume_term(const float* __restrict__ V, const uint32_t* __restrict__ I, uint64_t t,
                                             const float c[3]) {
    float p[3][3];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int k = 0; k < 3; ++k) p[v][k] = __fsub_rn(V[3 * (uint64_t)I[3 * t + v] + k], c[k]);
    const float cx = __fsub_rn(__fmul_rn(p[0][1], p[1][2]), __fmul_rn(p[0][2], p[1][1]));
    const float cy = __fsub_rn(__fmul_rn(p[0][2], p[1][0]), __fmul_rn(p[0][0], p[1][2]));
    const float cz = __fsub_rn(__fmul_rn(p[0][0], p[1][1]), __fmul_rn(p[0][1], p[1][0]));
    return __fadd_rn(__fadd_rn(__fmul_rn(cx, p[2][0]), __fmul_rn(cy, p[2][1])), __fmul_rn(cz, p[2][2]));
}

__device__ __forceinline__ void box_centre(const ObjStats& s, float c[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = __fmul_rn(__fadd_rn(g_ord2f(s.box[k]), g_ord2f(s.box[3 + k])), 0.5f);
}

// Pass 2 (:88-114), objects stored contiguously: each object's valid triangles in order.
__global__ void k_gs_volume_span(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                                 ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_obj || o[i].first == kNone) return;
    float c[3];
    box_centre(o[i], c);
    double vol = 0.0;
    for (uint64_t t = o[i].first; t <= o[i].last; ++t)
        if (tri_valid(I, nV, t)) vol = __dadd_rn(vol, (double)volume_term(V, I, t, c));
    o[i].volume = vol;
}

// Sort keys (object << 32 | triangle) for the general case; invalid triangles and
// out-of-range objects get object n_obj and sort last.
__global__ void k_gs_tri_keys(const uint32_t* __restrict__ I, uint64_t nV, uint64_t nF, const int32_t* __restrict__ T,
                              uint64_t n_obj, uint64_t* __restrict__ keys) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    const int32_t obj = T[t];
    const bool ok = tri_valid(I, nV, t) && obj >= 0 && (uint64_t)obj < n_obj;
    keys[t] = ((ok ? (uint64_t)obj : n_obj) << 32) | t;
}

// Start of each object's run in the sorted keys.
__global__ void k_gs_run_starts(const uint64_t* __restrict__ keys, uint64_t nF, uint64_t n_obj,
                                uint32_t* __restrict__ start) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= nF) return;
    const uint64_t obj = keys[j] >> 32;
    if (obj < n_obj && (j == 0 || (keys[j - 1] >> 32) != obj)) start[obj] = (uint32_t)j;
}

// Pass 2, general case: the object's run of the sorted keys, in triangle order.
__global__ void k_gs_volume_sorted(const float* __restrict__ V, const uint32_t* __restrict__ I,
                                   const uint64_t* __restrict__ keys, uint64_t nF, const uint32_t* __restrict__ start,
                                   ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_obj || o[i].first == kNone) return;
    float c[3];
    box_centre(o[i], c);
    double vol = 0.0;
    for (uint64_t j = start[i]; j < nF && (keys[j] >> 32) == i; ++j)
        vol = __dadd_rn(vol, (double)volume_term(V, I, keys[j] & 0xffffffffull, c));
    o[i].volume = vol;
}

struct GridFrame {
    float mn[3], cs[3];
    int res;
};

// Per visited object (rank r, :116-160): ratio, mean extent, anchor cell (CenterCount is an
// integer count, added atomically), touched cell range and its size.
__global__ void k_gs_objects(const ObjStats* __restrict__ o, const uint32_t* __restrict__ order, uint64_t n_vis,
                             GridFrame f, uint32_t* __restrict__ cells, ObjCells* __restrict__ oc,
                             int32_t* __restrict__ ncell) {
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (r >= n_vis) return;
    const ObjStats& s = o[order[r]];
    float mnb[3], mxb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mnb[k] = g_ord2f(s.box[k]);
        mxb[k] = g_ord2f(s.box[3 + k]);
    }
    const float meshVol = __fdiv_rn(fabsf((float)s.volume), 6.0f);
    const float w = __fsub_rn(mxb[0], mnb[0]), h = __fsub_rn(mxb[1], mnb[1]), d = __fsub_rn(mxb[2], mnb[2]);
    float aabb = __fmul_rn(__fmul_rn(w, h), d);
    if (aabb < 1e-9f) aabb = 1e-9f;
    float ratio = __fdiv_rn(meshVol, aabb);
    if (ratio > 1.0f) ratio = 1.0f;
    ObjCells out;
    out.ratio = ratio;
    out.avg = __fdiv_rn(__fadd_rn(__fadd_rn(w, h), d), 3.0f);
    const int R = f.res;
    int a[3];
    long long n = 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ctr = __fmul_rn(__fadd_rn(mnb[k], mxb[k]), 0.5f);
        a[k] = (int)__fdiv_rn(__fsub_rn(ctr, f.mn[k]), f.cs[k]);
        out.lo[k] = max(0, (int)__fdiv_rn(__fsub_rn(mnb[k], f.mn[k]), f.cs[k]));
        out.hi[k] = min(R - 1, (int)__fdiv_rn(__fsub_rn(__fsub_rn(mxb[k], f.mn[k]), 1e-5f), f.cs[k]));
        n *= max(0, out.hi[k] - out.lo[k] + 1);
    }
    if (a[0] >= 0 && a[0] < R && a[1] >= 0 && a[1] < R && a[2] >= 0 && a[2] < R)
        atomicAdd(&cells[4 * ((uint64_t)(a[2] * R + a[1]) * R + a[0])], 1u);
    oc[r] = out;
    ncell[r] = (int32_t)n;
}

// One (cell, rank) record per touched cell, objects in rank order.
__global__ void k_gs_emit(const ObjCells* __restrict__ oc, const int64_t* __restrict__ off, uint64_t n_vis, int R,
                          uint64_t* __restrict__ cell_key, uint32_t* __restrict__ rank) {
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (r >= n_vis) return;
    const ObjCells c = oc[r];
    uint64_t j = (uint64_t)off[r];
    for (int z = c.lo[2]; z <= c.hi[2]; ++z)
        for (int y = c.lo[1]; y <= c.hi[1]; ++y)
            for (int x = c.lo[0]; x <= c.hi[0]; ++x) {
                cell_key[j] = (uint64_t)(z * R + y) * R + x;
                rank[j] = (uint32_t)r;
                ++j;
            }
}

// Per cell (:162-177): the float sums in visit order, then the means.
__global__ void k_gs_cell_sums(const uint64_t* __restrict__ cell_key, const uint32_t* __restrict__ rank, uint64_t n,
                               const ObjCells* __restrict__ oc, uint32_t* __restrict__ cells) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= n || (j > 0 && cell_key[j - 1] == cell_key[j])) return;
    const uint64_t cell = cell_key[j];
    uint32_t touch = 0;
    float asum = 0.0f, rsum = 0.0f;
    for (uint64_t q = j; q < n && cell_key[q] == cell; ++q) {
        const ObjCells& c = oc[rank[q]];
        asum = __fadd_rn(asum, c.avg);
        rsum = __fadd_rn(rsum, c.ratio);
        ++touch;
    }
    uint32_t* out = cells + 4 * cell;
    out[1] = touch;
    reinterpret_cast<float*>(out)[2] = __fdiv_rn(asum, (float)touch);
    reinterpret_cast<float*>(out)[3] = __fdiv_rn(rsum, (float)touch);
}

__global__ void k_gs_vbounds(const float* __restrict__ V, uint64_t nV, int* __restrict__ b) {
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nV; i += (uint64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], V[3 * i + k]);
            mx[k] = fmaxf(mx[k], V[3 * i + k]);
        }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        atomicMin(&b[k], g_f2ord(mn[k]));
        atomicMax(&b[3 + k], g_f2ord(mx[k]));
    }
}


// Iteration order of a std::unordered_map<int, V> after operator[] on each key in turn:
// the order in which the reference's pass 3 visits its objects.
std::vector<uint32_t> map_visit_order(const std::vector<uint32_t>& first_seen) {
    std::unordered_map<int, char> m;
    for (uint32_t o : first_seen) m[(int)o];
    std::vector<uint32_t> out;
    out.reserve(m.size());
    for (const auto& kv : m) out.push_back((uint32_t)kv.first);
    return out;
}


}  // namespace
}  // namespace rs

using namespace rs;

extern "C" int rs_grid_stats(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                             const int32_t* d_tri2obj, uint64_t n_obj, int resolution, float world_size,
                             void* d_cells, float* h_bounds6, void* stream) {
    if (resolution <= 0 || resolution > 1024 || !d_cells || (nF && (!d_indices || !d_tri2obj)) ||
        (nV && !d_vertices) || n_obj > 0x7fffffffull)
        return RS_ERR_INVALID;
    if (nF >= 0xffffffffull) return RS_ERR_TOO_LARGE;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t ncell = (uint64_t)resolution * resolution * resolution;
    Scratch sc{s};
    // Frame: [0, world]^3, or the bounds of all vertices (:40-60).
    float mn[3], mx[3];
    if (world_size > 0.0f) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = 0.0f;
            mx[k] = world_size;
        }
    } else {
        int* b = nullptr;
        cudaError_t e = sc.get(&b, 6 * sizeof(int));
        if (e != cudaSuccess) return to_status(e);
        const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
        int hb[6];
        e = cudaMemcpyAsync(b, init, sizeof(init), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nV) launch(k_gs_vbounds, 2 * sm_count(), kGT, 0, s, d_vertices, nV, b);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hb, b, sizeof(hb), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return to_status(e);
        for (int k = 0; k < 3; ++k) {
            auto dec = [](int i) {
                int v = i >= 0 ? i : i ^ 0x7fffffff;
                float f;
                std::memcpy(&f, &v, 4);
                return f;
            };
            // The reference starts its min/max at +-1e30 (an empty set keeps them).
            mn[k] = nV ? dec(hb[k]) : 1e30f;
            mx[k] = nV ? dec(hb[3 + k]) : -1e30f;
        }
    }
    GridFrame f;
    f.res = resolution;
    for (int k = 0; k < 3; ++k) {
        f.mn[k] = mn[k];
        f.cs[k] = (mx[k] - mn[k]) / (float)resolution;
        if (h_bounds6) {
            h_bounds6[k] = mn[k];
            h_bounds6[3 + k] = mx[k];
        }
    }
    cudaError_t e = cudaMemsetAsync(d_cells, 0, ncell * 16, s);
    if (e != cudaSuccess) return to_status(e);
    if (!n_obj || !nF) {
        e = cudaStreamSynchronize(s);
        return to_status(e);
    }
    ObjStats* o = nullptr;
    uint32_t* flags = nullptr;
    e = sc.get(&o, n_obj * sizeof(ObjStats));
    if (e == cudaSuccess) e = sc.get(&flags, 2 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return to_status(e);
    const unsigned go = (unsigned)((n_obj + kGT - 1) / kGT), gt = (unsigned)((nF + kGT - 1) / kGT);
    launch(k_gs_init, go, kGT, 0, s, o, n_obj);
    launch(k_gs_boxes, gt, kGT, 0, s, d_vertices, nV, d_indices, nF, d_tri2obj, o, n_obj, flags);
    uint32_t hf[2] = {0, 0};
    e = cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return to_status(e);
    if (hf[0]) return RS_ERR_INVALID;  // an object id outside [0, n_obj)
    if (!hf[1]) {
        launch(k_gs_volume_span, go, kGT, 0, s, d_vertices, nV, d_indices, o, n_obj);
    } else {
        uint64_t* keys = nullptr;
        uint32_t* start = nullptr;
        e = sc.get(&keys, nF * sizeof(uint64_t));
        if (e == cudaSuccess) e = sc.get(&start, n_obj * sizeof(uint32_t));
        if (e != cudaSuccess) return to_status(e);
        launch(k_gs_tri_keys, gt, kGT, 0, s, d_indices, nV, nF, d_tri2obj, n_obj, keys);
        // Stable from triangle order, so only the object bits need sorting.
        e = radix_sort_u64(keys, nullptr, nF, 32 + bits_for(n_obj), s, 32);
        if (e != cudaSuccess) return to_status(e);
        launch(k_gs_run_starts, gt, kGT, 0, s, (const uint64_t*)keys, nF, n_obj, start);
        launch(k_gs_volume_sorted, go, kGT, 0, s, d_vertices, d_indices, (const uint64_t*)keys, nF,
               (const uint32_t*)start, o, n_obj);
    }
    // Visit order: objects by first valid triangle, through the map.
    std::vector<ObjStats> ho(n_obj);
    e = cudaMemcpyAsync(ho.data(), o, n_obj * sizeof(ObjStats), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return to_status(e);
    std::vector<uint32_t> seen;
    for (uint64_t i = 0; i < n_obj; ++i)
        if (ho[i].first != kNone) seen.push_back((uint32_t)i);
    std::stable_sort(seen.begin(), seen.end(), [&](uint32_t a, uint32_t b) { return ho[a].first < ho[b].first; });
    const std::vector<uint32_t> order = map_visit_order(seen);
    const uint64_t n_vis = order.size();
    if (!n_vis) {
        e = cudaStreamSynchronize(s);
        return to_status(e);
    }
    uint32_t* d_order = nullptr;
    ObjCells* oc = nullptr;
    int32_t* ncells = nullptr;
    int64_t* off = nullptr;
    int64_t h_total = 0;
    e = sc.get(&d_order, n_vis * sizeof(uint32_t));
    if (e == cudaSuccess) e = sc.get(&oc, n_vis * sizeof(ObjCells));
    if (e == cudaSuccess) e = sc.get(&ncells, n_vis * sizeof(int32_t));
    if (e == cudaSuccess) e = sc.get(&off, (n_vis + 1) * sizeof(int64_t));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_order, order.data(), n_vis * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return to_status(e);
    const unsigned gv = (unsigned)((n_vis + kGT - 1) / kGT);
    launch(k_gs_objects, gv, kGT, 0, s, (const ObjStats*)o, (const uint32_t*)d_order, n_vis, f, (uint32_t*)d_cells,
           oc, ncells);
    e = exclusive_scan_i32_to_i64(ncells, off, n_vis, off + n_vis, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_total, off + n_vis, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return to_status(e);
    if (h_total > 0) {
        if (h_total > 0x7fffffffLL) return RS_ERR_TOO_LARGE;
        const uint64_t n = (uint64_t)h_total;
        uint64_t* cell_key = nullptr;
        uint32_t* rank = nullptr;
        e = sc.get(&cell_key, n * sizeof(uint64_t));
        if (e == cudaSuccess) e = sc.get(&rank, n * sizeof(uint32_t));
        if (e != cudaSuccess) return to_status(e);
        launch(k_gs_emit, gv, kGT, 0, s, (const ObjCells*)oc, (const int64_t*)off, n_vis, resolution, cell_key, rank);
        e = radix_sort_u64(cell_key, rank, n, bits_for(ncell - 1), s);
        if (e != cudaSuccess) return to_status(e);
        launch(k_gs_cell_sums, (unsigned)((n + kGT - 1) / kGT), kGT, 0, s, (const uint64_t*)cell_key,
               (const uint32_t*)rank, n, (const ObjCells*)oc, (uint32_t*)d_cells);
    }
    uint32_t sort_err = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = sort_error_read(&sort_err, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && sort_err) {
        sort_error_clear(s);
        return RS_ERR_ITER_LIMIT;
    }
    return to_status(e);
}
