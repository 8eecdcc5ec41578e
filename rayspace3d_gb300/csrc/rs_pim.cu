// rs_pim.cu -- point-in-mesh parity and the fused bounding-box filter.
//
// Replaces __raygen__rg (query/src/cuda/raytracing.cu:9-78) + __closesthit__ch
// (optix_common_shaders.cuh:12-19), RayLauncher (query/src/raytracing/RayLauncher.cpp:14-64),
// FilterRefinePipeline (query/src/raytracing/FilterRefine.cpp:10-122) and ResultProcessor
// (query/src/raytracing/ResultProcessor.cpp:8-60).
//
// The reference re-traces a closest-hit query from t_min = t + 1e-6 until it misses
// (crossings + 1 traversals per ray).  Here every crossing with t in [1e-6, 1e16] is
// collected once into a per-thread register list, sorted by (t, triangle id), and the
// reference's advance rule is applied to the sorted list.  A ray with more crossings
// than the list holds is queued for an exact fallback that walks the hits in the same
// order by re-traversal.
//
// Candidates come from one of two structures with the same hit set:
//  * rays along +x, +y or +z use a column grid: a uniform 2D grid over the projection
//    of the leaf-ordered triangles.  Triangle boxes and query points go through the
//    same monotone cell formula, so every triangle whose projection can contain the
//    (perturbed) point is in the point's cell;
//  * any other direction traverses the BVH.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>

#include "rs_engine.h"
#include "rs_prims.cuh"
#include "rs_query_core.cuh"

namespace rs {
namespace {

constexpr int kT = 256;
template <int AXIS>
__device__ __forceinline__ bool box_filter(const float* __restrict__ box, const Ray& r) {
    HitList hl;
#pragma unroll 1
    for (int k = 0; k < 12; ++k) {
        float a[3], b[3], c[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            a[q] = __ldg(&box[9 * k + q]);
            b[q] = __ldg(&box[9 * k + 3 + q]);
            c[q] = __ldg(&box[9 * k + 6 + q]);
        }
        float t;
        if (hit_triangle<AXIS>(r, a, b, c, t)) hl.add(t, (uint32_t)k, 0);
    }
    // A ray crosses at most two of the 12 faces under the hit contract.
    const Chain ch = hl.finish();
    return (ch.count & 1) != 0;
}


template <int AXIS, bool FILTER>
__global__ void __launch_bounds__(kT) k_pim(const float* __restrict__ pts, uint64_t n, float dx, float dy, float dz,
                                            const BNode* __restrict__ nodes, uint32_t max_steps,
                                            const float4* __restrict__ tris, const float* __restrict__ box,
                                            int32_t* __restrict__ out_obj, uint8_t* __restrict__ out_in,
                                            unsigned int* __restrict__ status, uint32_t* __restrict__ ovf_list,
                                            unsigned long long* __restrict__ ovf_count) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Ray r = make_ray(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], dx, dy, dz, kEps, kTmax);
    if (FILTER && !box_filter<AXIS>(box, r)) {
        write_result(Chain{}, i, out_obj, out_in);
        return;
    }
    HitList hl;
    unsigned int tests = 0;
    const bool ok = pim_collect<AXIS, kStack>(nodes, max_steps, tris, r, hl, tests);
    add_tests(tests);
    if (!ok) {
        atomicOr(status, ST_STACK_OVERFLOW);
        return;
    }
    if (hl.ovf) {
        ovf_list[atomicAdd(ovf_count, 1ull)] = (uint32_t)i;
        return;
    }
    write_result(hl.finish(), i, out_obj, out_in);
}

// Warp-cooperative column-grid query.  Each warp owns 32 points; their candidate
// lists are flattened into one (point, triangle) work list with a warp scan, so every
// lane tests one candidate per round however unevenly the candidates are spread over
// the points (points outside the projected bounds contribute none).  Crossings go to
// per-point slots in shared memory; each lane then sorts and counts its own point's.
constexpr int kWarps = kT / 32;

template <int AXIS, bool FILTER>
__global__ void __launch_bounds__(kT) k_pim_grid(const float* __restrict__ pts, uint64_t n, GridView g,
                                                 const float4* __restrict__ tris, const float* __restrict__ box,
                                                 int32_t* __restrict__ out_obj, uint8_t* __restrict__ out_in,
                                                 uint32_t* __restrict__ ovf_list,
                                                 unsigned long long* __restrict__ ovf_count) {
    __shared__ GridWarpSlots slots[kWarps];
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const bool valid = i < n;
    float p[3] = {0.0f, 0.0f, 0.0f};
    if (valid) {
        p[0] = pts[3 * i];
        p[1] = pts[3 * i + 1];
        p[2] = pts[3 * i + 2];
    }
    bool keep = valid;
    if (FILTER && valid)
        keep = box_filter<AXIS>(box, make_ray(p[0], p[1], p[2], AXIS == 0 ? 1.0f : 0.0f, AXIS == 1 ? 1.0f : 0.0f,
                                              AXIS == 2 ? 1.0f : 0.0f, kEps, kTmax));
    pim_grid_warp<AXIS>(g, tris, p, valid, keep, i, out_obj, out_in, slots[threadIdx.x >> 5],
                        [&]() { ovf_list[atomicAdd(ovf_count, 1ull)] = (uint32_t)i; });
}

// Exact fallback for rays with more than kHits crossings (pim_fallback_ray).
template <int AXIS>
__global__ void __launch_bounds__(kT) k_pim_fallback(const float* __restrict__ pts, float dx, float dy, float dz,
                                                     const BNode* __restrict__ nodes, uint32_t max_steps,
                                                     const float4* __restrict__ tris,
                                                     int32_t* __restrict__ out_obj, uint8_t* __restrict__ out_in,
                                                     unsigned int* __restrict__ status,
                                                     const uint32_t* __restrict__ ovf_list,
                                                     const unsigned long long* __restrict__ ovf_count) {
    const unsigned long long cnt = *ovf_count;
    for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < cnt;
         q += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t i = ovf_list[q];
        const Ray r = make_ray(pts[3 * (uint64_t)i], pts[3 * (uint64_t)i + 1], pts[3 * (uint64_t)i + 2], dx, dy, dz,
                               kEps, kTmax);
        pim_fallback_ray<AXIS, kStack>(nodes, max_steps, tris, r, status, out_obj, out_in, i);
    }
}

// --- column grid build ---------------------------------------------------------------

template <int AXIS>
__device__ __forceinline__ void tri_uv_box(const float4* __restrict__ tris, int k, float& ul, float& uh, float& vl,
                                           float& vh) {
    const float4 a = __ldg(&tris[3 * (size_t)k]), b = __ldg(&tris[3 * (size_t)k + 1]),
                 c = __ldg(&tris[3 * (size_t)k + 2]);
    const float au = AXIS == 0 ? a.y : (AXIS == 1 ? a.z : a.x), av = AXIS == 0 ? a.z : (AXIS == 1 ? a.x : a.y);
    const float bu = AXIS == 0 ? b.y : (AXIS == 1 ? b.z : b.x), bv = AXIS == 0 ? b.z : (AXIS == 1 ? b.x : b.y);
    const float cu = AXIS == 0 ? c.y : (AXIS == 1 ? c.z : c.x), cv = AXIS == 0 ? c.z : (AXIS == 1 ? c.x : c.y);
    ul = fminf(fminf(au, bu), cu);
    uh = fmaxf(fmaxf(au, bu), cu);
    vl = fminf(fminf(av, bv), cv);
    vh = fmaxf(fmaxf(av, bv), cv);
}

__device__ __forceinline__ int ford(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

template <int AXIS>
__global__ void k_cg_bounds(const float4* __restrict__ tris, int n, int* __restrict__ b) {
    float ul = INFINITY, uh = -INFINITY, vl = INFINITY, vh = -INFINITY;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float a0, a1, a2, a3;
        tri_uv_box<AXIS>(tris, k, a0, a1, a2, a3);
        ul = fminf(ul, a0);
        uh = fmaxf(uh, a1);
        vl = fminf(vl, a2);
        vh = fmaxf(vh, a3);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ul = fminf(ul, __shfl_xor_sync(0xffffffffu, ul, o));
        uh = fmaxf(uh, __shfl_xor_sync(0xffffffffu, uh, o));
        vl = fminf(vl, __shfl_xor_sync(0xffffffffu, vl, o));
        vh = fmaxf(vh, __shfl_xor_sync(0xffffffffu, vh, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&b[0], ford(ul));
        atomicMax(&b[1], ford(uh));
        atomicMin(&b[2], ford(vl));
        atomicMax(&b[3], ford(vh));
    }
}

template <int AXIS, bool FILL>
__global__ void k_cg_cells(const float4* __restrict__ tris, int n, GridView g, uint32_t* __restrict__ count,
                           uint32_t* __restrict__ list) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float ul, uh, vl, vh;
    tri_uv_box<AXIS>(tris, k, ul, uh, vl, vh);
    const int cu0 = cell_of(ul, g.u0, g.su, g.gu), cu1 = cell_of(uh, g.u0, g.su, g.gu);
    const int cv0 = cell_of(vl, g.v0, g.sv, g.gv), cv1 = cell_of(vh, g.v0, g.sv, g.gv);
    for (int cv = cv0; cv <= cv1; ++cv)
        for (int cu = cu0; cu <= cu1; ++cu) {
            const int c = cv * g.gu + cu;
            const uint32_t slot = atomicAdd(&count[c], 1u);
            if (FILL) list[g.start[c] + slot] = (uint32_t)k;
        }
}

std::mutex g_grid_mu;

float dec_ord(int i) {
    int x = i >= 0 ? i : i ^ 0x7fffffff;
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

template <int AXIS>
cudaError_t build_grid(rs_bvh* bvh, cudaStream_t s) {
    rs_column_grid& cg = bvh->cgrid[AXIS];
    const int n = (int)bvh->n_tris;
    int* b = nullptr;
    cudaError_t e = dmalloc((void**)&b, 4 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int init[4] = {0x7fffffff, (int)0x80000000, 0x7fffffff, (int)0x80000000};
    cudaMemcpyAsync(b, init, sizeof(init), cudaMemcpyHostToDevice, s);
    launch(k_cg_bounds<AXIS>, 2 * sm_count(), 256, 0, s, (const float4*)bvh->tris, n, b);
    int hb[4];
    e = cudaMemcpyAsync(hb, b, sizeof(hb), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(b, s);
    if (e != cudaSuccess) return e;
    cg.u0 = dec_ord(hb[0]);
    cg.u1 = dec_ord(hb[1]);
    cg.v0 = dec_ord(hb[2]);
    cg.v1 = dec_ord(hb[3]);
    // About four cells per triangle, shaped like the projected bounds.
    const double target = std::min(std::max(4.0 * n, 1.0), (double)(1 << 24));
    const double w = (double)cg.u1 - cg.u0, h = (double)cg.v1 - cg.v0;
    int gu = 1, gv = 1;
    if (w > 0 && h > 0) {
        gu = (int)std::lround(std::sqrt(target * w / h));
        gu = std::min(std::max(gu, 1), 8192);
        gv = (int)std::min(std::max(std::lround(target / gu), 1L), 8192L);
    } else if (w > 0) {
        gu = (int)std::min(target, 8192.0);
    } else if (h > 0) {
        gv = (int)std::min(target, 8192.0);
    }
    cg.gu = gu;
    cg.gv = gv;
    cg.su = w > 0 ? (float)gu / (float)w : 0.0f;
    cg.sv = h > 0 ? (float)gv / (float)h : 0.0f;
    const size_t ncell = (size_t)gu * gv;
    uint32_t* count = nullptr;
    e = dmalloc((void**)&count, ncell * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = dmalloc((void**)&cg.start, (ncell + 1) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    GridView gvw{cg.u0, cg.v0, cg.su, cg.sv, cg.u1, cg.v1, gu, gv, cg.start, nullptr};
    cudaMemsetAsync(count, 0, ncell * sizeof(uint32_t), s);
    const unsigned grid = (unsigned)((n + 255) / 256);
    launch(k_cg_cells<AXIS, false>, grid, 256, 0, s, (const float4*)bvh->tris, n, gvw, count, (uint32_t*)nullptr);
    e = exclusive_scan_u32(count, cg.start, ncell, cg.start + ncell, s);
    uint32_t total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, cg.start + ncell, sizeof(total), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = dmalloc((void**)&cg.list, (size_t)std::max<uint32_t>(total, 1) * 4, s);
    if (e == cudaSuccess) {
        cudaMemsetAsync(count, 0, ncell * sizeof(uint32_t), s);
        launch(k_cg_cells<AXIS, true>, grid, 256, 0, s, (const float4*)bvh->tris, n, gvw, count, cg.list);
        e = cudaGetLastError();
    }
    cudaFreeAsync(count, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cg.nlist = total;
    if (e == cudaSuccess) cg.built = 1;
    return e;
}

template <int AXIS, bool FILTER>
cudaError_t launch_pim(const rs_bvh* bvh, const float* pts, uint64_t n, float dx, float dy, float dz,
                       const float* box, int32_t* obj, uint8_t* in, unsigned int* status, uint32_t* ovf_list,
                       unsigned long long* ovf_count, cudaStream_t s) {
    const unsigned grid = (unsigned)((n + kT - 1) / kT);
    constexpr int GA = AXIS < 0 ? 0 : AXIS;
    const int ptok = prof_begin(P_PIM, s);
    if (AXIS >= 0 && bvh->cgrid[GA].built) {
        const rs_column_grid& cg = bvh->cgrid[GA];
        GridView g{cg.u0, cg.v0, cg.su, cg.sv, cg.u1, cg.v1, cg.gu, cg.gv, cg.start, cg.list};
        launch(k_pim_grid<GA, FILTER>, grid, kT, 0, s, pts, n, g, (const float4*)bvh->tris, box, obj, in, ovf_list,
               ovf_count);
    } else {
        launch(k_pim<AXIS, FILTER>, grid, kT, 0, s, pts, n, dx, dy, dz, bvh->nodes, max_steps(bvh),
               (const float4*)bvh->tris, box, obj, in, status, ovf_list, ovf_count);
    }
    prof_end(P_PIM, s, ptok);
    // One thread per possible overflow entry (the count is only known on the device);
    // threads past it return at once.
    launch(k_pim_fallback<AXIS>, (unsigned)((n + kT - 1) / kT), kT, 0, s, pts, dx, dy, dz, bvh->nodes, max_steps(bvh),
           (const float4*)bvh->tris, obj, in, status, ovf_list, ovf_count);
    return cudaGetLastError();
}

BoxMesh make_box(const rs_bvh* bvh) {
    // BoundingBox::createBoxMesh (query/src/geometry/BoundingBox.cpp:12-50).
    const float* mn = bvh->vmin;
    const float* mx = bvh->vmax;
    const float verts[8][3] = {{mn[0], mn[1], mn[2]}, {mx[0], mn[1], mn[2]}, {mx[0], mx[1], mn[2]},
                               {mn[0], mx[1], mn[2]}, {mn[0], mn[1], mx[2]}, {mx[0], mn[1], mx[2]},
                               {mx[0], mx[1], mx[2]}, {mn[0], mx[1], mx[2]}};
    const int tri[12][3] = {{0, 2, 1}, {0, 3, 2}, {4, 5, 6}, {4, 6, 7}, {0, 1, 5}, {0, 5, 4},
                            {3, 6, 2}, {3, 7, 6}, {0, 4, 7}, {0, 7, 3}, {1, 2, 6}, {1, 6, 5}};
    BoxMesh b;
    for (int t = 0; t < 12; ++t)
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) b.v[t][3 * c + k] = verts[tri[t][c]][k];
    return b;
}

int pim_impl(const rs_bvh* cbvh, const float* pts, uint64_t n, float dx, float dy, float dz, int32_t* obj,
             uint8_t* in, bool filter, cudaStream_t s) {
    if (!cbvh || (n && !pts)) return RS_ERR_INVALID;
    if (n == 0) return RS_OK;
    if (n > 0xffffffffull) return RS_ERR_INVALID;
    rs_bvh* bvh = const_cast<rs_bvh*>(cbvh);
    int st = filter ? bvh_ready(bvh) : RS_OK;
    if (st == RS_OK) st = bvh_use(bvh, s);
    if (st != RS_OK) return st;
    if (filter && bvh->nV == 0) {
        cudaError_t e = cudaSuccess;
        if (obj) e = cudaMemsetAsync(obj, 0xff, n * sizeof(int32_t), s);
        if (e == cudaSuccess && in) e = cudaMemsetAsync(in, 0, n, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return to_status(e);
    }
    const bool zx = dx == 0.0f, zy = dy == 0.0f, zz = dz == 0.0f;
    int axis = -1;
    if (dz == 1.0f && zx && zy) axis = 2;
    else if (dx == 1.0f && zy && zz) axis = 0;
    else if (dy == 1.0f && zx && zz) axis = 1;
    if (axis >= 0) {
        st = ensure_grid(bvh, axis, s);
        if (st != RS_OK) return st;
    }
    unsigned long long* meta = nullptr;  // [0] status, [1] overflow count, then the 12 box triangles
    uint32_t* ovf = nullptr;
    cudaError_t e = dmalloc((void**)&meta, 2 * sizeof(unsigned long long) + sizeof(BoxMesh), s);
    if (e == cudaSuccess) e = dmalloc((void**)&ovf, n * sizeof(uint32_t), s);
    if (e != cudaSuccess) {
        if (meta) cudaFreeAsync(meta, s);
        cudaStreamSynchronize(s);
        return to_status(e);
    }
    cudaMemsetAsync(meta, 0, 2 * sizeof(unsigned long long), s);
    unsigned int* status = reinterpret_cast<unsigned int*>(meta);
    static_assert(sizeof(BoxMesh) == 108 * sizeof(float), "box mesh layout");
    BoxMesh hbox = filter ? make_box(bvh) : BoxMesh{};
    float* box = reinterpret_cast<float*>(meta + 2);
    if (filter) cudaMemcpyAsync(box, &hbox, sizeof(BoxMesh), cudaMemcpyHostToDevice, s);
    if (axis == 2) {
        e = filter ? launch_pim<2, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<2, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    } else if (axis == 0) {
        e = filter ? launch_pim<0, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<0, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    } else if (axis == 1) {
        e = filter ? launch_pim<1, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<1, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    } else {
        e = filter ? launch_pim<-1, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<-1, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    }
    unsigned long long hmeta[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hmeta, meta, sizeof(hmeta), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(meta, s);
    cudaFreeAsync(ovf, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    prof_collect();
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return to_status(e);
    return status_from_bits((uint32_t)hmeta[0]);
}

__global__ void k_hit_flags(const int32_t* __restrict__ obj, uint64_t n, uint32_t* __restrict__ flags) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) flags[i] = obj[i] != -1;
}

__global__ void k_hit_scatter(const int32_t* __restrict__ obj, uint64_t n, const uint32_t* __restrict__ pos,
                              int32_t* __restrict__ ids, int32_t* __restrict__ objs, uint64_t capacity) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n || obj[i] == -1) return;
    const uint32_t p = pos[i];
    if (p < capacity) {
        if (ids) ids[p] = (int32_t)i;
        if (objs) objs[p] = obj[i];
    }
}

}  // namespace

// The column grid of one axis is built once per handle, like the index build of the
// reference (allocates and synchronises the stream).
int ensure_grid(const rs_bvh* cbvh, int axis, cudaStream_t s) {
    rs_bvh* bvh = const_cast<rs_bvh*>(cbvh);
    if (axis < 0 || axis > 2 || bvh->n_tris == 0 || bvh->cgrid[axis].built) return RS_OK;
    std::lock_guard<std::mutex> g(g_grid_mu);
    if (!bvh->cgrid[axis].built) {
        cudaError_t e = axis == 0 ? build_grid<0>(bvh, s) : (axis == 1 ? build_grid<1>(bvh, s) : build_grid<2>(bvh, s));
        if (e != cudaSuccess) return to_status(e);
    }
    return RS_OK;
}


int recheck_pim(int op, unsigned long long* out) { return recheck_op(op, out); }

}  // namespace rs

// ---------------------------------------------------------------------------
// Point-in-mesh without device allocation.
//
// Callers that cannot allocate device memory on their query path -- services whose
// own allocator has reserved the whole GPU, or hosts with a fixed device-memory budget
// checked per request -- use rs_pim_noalloc.  It waits for the stream and returns once
// the results are written.  Its per-call scratch (status word, overflow count, the twelve
// filter-box triangles and the list of points with more than kHits crossings) lives
// in the fixed array below instead of coming from an allocator.  Host code may not
// use the array's name as a device address, so its address is looked up with
// cudaGetSymbolAddress once per device (with that device current) and passed to
// the kernels.
// ---------------------------------------------------------------------------
constexpr uint64_t kNoAllocMaxPoints = 1ull << 20;  // 1,048,576 points per call
constexpr size_t kNoAllocMetaOffset = 0;            // u64 status, u64 overflow count
constexpr size_t kNoAllocBoxOffset = 256;           // 108 floats
constexpr size_t kNoAllocListOffset = 1024;         // u32 per point
constexpr size_t kNoAllocBytes = kNoAllocListOffset + kNoAllocMaxPoints * sizeof(uint32_t);

static __device__ __align__(256) unsigned char g_pim_scratch[kNoAllocBytes];

namespace rs {
namespace {
std::mutex g_scratch_mu;
void* g_scratch_ptr[64] = {};

// Device address of g_pim_scratch on the current device (looked up on first use).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_pim_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}
}  // namespace
}  // namespace rs

using namespace rs;

extern "C" int rs_pim_noalloc(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
                              int32_t* d_obj, uint8_t* d_inside, int filtered, void* stream) {
    if (!bvh || (n && !d_points)) return RS_ERR_INVALID;
    if (n > kNoAllocMaxPoints) return RS_ERR_TOO_LARGE;
    if (n == 0) return RS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int st = filtered ? bvh_ready(bvh) : RS_OK;
    if (st == RS_OK) st = bvh_use(bvh, s);
    if (st != RS_OK) return st;
    if (filtered && bvh->nV == 0) {
        cudaError_t e = cudaSuccess;
        if (d_obj) e = cudaMemsetAsync(d_obj, 0xff, n * sizeof(int32_t), s);
        if (e == cudaSuccess && d_inside) e = cudaMemsetAsync(d_inside, 0, n, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return to_status(e);
    }
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return to_status(e);
    unsigned char* sc = static_cast<unsigned char*>(base);
    unsigned long long* meta = reinterpret_cast<unsigned long long*>(sc + kNoAllocMetaOffset);
    float* box = reinterpret_cast<float*>(sc + kNoAllocBoxOffset);
    uint32_t* ovf = reinterpret_cast<uint32_t*>(sc + kNoAllocListOffset);
    // The array keeps the previous call's contents: the status word and overflow count
    // must start at zero (the list is written before it is read).
    e = cudaMemsetAsync(meta, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return to_status(e);
    if (filtered) {
        const BoxMesh hbox = make_box(bvh);
        e = cudaMemcpyAsync(box, &hbox, sizeof(BoxMesh), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return to_status(e);
    }
    unsigned int* status = reinterpret_cast<unsigned int*>(meta);
    const bool zx = dx == 0.0f, zy = dy == 0.0f, zz = dz == 0.0f;
    // The column grid is used when it already exists; it is never built here, because
    // building it allocates.  Without it the BVH path gives the same results.
    const bool f = filtered != 0;
    if (dz == 1.0f && zx && zy) {
        e = f ? launch_pim<2, true>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s)
              : launch_pim<2, false>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s);
    } else if (dx == 1.0f && zy && zz) {
        e = f ? launch_pim<0, true>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s)
              : launch_pim<0, false>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s);
    } else if (dy == 1.0f && zx && zz) {
        e = f ? launch_pim<1, true>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s)
              : launch_pim<1, false>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s);
    } else {
        e = f ? launch_pim<-1, true>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s)
              : launch_pim<-1, false>(bvh, d_points, n, dx, dy, dz, box, d_obj, d_inside, status, ovf, meta + 1, s);
    }
    unsigned long long hmeta[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hmeta, meta, sizeof(hmeta), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    prof_collect();
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return to_status(e);
    return status_from_bits((uint32_t)hmeta[0]);
}

extern "C" int rs_pim(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
                      int32_t* d_obj, uint8_t* d_inside, void* stream) {
    return pim_impl(bvh, d_points, n, dx, dy, dz, d_obj, d_inside, false, (cudaStream_t)stream);
}

extern "C" int rs_pim_filtered(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
                               int32_t* d_obj, uint8_t* d_inside, void* stream) {
    return pim_impl(bvh, d_points, n, dx, dy, dz, d_obj, d_inside, true, (cudaStream_t)stream);
}

extern "C" int rs_compact_hits(const int32_t* d_obj, uint64_t n, int32_t* d_point_ids, int32_t* d_point_obj,
                               uint64_t capacity, uint64_t* h_count, void* stream) {
    if (!h_count || (n && !d_obj) || n > 0xffffffffull) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    *h_count = 0;
    if (n == 0) return RS_OK;
    uint32_t* flags = nullptr;
    uint32_t* total = nullptr;
    cudaError_t e = dmalloc((void**)&flags, n * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = dmalloc((void**)&total, sizeof(uint32_t), s);
    if (e == cudaSuccess) {
        const unsigned grid = (unsigned)((n + kT - 1) / kT);
        launch(k_hit_flags, grid, kT, 0, s, d_obj, n, flags);
        e = exclusive_scan_u32(flags, flags, n, total, s);
        if (e == cudaSuccess) launch(k_hit_scatter, grid, kT, 0, s, d_obj, n, flags, d_point_ids, d_point_obj, capacity);
    }
    uint32_t ht = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ht, total, sizeof(ht), cudaMemcpyDeviceToHost, s);
    if (flags) cudaFreeAsync(flags, s);
    if (total) cudaFreeAsync(total, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return to_status(e);
    *h_count = ht;
    return ht > capacity ? RS_ERR_OUTPUT_OVERFLOW : RS_OK;
}
