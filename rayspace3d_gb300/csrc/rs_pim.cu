// rs_pim.cu -- point-in-mesh parity and the fused bounding-box filter.
//
// Replaces __raygen__rg (query/src/cuda/raytracing.cu:9-78) + __closesthit__ch
// (optix_common_shaders.cuh:12-19), RayLauncher (query/src/raytracing/RayLauncher.cpp:14-64),
// FilterRefinePipeline (query/src/raytracing/FilterRefine.cpp:10-122) and ResultProcessor
// (query/src/raytracing/ResultProcessor.cpp:8-60).
//
// The reference re-traces a closest-hit query from t_min = t + 1e-6 until it misses
// (crossings + 1 traversals per ray).  Here one traversal collects every crossing
// with t in [1e-6, 1e16] into a per-thread list kept sorted by (t, triangle id);
// the reference's advance rule is then applied to the sorted list.  A ray with more
// crossings than the list holds is queued for an exact fallback that walks the hits
// in the same order by re-traversal.
#include <climits>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kT = 256;
constexpr int kHits = 8;
constexpr float kEps = 1e-6f;
constexpr float kTmax = 1e16f;
constexpr int kFallbackIters = 1 << 16;

struct BoxMesh {
    float v[12][9];  // 12 triangles x (a,b,c)
};

__device__ __forceinline__ bool hit_less(float t0, uint32_t i0, float t1, uint32_t i1) {
    return t0 < t1 || (t0 == t1 && i0 < i1);
}

// Advance rule of raytracing.cu:23-60 on hits sorted by (t, id): a hit counts when
// t >= threshold; the next threshold is t + 1e-6, or the next float when that does
// not advance.
struct Chain {
    float thr = kEps;
    uint32_t count = 0;
    int32_t first_obj = -1;
    __device__ __forceinline__ void step(float t, int32_t obj) {
        if (t >= thr && t < kTmax) {
            if (count == 0) first_obj = obj;
            ++count;
            float nt = __fadd_rn(t, kEps);
            if (!(nt > t)) nt = nextafterf(t, INFINITY);
            thr = nt;
        }
    }
};

template <int AXIS>
__device__ __forceinline__ bool box_filter(const float* __restrict__ box, const Ray& r) {
    float ht[12];
    uint32_t hid[12];
    int nh = 0;
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
        if (hit_triangle<AXIS>(r, a, b, c, t)) {
            int j = nh++;
            while (j > 0 && hit_less(t, (uint32_t)k, ht[j - 1], hid[j - 1])) {
                ht[j] = ht[j - 1];
                hid[j] = hid[j - 1];
                --j;
            }
            ht[j] = t;
            hid[j] = (uint32_t)k;
        }
    }
    Chain c;
    for (int j = 0; j < nh; ++j) c.step(ht[j], 0);
    return (c.count & 1) != 0;
}

template <int AXIS, bool FILTER>
__global__ void __launch_bounds__(kT) k_pim(const float* __restrict__ pts, uint64_t n, float dx, float dy, float dz,
                                            const BNode* __restrict__ nodes, uint32_t max_steps,
                                            const float4* __restrict__ tris,
                                            const float* __restrict__ box, int32_t* __restrict__ out_obj,
                                            uint8_t* __restrict__ out_in,
                                            unsigned int* __restrict__ status, uint32_t* __restrict__ ovf_list,
                                            unsigned long long* __restrict__ ovf_count) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    const Ray r = make_ray(px, py, pz, dx, dy, dz, kEps, kTmax);
    if (FILTER && !box_filter<AXIS>(box, r)) {
        if (out_obj) out_obj[i] = -1;
        if (out_in) out_in[i] = 0;
        return;
    }
    float ht[kHits];
    uint32_t hid[kHits];
    int32_t hob[kHits];
    int nh = 0;
    bool ovf = false;
    const bool ok = traverse<AXIS>(nodes, max_steps, r, [&](int first, int cnt) {
        for (int k = first; k < first + cnt; ++k) {
            float a[3], b[3], c[3];
            uint32_t tid;
            int32_t obj;
            load_tri(tris, k, a, b, c, tid, obj);
            float t;
            if (!hit_triangle<AXIS>(r, a, b, c, t)) continue;
            if (nh == kHits) {
                ovf = true;
                continue;
            }
            int j = nh++;
            while (j > 0 && hit_less(t, tid, ht[j - 1], hid[j - 1])) {
                ht[j] = ht[j - 1];
                hid[j] = hid[j - 1];
                hob[j] = hob[j - 1];
                --j;
            }
            ht[j] = t;
            hid[j] = tid;
            hob[j] = obj;
        }
    });
    if (!ok) {
        atomicOr(status, ST_STACK_OVERFLOW);
        return;
    }
    if (ovf) {
        const unsigned long long slot = atomicAdd(ovf_count, 1ull);
        ovf_list[slot] = (uint32_t)i;
        return;
    }
    Chain ch;
    for (int j = 0; j < nh; ++j) ch.step(ht[j], hob[j]);
    const bool inside = (ch.count & 1) != 0;
    if (out_obj) out_obj[i] = inside ? ch.first_obj : -1;
    if (out_in) out_in[i] = inside ? 1 : 0;
}

// Exact fallback for rays with more than kHits crossings: each round re-traverses
// and takes the smallest (t, id) above the previous one.
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
        Chain ch;
        float pt = -INFINITY;
        uint32_t pid = 0;
        bool have_prev = false;
        int it = 0;
        for (; it < kFallbackIters; ++it) {
            float bt = INFINITY;
            uint32_t bid = 0xffffffffu;
            int32_t bobj = -1;
            bool found = false;
            const bool ok = traverse<AXIS>(nodes, max_steps, r, [&](int first, int c) {
                for (int k = first; k < first + c; ++k) {
                    float a[3], b[3], cc[3];
                    uint32_t tid;
                    int32_t obj;
                    load_tri(tris, k, a, b, cc, tid, obj);
                    float t;
                    if (!hit_triangle<AXIS>(r, a, b, cc, t)) continue;
                    if (have_prev && !hit_less(pt, pid, t, tid)) continue;
                    if (!found || hit_less(t, tid, bt, bid)) {
                        found = true;
                        bt = t;
                        bid = tid;
                        bobj = obj;
                    }
                }
            });
            if (!ok) {
                atomicOr(status, ST_STACK_OVERFLOW);
                break;
            }
            if (!found) break;
            ch.step(bt, bobj);
            pt = bt;
            pid = bid;
            have_prev = true;
        }
        if (it == kFallbackIters) atomicOr(status, ST_ITER_LIMIT);
        const bool inside = (ch.count & 1) != 0;
        if (out_obj) out_obj[i] = inside ? ch.first_obj : -1;
        if (out_in) out_in[i] = inside ? 1 : 0;
    }
}

template <int AXIS, bool FILTER>
cudaError_t launch_pim(const rs_bvh* bvh, const float* pts, uint64_t n, float dx, float dy, float dz,
                       const float* box, int32_t* obj, uint8_t* in, unsigned int* status, uint32_t* ovf_list,
                       unsigned long long* ovf_count, cudaStream_t s) {
    const unsigned grid = (unsigned)((n + kT - 1) / kT);
    k_pim<AXIS, FILTER><<<grid, kT, 0, s>>>(pts, n, dx, dy, dz, bvh->nodes, max_steps(bvh), bvh->tris, box, obj, in, status,
                                            ovf_list, ovf_count);
    k_pim_fallback<AXIS><<<2 * sm_count(), 128, 0, s>>>(pts, dx, dy, dz, bvh->nodes, max_steps(bvh), bvh->tris, obj, in, status,
                                                        ovf_list, ovf_count);
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

int pim_impl(const rs_bvh* bvh, const float* pts, uint64_t n, float dx, float dy, float dz, int32_t* obj,
             uint8_t* in, bool filter, cudaStream_t s) {
    if (!bvh || (n && !pts)) return RS_ERR_INVALID;
    if (n == 0) return RS_OK;
    if (n > 0xffffffffull) return RS_ERR_INVALID;
    if (filter && bvh->nV == 0) {
        cudaError_t e = cudaSuccess;
        if (obj) e = cudaMemsetAsync(obj, 0xff, n * sizeof(int32_t), s);
        if (e == cudaSuccess && in) e = cudaMemsetAsync(in, 0, n, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        return to_status(e);
    }
    unsigned long long* meta = nullptr;  // [0] status, [1] overflow count, then the 12 box triangles
    uint32_t* ovf = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&meta, 2 * sizeof(unsigned long long) + sizeof(BoxMesh), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&ovf, n * sizeof(uint32_t), s);
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
    const bool zx = dx == 0.0f, zy = dy == 0.0f, zz = dz == 0.0f;
    if (dz == 1.0f && zx && zy) {
        e = filter ? launch_pim<2, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<2, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    } else if (dx == 1.0f && zy && zz) {
        e = filter ? launch_pim<0, true>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s)
                   : launch_pim<0, false>(bvh, pts, n, dx, dy, dz, box, obj, in, status, ovf, meta + 1, s);
    } else if (dy == 1.0f && zx && zz) {
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
}  // namespace rs

using namespace rs;

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
    cudaError_t e = cudaMallocAsync((void**)&flags, n * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&total, sizeof(uint32_t), s);
    if (e == cudaSuccess) {
        const unsigned grid = (unsigned)((n + kT - 1) / kT);
        k_hit_flags<<<grid, kT, 0, s>>>(d_obj, n, flags);
        e = exclusive_scan_u32(flags, flags, n, total, s);
        if (e == cudaSuccess) k_hit_scatter<<<grid, kT, 0, s>>>(d_obj, n, flags, d_point_ids, d_point_obj, capacity);
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
