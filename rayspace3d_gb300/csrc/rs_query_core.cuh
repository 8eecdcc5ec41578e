// rs_query_core.cuh -- per-ray bodies shared by the single-query kernels (rs_pim.cu,
// rs_join.cu) and the batched persistent kernel (rs_batch.cu).
#pragma once
#include <climits>

#include "rs_device.cuh"

namespace rs {
namespace {

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

// Up to kHits crossings in registers: predicated append, sorting network at the end.
struct HitList {
    float t[kHits];
    uint32_t id[kHits];
    int32_t obj[kHits];
    int n = 0;
    bool ovf = false;
    __device__ __forceinline__ void add(float tt, uint32_t ii, int32_t oo) {
        if (n >= kHits) {
            ovf = true;
            return;
        }
#pragma unroll
        for (int j = 0; j < kHits; ++j)
            if (j == n) {
                t[j] = tt;
                id[j] = ii;
                obj[j] = oo;
            }
        ++n;
    }
    // Odd-even transposition sort of all kHits slots (empty slots sort last).
    __device__ __forceinline__ Chain finish() {
#pragma unroll
        for (int j = 0; j < kHits; ++j)
            if (j >= n) {
                t[j] = INFINITY;
                id[j] = 0xffffffffu;
                obj[j] = -1;
            }
#pragma unroll
        for (int r = 0; r < kHits; ++r) {
#pragma unroll
            for (int j = r & 1; j + 1 < kHits; j += 2) {
                if (hit_less(t[j + 1], id[j + 1], t[j], id[j])) {
                    const float tt = t[j]; t[j] = t[j + 1]; t[j + 1] = tt;
                    const uint32_t ii = id[j]; id[j] = id[j + 1]; id[j + 1] = ii;
                    const int32_t oo = obj[j]; obj[j] = obj[j + 1]; obj[j + 1] = oo;
                }
            }
        }
        Chain c;
#pragma unroll
        for (int j = 0; j < kHits; ++j)
            if (j < n) c.step(t[j], obj[j]);
        return c;
    }
};


__device__ __forceinline__ void write_result(const Chain& ch, uint64_t i, int32_t* out_obj, uint8_t* out_in) {
    const bool inside = (ch.count & 1) != 0;
    if (out_obj) out_obj[i] = inside ? ch.first_obj : -1;
    if (out_in) out_in[i] = inside ? 1 : 0;
}

// Every crossing of ray r with t in [1e-6, 1e16] into hl (BVH traversal).  Returns false
// on an exhausted traversal budget or stack.
template <int AXIS, int STACK>
__device__ __forceinline__ bool pim_collect(const BNode* __restrict__ nodes, uint32_t max_steps,
                                            const float4* __restrict__ tris, const Ray& r, HitList& hl,
                                            unsigned int& tests) {
    return traverse<AXIS, STACK>(nodes, max_steps, r, [&](int first, int cnt) {
        tests += (unsigned int)cnt;
        for (int k = first; k < first + cnt; ++k) {
            float a[3], b[3], c[3];
            uint32_t tid;
            int32_t obj;
            load_tri(tris, k, a, b, c, tid, obj);
            float t;
            if (hit_triangle<AXIS>(r, a, b, c, t)) hl.add(t, tid, obj);
        }
    });
}

// Exact fallback for a ray with more than kHits crossings: each round re-traverses the
// BVH and takes the smallest (t, id) above the previous one, so the crossings are
// walked in the same order as the sorted list.
template <int AXIS, int STACK>
__device__ __forceinline__ void pim_fallback_ray(const BNode* __restrict__ nodes, uint32_t max_steps,
                                                 const float4* __restrict__ tris, const Ray& r,
                                                 unsigned int* __restrict__ status, int32_t* __restrict__ out_obj,
                                                 uint8_t* __restrict__ out_in, uint64_t i) {
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
        const bool ok = traverse<AXIS, STACK>(nodes, max_steps, r, [&](int first, int c) {
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
    write_result(ch, i, out_obj, out_in);
}

// Edge ray i of mesh_overlap_edges.cu:106-216: every target object crossed with t in
// [1e-6, len + 1e-6] is paired with every source object of the edge.
template <int STACK>
__device__ __forceinline__ void edge_ray(const float* __restrict__ starts, const float* __restrict__ ends,
                                         const int32_t* __restrict__ offsets, const int32_t* __restrict__ counts,
                                         const int32_t* __restrict__ sources, uint64_t i,
                                         const BNode* __restrict__ nodes, uint32_t max_steps,
                                         const float4* __restrict__ tris, int swap, const PairTable& table) {
    const float sx = starts[3 * i], sy = starts[3 * i + 1], sz = starts[3 * i + 2];
    const float ex = ends[3 * i], ey = ends[3 * i + 1], ez = ends[3 * i + 2];
    // distance3f / normalize3f of mesh_overlap_edges.cu:47-60 as individually rounded operations.
    const float dx = __fsub_rn(ex, sx), dy = __fsub_rn(ey, sy), dz = __fsub_rn(ez, sz);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    if (len < 1e-6f) return;
    const Ray r = make_ray(sx, sy, sz, __fdiv_rn(dx, len), __fdiv_rn(dy, len), __fdiv_rn(dz, len), 1e-6f,
                           __fadd_rn(len, 1e-6f));
    const int nsrc = counts[i];
    const int32_t* src = sources + offsets[i];
    int32_t last[4] = {INT_MIN, INT_MIN, INT_MIN, INT_MIN};
    int lp = 0;
    unsigned int crossings = 0, tests = 0;
    const bool ok = traverse<-1, STACK>(nodes, max_steps, r, [&](int first, int cnt) {
        tests += (unsigned int)cnt;
        for (int k = first; k < first + cnt; ++k) {
            float a[3], b[3], c[3];
            uint32_t tid;
            int32_t obj;
            load_tri(tris, k, a, b, c, tid, obj);
            float t;
            if (!hit_triangle<-1>(r, a, b, c, t)) continue;
            ++crossings;
            if (obj == last[0] || obj == last[1] || obj == last[2] || obj == last[3]) continue;
            last[lp] = obj;
            lp = (lp + 1) & 3;
            for (int q = 0; q < nsrc; ++q) {
                const uint32_t sobj = (uint32_t)src[q];
                const unsigned long long key = swap ? (((unsigned long long)(uint32_t)obj << 32) | sobj)
                                                    : (((unsigned long long)sobj << 32) | (uint32_t)obj);
                table_insert(table, key);
            }
        }
    });
    if (!ok) atomicOr(table.status, ST_STACK_OVERFLOW);
    add_tests(tests);
    if (table.stats) {
        atomicAdd(&table.stats[2], 1ull);
        if (crossings) atomicAdd(&table.stats[3], (unsigned long long)crossings);
    }
}

}  // namespace
}  // namespace rs
