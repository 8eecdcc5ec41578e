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

struct GridView {
    float u0, v0, su, sv, u1, v1;
    int gu, gv;
    const uint32_t* start;
    const uint32_t* list;
};

// Monotone cell index: identical for triangle boxes and query points.
__device__ __forceinline__ int cell_of(float x, float x0, float s, int g) {
    float f = floorf(__fmul_rn(__fsub_rn(x, x0), s));
    f = fminf(fmaxf(f, 0.0f), (float)(g - 1));
    return (int)f;
}

// Candidates of a point from the column grid of the +e_AXIS direction (a crossed
// triangle's projected box contains the point; all boxes lie in [u0,u1]x[v0,v1]).
template <int AXIS>
__device__ __forceinline__ void grid_cell(const GridView& g, const float* p, uint32_t& begin, uint32_t& count) {
    constexpr int U = (AXIS + 1) % 3, V = (AXIS + 2) % 3;
    begin = 0;
    count = 0;
    if (p[U] >= g.u0 && p[U] <= g.u1 && p[V] >= g.v0 && p[V] <= g.v1) {
        const int c = cell_of(p[V], g.v0, g.sv, g.gv) * g.gu + cell_of(p[U], g.u0, g.su, g.gu);
        begin = __ldg(&g.start[c]);
        count = __ldg(&g.start[c + 1]) - begin;
    }
}

// Shared-memory crossing slots of one warp for pim_grid_warp.
struct GridWarpSlots {
    float t[kHits][32];
    uint32_t id[kHits][32];
    int32_t obj[kHits][32];
    int n[32];
};

// Warp-cooperative column-grid query of the warp's 32 points (all lanes call it; lanes
// without a point pass valid = false, lanes whose point was filtered out keep = false).
// The candidate lists are flattened into one (point, triangle) work list with a warp
// scan, so every lane tests one candidate per round however unevenly candidates are
// spread over the points.  Crossings go to per-point slots in shared memory; each lane
// then sorts and counts its own point's, or calls overflow() when it has more than
// kHits of them.
template <int AXIS, class Ovf>
__device__ __forceinline__ void pim_grid_warp(const GridView& g, const float4* __restrict__ tris, const float* p,
                                              bool valid, bool keep, uint64_t i, int32_t* __restrict__ out_obj,
                                              uint8_t* __restrict__ out_in, GridWarpSlots& sl, Ovf&& overflow) {
    const int lane = threadIdx.x & 31;
    const float dx = AXIS == 0 ? 1.0f : 0.0f, dy = AXIS == 1 ? 1.0f : 0.0f, dz = AXIS == 2 ? 1.0f : 0.0f;
    uint32_t b = 0, cnt = 0;
    if (keep) grid_cell<AXIS>(g, p, b, cnt);
    sl.n[lane] = 0;
    // Warp exclusive scan of the candidate counts.
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    const uint32_t pre = inc - cnt;
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    __syncwarp();
    add_tests(lane == 0 ? total : 0u);
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t j = base + lane;
        // Owner of work item j: the last lane whose prefix is <= j.
        int owner = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t pc = __shfl_sync(0xffffffffu, pre, owner + step);
            if (pc <= j) owner += step;
        }
        const uint32_t ob = __shfl_sync(0xffffffffu, b, owner);
        const uint32_t opre = __shfl_sync(0xffffffffu, pre, owner);
        const float ox = __shfl_sync(0xffffffffu, p[0], owner);
        const float oy = __shfl_sync(0xffffffffu, p[1], owner);
        const float oz = __shfl_sync(0xffffffffu, p[2], owner);
        if (j < total) {
            const int k = (int)__ldg(&g.list[ob + (j - opre)]);
            float a[3], bb[3], cc[3];
            uint32_t tid;
            int32_t obj;
            load_tri(tris, k, a, bb, cc, tid, obj);
            const Ray r = make_ray(ox, oy, oz, dx, dy, dz, kEps, kTmax);
            float t;
            if (hit_triangle<AXIS>(r, a, bb, cc, t)) {
                const int slot = atomicAdd(&sl.n[owner], 1);
                if (slot < kHits) {
                    sl.t[slot][owner] = t;
                    sl.id[slot][owner] = tid;
                    sl.obj[slot][owner] = obj;
                }
            }
        }
    }
    __syncwarp();
    if (!valid) return;
    const int nh = sl.n[lane];
    if (nh > kHits) {
        overflow();
        return;
    }
    HitList hl;
#pragma unroll
    for (int q = 0; q < kHits; ++q)
        if (q < nh) {
            hl.t[q] = sl.t[q][lane];
            hl.id[q] = sl.id[q][lane];
            hl.obj[q] = sl.obj[q][lane];
        }
    hl.n = nh;
    write_result(hl.finish(), i, out_obj, out_in);
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
constexpr int kLongHits = 64;

template <int AXIS, int STACK>
__device__ __forceinline__ void pim_fallback_ray(const BNode* __restrict__ nodes, uint32_t max_steps,
                                                 const float4* __restrict__ tris, const Ray& r,
                                                 unsigned int* __restrict__ status, int32_t* __restrict__ out_obj,
                                                 uint8_t* __restrict__ out_in, uint64_t i) {
    // One traversal into a local list of up to kLongHits crossings, insertion-sorted by
    // (t, id); only rays with more crossings walk them by re-traversal below.
    {
        float lt[kLongHits];
        uint32_t lid[kLongHits];
        int32_t lobj[kLongHits];
        int n = 0;
        bool more = false;
        const bool ok = traverse<AXIS, STACK>(nodes, max_steps, r, [&](int first, int c) {
            for (int k = first; k < first + c; ++k) {
                float a[3], b[3], cc[3];
                uint32_t tid;
                int32_t obj;
                load_tri(tris, k, a, b, cc, tid, obj);
                float t;
                if (!hit_triangle<AXIS>(r, a, b, cc, t)) continue;
                if (n == kLongHits) {
                    more = true;
                    continue;
                }
                int j = n++;
                while (j > 0 && hit_less(t, tid, lt[j - 1], lid[j - 1])) {
                    lt[j] = lt[j - 1];
                    lid[j] = lid[j - 1];
                    lobj[j] = lobj[j - 1];
                    --j;
                }
                lt[j] = t;
                lid[j] = tid;
                lobj[j] = obj;
            }
        });
        if (!ok) {
            atomicOr(status, ST_STACK_OVERFLOW);
            write_result(Chain{}, i, out_obj, out_in);
            return;
        }
        if (!more) {
            Chain ch;
            for (int j = 0; j < n; ++j) ch.step(lt[j], lobj[j]);
            write_result(ch, i, out_obj, out_in);
            return;
        }
    }
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
// The segment (sx,sy,sz) -> (ex,ey,ez) with its nsrc source objects src[0..nsrc).
template <int STACK>
__device__ __forceinline__ void segment_ray(float sx, float sy, float sz, float ex, float ey, float ez,
                                            const int32_t* __restrict__ src, int nsrc,
                                            const BNode* __restrict__ nodes, uint32_t max_steps,
                                            const float4* __restrict__ tris, int swap, const PairTable& table) {
    // distance3f / normalize3f of mesh_overlap_edges.cu:47-60 as individually rounded operations.
    const float dx = __fsub_rn(ex, sx), dy = __fsub_rn(ey, sy), dz = __fsub_rn(ez, sz);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    if (len < 1e-6f) return;
    const Ray r = make_ray(sx, sy, sz, __fdiv_rn(dx, len), __fdiv_rn(dy, len), __fdiv_rn(dz, len), 1e-6f,
                           __fadd_rn(len, 1e-6f));
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

template <int STACK>
__device__ __forceinline__ void edge_ray(const float* __restrict__ starts, const float* __restrict__ ends,
                                         const int32_t* __restrict__ offsets, const int32_t* __restrict__ counts,
                                         const int32_t* __restrict__ sources, uint64_t i,
                                         const BNode* __restrict__ nodes, uint32_t max_steps,
                                         const float4* __restrict__ tris, int swap, const PairTable& table) {
    segment_ray<STACK>(starts[3 * i], starts[3 * i + 1], starts[3 * i + 2], ends[3 * i], ends[3 * i + 1],
                       ends[3 * i + 2], sources + offsets[i], counts[i], nodes, max_steps, tris, swap, table);
}

// Edge e of triangle t of a source mesh, in the triangle's own orientation (v0v1, v1v2,
// v2v0), with the triangle's object as its one source: the legacy per-triangle overlap
// (mesh_overlap.cu:126-179), which traces shared edges once per triangle.
template <int STACK>
__device__ __forceinline__ void triangle_edge_ray(const float* __restrict__ V, const uint32_t* __restrict__ I,
                                                  const int32_t* __restrict__ T, uint64_t r,
                                                  const BNode* __restrict__ nodes, uint32_t max_steps,
                                                  const float4* __restrict__ tris, int swap, const PairTable& table) {
    const uint64_t t = r / 3;
    const int e = (int)(r % 3);
    const uint64_t a = I[3 * t + e], b = I[3 * t + (e == 2 ? 0 : e + 1)];
    segment_ray<STACK>(V[3 * a], V[3 * a + 1], V[3 * a + 2], V[3 * b], V[3 * b + 1], V[3 * b + 2], T + t, 1, nodes,
                       max_steps, tris, swap, table);
}

}  // namespace
}  // namespace rs
