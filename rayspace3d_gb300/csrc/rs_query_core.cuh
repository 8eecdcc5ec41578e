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

// Iteration cap of the parity loop (raytracing.cu:26).
constexpr uint32_t kPimMaxIters = 10000;

// Advance rule of raytracing.cu:23-60 on hits sorted by (t, id): a hit counts when
// t >= threshold; the next threshold is t + 1e-6.  When t + 1e-6 rounds back to t
// (t >= 32) the reference's next trace starts at t and finds that hit again on every
// remaining iteration, so the count ends at the 10000-iteration cap; the count is
// capped there in any case.
struct Chain {
    float thr = kEps;
    uint32_t count = 0;
    int32_t first_obj = -1;
    __device__ __forceinline__ void step(float t, int32_t obj) {
        if (count < kPimMaxIters && t >= thr && t < kTmax) {
            if (count == 0) first_obj = obj;
            ++count;
            const float nt = __fadd_rn(t, kEps);
            if (!(nt > t)) count = kPimMaxIters;
            thr = nt;
        }
    }
};

// Hit sequence of the edge loops (mesh_overlap_edges.cu:106-178, mesh_intersection.cu:16-91,
// mesh_overlap.cu:13-70): repeated closest-hit traces over [t_min, len + 1e-6] with t_min
// starting at 1e-6 and moving to t + 1e-6 after each hit (t + 2e-4 when that does not
// advance), at most max_hits traces.  On hits sorted by (t, id) that is a greedy walk:
// a hit is taken when t >= t_min.  When neither step advances, every later trace finds the
// same hit again, which adds no pair, so the walk stops.  next_float selects the strict
// containment join's edge loop (mesh_containment.cu:99-170): t_min moves to the next float
// after t, so every distinct distance is taken once.
struct EdgeWalk {
    float thr = kEps;
    int n = 0;
    bool done = false;
    __device__ __forceinline__ bool take(float t, int max_hits, int next_float) {
        if (done || !(t >= thr)) return false;
        if (++n >= max_hits) done = true;
        float nt;
        if (next_float) {
            nt = nextafterf(t, INFINITY);
        } else {
            nt = __fadd_rn(t, kEps);
            if (!(nt > t)) nt = __fadd_rn(t, 2e-4f);
            if (!(nt > t)) done = true;
        }
        thr = nt;
        return true;
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
    __device__ __forceinline__ void sort() {
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
    }
    __device__ __forceinline__ Chain finish() {
        sort();
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
    for (; it < kFallbackIters && ch.count < kPimMaxIters; ++it) {
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

// ---------------------------------------------------------------------------
// Edge rays.  The fast path traces an edge once with its stack and its crossings
// (up to kEdgeHits) in a column of shared memory; an edge with more crossings, or a
// traversal deeper than the fast stack, is deferred untouched to the long path, which
// runs the reference's trace loop literally.
// ---------------------------------------------------------------------------
constexpr int kEdgeHits = 4;

// One thread's shared-memory column: element k of an array at base[k * stride].
struct EdgeColumn {
    int* stack;
    float* t;
    uint32_t* id;
    int32_t* obj;
    int stride;
};

// Shared-memory block of the fast path for T threads and a STACK-entry stack.
template <int T, int STACK>
struct EdgeSmem {
    int stack[STACK][T];
    float t[kEdgeHits][T];
    uint32_t id[kEdgeHits][T];
    int32_t obj[kEdgeHits][T];
    __device__ __forceinline__ EdgeColumn column(int tid) {
        return EdgeColumn{&stack[0][tid], &t[0][tid], &id[0][tid], &obj[0][tid], T};
    }
};

// The segment's ray as distance3f / normalize3f of mesh_overlap_edges.cu:47-60 compute it,
// one rounded operation at a time; false for edges shorter than 1e-6 (never traced).
__device__ __forceinline__ bool segment_ray_of(float sx, float sy, float sz, float ex, float ey, float ez, Ray& r) {
    const float dx = __fsub_rn(ex, sx), dy = __fsub_rn(ey, sy), dz = __fsub_rn(ez, sz);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    if (len < 1e-6f) return false;
    r = make_ray(sx, sy, sz, __fdiv_rn(dx, len), __fdiv_rn(dy, len), __fdiv_rn(dz, len), 1e-6f, __fadd_rn(len, 1e-6f));
    return true;
}

// (source, target) -- (target, source) when swap -- for every source object of the edge.
__device__ __forceinline__ void insert_sources(const PairTable& table, const int32_t* __restrict__ src, int nsrc,
                                               int32_t obj, int swap) {
    for (int q = 0; q < nsrc; ++q) {
        const uint32_t sobj = (uint32_t)src[q];
        const unsigned long long key = swap ? (((unsigned long long)(uint32_t)obj << 32) | sobj)
                                            : (((unsigned long long)sobj << 32) | (uint32_t)obj);
        table_insert(table, key);
    }
}

__device__ __forceinline__ void count_edge(const PairTable& table, int taken) {
    if (table.stats) {
        atomicAdd(&table.stats[2], 1ull);
        if (taken) atomicAdd(&table.stats[3], (unsigned long long)taken);
    }
}

// Edge ray of mesh_overlap_edges.cu:106-216, fast path: one traversal over
// t in [1e-6, len + 1e-6] with the stack and crossings in the thread's shared-memory
// column; the crossings, sorted by (t, triangle id), are walked with the table's hit rule
// (EdgeWalk) and every target object of a hit taken is paired with every source object.
// Returns false, having inserted nothing, when the edge has more than kEdgeHits crossings
// or the traversal ran out of stack or steps: the caller then defers it to segment_long.
template <int STACK>
__device__ __forceinline__ bool segment_fast(const EdgeColumn& col, const Ray& r, const int32_t* __restrict__ src,
                                             int nsrc, const BNode* __restrict__ nodes, uint32_t max_steps,
                                             const float4* __restrict__ tris, int swap, const PairTable& table,
                                             int start = 0) {
    const int S = col.stride;
    int n = 0;
    unsigned int tests = 0;
    const bool ok = traverse_with<-1, STACK>(col.stack, S, nodes, max_steps, r, [&](int first, int cnt) {
        tests += (unsigned int)cnt;
        for (int k = first; k < first + cnt; ++k) {
            float a[3], b[3], c[3];
            uint32_t tid;
            int32_t obj;
            load_tri(tris, k, a, b, c, tid, obj);
            float t;
            if (!hit_triangle<-1>(r, a, b, c, t)) continue;
            if (n < kEdgeHits) {
                // Insertion into the sorted column.
                int j = n;
                while (j > 0 && hit_less(t, tid, col.t[(j - 1) * S], col.id[(j - 1) * S])) {
                    col.t[j * S] = col.t[(j - 1) * S];
                    col.id[j * S] = col.id[(j - 1) * S];
                    col.obj[j * S] = col.obj[(j - 1) * S];
                    --j;
                }
                col.t[j * S] = t;
                col.id[j * S] = tid;
                col.obj[j * S] = obj;
            }
            ++n;
        }
    }, start);
    add_tests(tests);
    if (!ok || n > kEdgeHits) return false;
    EdgeWalk w;
    int32_t last = INT_MIN;
    for (int j = 0; j < n; ++j) {
        if (!w.take(col.t[j * S], table.max_hits, table.next_float)) continue;
        const int32_t obj = col.obj[j * S];
        if (obj == last) continue;
        last = obj;
        insert_sources(table, src, nsrc, obj, swap);
    }
    count_edge(table, w.n);
    return true;
}

// Long path, in the reference loop's order: the crossings in [t_min, len + 1e-6] are
// walked in (t, triangle id) order with the table's hit rule, kLongChunk at a time.  Each
// pass traverses once, nearer child first, and keeps the kLongChunk smallest crossings
// beyond the last one walked (the ray's tmax shrinks to the largest kept one once the
// chunk is full, so the pass visits little beyond it); the walk then takes them, and a full chunk starts the
// next pass after its last crossing.  A crossing's t does not depend on tmin or tmax (the
// node and triangle slab tests only accept or reject), so the passes see exactly the
// crossings the reference's one-hit-per-trace loop sees, in the same order, while an
// edge with h crossings costs about h / kLongChunk traversals instead of h.
constexpr int kLongChunk = 16;

__device__ __forceinline__ void segment_long(Ray r, const int32_t* __restrict__ src, int nsrc,
                                             const BNode* __restrict__ nodes, uint32_t max_steps,
                                             const float4* __restrict__ tris, int swap, const PairTable& table) {
    EdgeWalk w;
    int32_t last = INT_MIN;
    const float tmax0 = r.tmax;
    bool cursor = false;  // (ct, cid): the last crossing of the previous pass
    float ct = 0.0f;
    uint32_t cid = 0;
    while (!w.done) {
        r.tmin = w.thr;
        r.tmax = tmax0;
        float lt[kLongChunk];
        uint32_t lid[kLongChunk];
        int32_t lobj[kLongChunk];
        int n = 0;
        const bool ok = traverse<-1, kStack, true>(nodes, max_steps, r, [&](int first, int cnt) {
            for (int k = first; k < first + cnt; ++k) {
                float a[3], b[3], c[3];
                uint32_t tid;
                int32_t obj;
                load_tri(tris, k, a, b, c, tid, obj);
                float t;
                if (!hit_triangle<-1>(r, a, b, c, t)) continue;
                if (cursor && !hit_less(ct, cid, t, tid)) continue;  // walked in an earlier pass
                if (n == kLongChunk && !hit_less(t, tid, lt[kLongChunk - 1], lid[kLongChunk - 1])) continue;
                int j = n < kLongChunk ? n++ : kLongChunk - 1;
                while (j > 0 && hit_less(t, tid, lt[j - 1], lid[j - 1])) {
                    lt[j] = lt[j - 1];
                    lid[j] = lid[j - 1];
                    lobj[j] = lobj[j - 1];
                    --j;
                }
                lt[j] = t;
                lid[j] = tid;
                lobj[j] = obj;
                if (n == kLongChunk) r.tmax = lt[kLongChunk - 1];
            }
        });
        if (!ok) {
            atomicOr(table.status, ST_STACK_OVERFLOW);
            break;
        }
        for (int j = 0; j < n && !w.done; ++j) {
            if (!w.take(lt[j], table.max_hits, table.next_float)) continue;
            if (lobj[j] != last) {
                last = lobj[j];
                insert_sources(table, src, nsrc, last, swap);
            }
        }
        if (n < kLongChunk) break;
        cursor = true;
        ct = lt[kLongChunk - 1];
        cid = lid[kLongChunk - 1];
    }
    count_edge(table, w.n);
}

// Edge i of a .pre edge payload (starts/ends float3, offsets/counts into sources).
struct EdgePayload {
    const float* starts;
    const float* ends;
    const int32_t* offsets;
    const int32_t* counts;
    const int32_t* sources;
};

template <int STACK>
__device__ __forceinline__ bool edge_ray_fast(const EdgeColumn& col, const EdgePayload& p, uint64_t i,
                                              const BNode* __restrict__ nodes, uint32_t max_steps,
                                              const float4* __restrict__ tris, int swap, const PairTable& table,
                                              int start = 0) {
    Ray r;
    if (!segment_ray_of(p.starts[3 * i], p.starts[3 * i + 1], p.starts[3 * i + 2], p.ends[3 * i], p.ends[3 * i + 1],
                        p.ends[3 * i + 2], r))
        return true;
    return segment_fast<STACK>(col, r, p.sources + p.offsets[i], p.counts[i], nodes, max_steps, tris, swap, table,
                               start);
}

__device__ __forceinline__ void edge_ray_long(const EdgePayload& p, uint64_t i, const BNode* __restrict__ nodes,
                                              uint32_t max_steps, const float4* __restrict__ tris, int swap,
                                              const PairTable& table) {
    Ray r;
    if (!segment_ray_of(p.starts[3 * i], p.starts[3 * i + 1], p.starts[3 * i + 2], p.ends[3 * i], p.ends[3 * i + 1],
                        p.ends[3 * i + 2], r))
        return;
    segment_long(r, p.sources + p.offsets[i], p.counts[i], nodes, max_steps, tris, swap, table);
}

// Record r = 3 t + e: edge e of triangle t of a source mesh, in the triangle's own
// orientation (v0v1, v1v2, v2v0), with the triangle's object as its one source -- the
// legacy per-triangle overlap (mesh_overlap.cu:126-179), which traces shared edges once
// per triangle.
__device__ __forceinline__ bool triangle_edge_of(const float* __restrict__ V, const uint32_t* __restrict__ I,
                                                 uint64_t r, Ray& ray) {
    const uint64_t t = r / 3;
    const int e = (int)(r % 3);
    const uint64_t a = I[3 * t + e], b = I[3 * t + (e == 2 ? 0 : e + 1)];
    return segment_ray_of(V[3 * a], V[3 * a + 1], V[3 * a + 2], V[3 * b], V[3 * b + 1], V[3 * b + 2], ray);
}

}  // namespace
}  // namespace rs
