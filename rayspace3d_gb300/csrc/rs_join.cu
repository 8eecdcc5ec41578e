// rs_join.cu -- edge-ray overlap and the containment fallback.
//
// Edge rays replace __raygen__mesh_overlap_edges / trace_edge_multi_hits_edges
// (query/src/cuda/mesh_overlap_edges.cu:106-216) and __raygen__mesh_overlap
// (mesh_intersection.cu:16-91,288-334): one thread per unique edge traces the
// segment once (the reference re-traces per hit and, in the intersection variant,
// per source object), takes its crossings with the reference's hit rule and inserts
// (source, target) pairs straight into the pair table.  The edges a broad phase keeps
// are binned by the Morton cell of their midpoint first, so the 32 rays of a warp
// start close together and descend the same subtrees.  Containment replaces
// __raygen__mesh_containment_anyhit + __anyhit__ah_containment
// (mesh_intersection_anyhit.cu:46-240): one +Z ray per
// source object, parity per target object kept in registers instead of a
// 256-slot global scratch per object.
#include <algorithm>
#include <climits>

#include <mutex>

#include "rs_engine.h"
#include "rs_prims.cuh"
#include "rs_query_core.cuh"

namespace rs {
namespace {

constexpr int kT = 128;
constexpr int kTargets = 32;
constexpr int kFastStack = 32;  // shared-memory stack entries per lane of the edge-ray kernels
constexpr int kCellBits = 5;    // 32^3 Morton cells order the live edges
constexpr int kCells = 1 << (3 * kCellBits);
// Jobs with more edges than this are traced in live-list order (no binning): the cell
// ranks and the ordered list would cost 8 more bytes per edge.
constexpr uint64_t kBinMaxEdges = 1ull << 27;
// Fewer live edges than this are traced in live-list order: the scan and the scatter would
// cost more than the coherence saves.
constexpr unsigned int kBinMinLive = 1u << 16;

// Live lists of at most kWarpRayMax edges are traced one warp per edge (k_edge_rays_warp),
// longer ones one thread per edge (k_edge_rays): with few rays the join waits on the
// longest chain of dependent node loads, which a warp shortens to the tree's depth plus
// its node count over 32.
constexpr unsigned int kWarpRayMax = 4096;
constexpr int kWarpRayWarps = 8;   // warps per block
constexpr int kWarpRayStack = 128; // entries of a warp's stack
constexpr int kWarpRayHits = 16;   // crossings a warp keeps; an edge with more is deferred

// Fast path over the edges order[0..*n_order) of a payload of n_direct edges (or over all
// of them when order is null); the edges it defers go to deferred[0..*n_def).
// entry / order_entry (nullable): the node each listed edge's traversal starts from.
__global__ void __launch_bounds__(kT) k_edge_rays(EdgePayload p, const uint32_t* __restrict__ order,
                                                  const uint32_t* __restrict__ live,
                                                  const unsigned int* __restrict__ n_order, uint64_t n_direct,
                                                  const BNode* __restrict__ nodes, uint32_t max_steps,
                                                  const float4* __restrict__ tris, int swap, PairTable table,
                                                  uint32_t* __restrict__ deferred, unsigned int* __restrict__ n_def,
                                                  const uint32_t* __restrict__ order_entry,
                                                  const uint32_t* __restrict__ live_entry) {
    __shared__ EdgeSmem<kT, kFastStack> sm;
    const EdgeColumn col = sm.column(threadIdx.x);
    const uint64_t n = live ? (uint64_t)*n_order : n_direct;
    if (live && n <= kWarpRayMax) return;  // k_edge_rays_warp traces short live lists
    // The cell-ordered list when the job was binned and is long enough, else the live list.
    const uint32_t* entry = nullptr;
    if (live) {
        const bool binned = order && n >= kBinMinLive;
        entry = binned ? order_entry : live_entry;
        order = binned ? order : live;
    }
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = order ? order[j] : (uint32_t)j;
        const int start = entry ? (int)entry[j] : 0;
        if (e >= n_direct) continue;  // never, for a list of this payload's edges
        if (!edge_ray_fast<kFastStack>(col, p, e, nodes, max_steps, tris, swap, table, start))
            deferred[atomicAdd(n_def, 1u)] = e;  // the deferred paths start from the root
    }
}

// Shared-memory columns of one warp's edge: a stack of STACK node entries, and HITS
// crossings twice (as found, then sorted).
template <int STACK, int HITS>
struct WarpEdgeSmem {
    int stack[STACK];
    float t[HITS], t2[HITS];
    uint32_t id[HITS], id2[HITS];
    int32_t obj[HITS], obj2[HITS];
};

// One edge by one warp: the lanes pop up to 32 nodes per step from the warp's
// shared-memory stack, test both children of each, test the triangles of the leaves hit
// and push the inner children hit; crossings go to a shared-memory list.  Visits the nodes
// the one-thread traversal visits (the same slab tests over the same [tmin, tmax]), so it
// finds the same crossings; the lanes rank them by (t, id) (triangle ids are distinct, so
// ranks are too) and lane 0 walks them with the table's hit rule.  Returns false, having
// inserted nothing, when there are more than HITS crossings or the stack or the step
// budget runs out.
template <int STACK, int HITS>
__device__ bool edge_ray_warp(WarpEdgeSmem<STACK, HITS>& w_sm, const EdgePayload& p, uint64_t i,
                              const BNode* __restrict__ nodes, uint32_t max_steps, const float4* __restrict__ tris,
                              int swap, const PairTable& table, int start = 0) {
    int* stack = w_sm.stack;
    float* ht = w_sm.t;
    uint32_t* hid = w_sm.id;
    int32_t* hobj = w_sm.obj;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    Ray r;
    if (!segment_ray_of(p.starts[3 * i], p.starts[3 * i + 1], p.starts[3 * i + 2], p.ends[3 * i], p.ends[3 * i + 1],
                        p.ends[3 * i + 2], r))
        return true;
    if (lane == 0) stack[0] = start;
    __syncwarp();
    int sp = 1, nh = 0;
    uint32_t visits = 0;
    bool ok = true;
    unsigned int tests = 0;
    while (sp > 0) {
        const int take = min(sp, 32);
        const int node = lane < take ? stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        visits += (uint32_t)take;
        if (visits > max_steps) {
            ok = false;
            break;
        }
        bool h[2] = {false, false};
        int first[2] = {0, 0}, cnt[2] = {0, 0};
        if (node >= 0) {
            const float4 na = __ldg(&nodes[node].a), nb = __ldg(&nodes[node].b), nc = __ldg(&nodes[node].c);
            const int4 nd = __ldg(&nodes[node].d);
            const float lo0[3] = {na.x, na.y, na.z}, hi0[3] = {na.w, nb.x, nb.y};
            const float lo1[3] = {nb.z, nb.w, nc.x}, hi1[3] = {nc.y, nc.z, nc.w};
            float e, x;
            h[0] = slab<-1>(r, lo0, hi0, r.tmin, r.tmax, e, x);
            h[1] = slab<-1>(r, lo1, hi1, r.tmin, r.tmax, e, x);
            first[0] = nd.x;
            cnt[0] = nd.y;
            first[1] = nd.z;
            cnt[1] = nd.w;
        }
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int mine = (h[side] && cnt[side] > 0) ? cnt[side] : 0;
            tests += (unsigned int)mine;
            const int rounds = __reduce_max_sync(0xffffffffu, mine);
            for (int k = 0; k < rounds; ++k) {
                bool hit = false;
                float t = 0.0f;
                uint32_t tid = 0;
                int32_t obj = 0;
                if (k < mine) {
                    float a[3], b[3], c[3];
                    load_tri(tris, first[side] + k, a, b, c, tid, obj);
                    hit = hit_triangle<-1>(r, a, b, c, t);
                }
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int pos = nh + __popc(m & lt);
                    if (pos < HITS) {
                        ht[pos] = t;
                        hid[pos] = tid;
                        hobj[pos] = obj;
                    }
                }
                nh += __popc(m);
            }
        }
        const bool p0 = h[0] && cnt[0] == 0, p1 = h[1] && cnt[1] == 0;
        const unsigned b0 = __ballot_sync(0xffffffffu, p0), b1 = __ballot_sync(0xffffffffu, p1);
        const int total = __popc(b0) + __popc(b1);
        if (sp + total > STACK) {
            ok = false;
            break;
        }
        int pos = sp + __popc(b0 & lt) + __popc(b1 & lt);
        if (p0) stack[pos++] = first[0];
        if (p1) stack[pos] = first[1];
        __syncwarp();
        sp += total;
    }
    add_tests(tests);
    __syncwarp();
    if (!ok || nh > HITS) return false;
    for (int a = lane; a < nh; a += 32) {
        const float t = ht[a];
        const uint32_t id = hid[a];
        int rank = 0;
        for (int b = 0; b < nh; ++b) rank += hit_less(ht[b], hid[b], t, id) ? 1 : 0;
        w_sm.t2[rank] = t;
        w_sm.id2[rank] = id;
        w_sm.obj2[rank] = hobj[a];
    }
    __syncwarp();
    if (lane == 0) {
        EdgeWalk w;
        int32_t last = INT_MIN;
        const int32_t* src = p.sources + p.offsets[i];
        const int nsrc = p.counts[i];
        for (int a = 0; a < nh && !w.done; ++a) {
            if (!w.take(w_sm.t2[a], table.max_hits, table.next_float)) continue;
            if (w_sm.obj2[a] == last) continue;
            last = w_sm.obj2[a];
            insert_sources(table, src, nsrc, last, swap);
        }
        count_edge(table, w.n);
    }
    __syncwarp();
    return true;
}

__global__ void __launch_bounds__(32 * kWarpRayWarps) k_edge_rays_warp(
    EdgePayload p, const uint32_t* __restrict__ live, const unsigned int* __restrict__ n_live, uint64_t n_direct,
    const BNode* __restrict__ nodes, uint32_t max_steps, const float4* __restrict__ tris, int swap, PairTable table,
    uint32_t* __restrict__ deferred, unsigned int* __restrict__ n_def, const uint32_t* __restrict__ live_entry) {
    __shared__ WarpEdgeSmem<kWarpRayStack, kWarpRayHits> sm[kWarpRayWarps];
    const unsigned int n = *n_live;
    if (n > kWarpRayMax) return;  // the one-thread kernel traces this list
    const int wi = threadIdx.x >> 5;
    const unsigned int nw = gridDim.x * kWarpRayWarps;
    for (unsigned int j = blockIdx.x * kWarpRayWarps + wi; j < n; j += nw) {  // warp-uniform
        const uint32_t e = live[j];
        const int start = live_entry ? (int)live_entry[j] : 0;
        if (e >= n_direct) continue;
        if (!edge_ray_warp<kWarpRayStack, kWarpRayHits>(sm[wi], p, e, nodes, max_steps, tris, swap, table, start) &&
            (threadIdx.x & 31) == 0)
            deferred[atomicAdd(n_def, 1u)] = e;
    }
}

// Long path over the deferred edges, one warp per edge: the warp collects every crossing
// of the edge in one traversal (up to kLongWarpHits; the reference's walk takes at most
// --overlap-max-iterations of them) instead of one thread re-traversing per chunk of 16;
// an edge with more crossings, or a wider traversal than the warp's stack, runs the
// one-thread chunked loop (segment_long) in lane 0.
constexpr int kLongWarps = 4;
constexpr int kLongWarpStack = 256;
constexpr int kLongWarpHits = 256;

__global__ void __launch_bounds__(32 * kLongWarps) k_edge_long_warp(EdgePayload p, const uint32_t* __restrict__ deferred,
                                                                    const unsigned int* __restrict__ n_def,
                                                                    const BNode* __restrict__ nodes, uint32_t max_steps,
                                                                    const float4* __restrict__ tris, int swap,
                                                                    PairTable table) {
    __shared__ WarpEdgeSmem<kLongWarpStack, kLongWarpHits> sm[kLongWarps];
    const unsigned int n = *n_def;
    const int wi = threadIdx.x >> 5;
    const unsigned int nw = gridDim.x * kLongWarps;
    for (unsigned int j = blockIdx.x * kLongWarps + wi; j < n; j += nw) {  // warp-uniform
        const uint32_t e = deferred[j];
        if (!edge_ray_warp<kLongWarpStack, kLongWarpHits>(sm[wi], p, e, nodes, max_steps, tris, swap, table) &&
            (threadIdx.x & 31) == 0)
            edge_ray_long(p, e, nodes, max_steps, tris, swap, table);
        __syncwarp();
    }
}


// Legacy per-triangle overlap (mesh_overlap.cu:126-179): record r = 3 t + e is edge e of
// source triangle t.  Triangles with an index >= nV set *bad and are skipped.  Records the
// fast path defers go to deferred (when given; else they run the long path here).
__global__ void __launch_bounds__(kT) k_tri_edge_join(const float* __restrict__ V, uint64_t nV,
                                                      const uint32_t* __restrict__ I,
                                                      const int32_t* __restrict__ T, uint64_t m,
                                                      const BNode* __restrict__ nodes, uint32_t max_steps,
                                                      const float4* __restrict__ tris, int swap, PairTable table,
                                                      unsigned int* __restrict__ bad, uint32_t* __restrict__ deferred,
                                                      unsigned int* __restrict__ n_def) {
    __shared__ EdgeSmem<kT, kFastStack> sm;
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (r >= m) return;
    const uint64_t t = r / 3;
    if (I[3 * t] >= nV || I[3 * t + 1] >= nV || I[3 * t + 2] >= nV) {
        if (r % 3 == 0) atomicOr(bad, 1u);
        return;
    }
    Ray ray;
    if (!triangle_edge_of(V, I, r, ray)) return;
    if (deferred) {
        if (!segment_fast<kFastStack>(sm.column(threadIdx.x), ray, T + t, 1, nodes, max_steps, tris, swap, table))
            deferred[atomicAdd(n_def, 1u)] = (uint32_t)r;
    } else {
        segment_long(ray, T + t, 1, nodes, max_steps, tris, swap, table);
    }
}

__global__ void __launch_bounds__(kT) k_tri_edge_long(const float* __restrict__ V, const uint32_t* __restrict__ I,
                                                      const int32_t* __restrict__ T,
                                                      const uint32_t* __restrict__ deferred,
                                                      const unsigned int* __restrict__ n_def,
                                                      const BNode* __restrict__ nodes, uint32_t max_steps,
                                                      const float4* __restrict__ tris, int swap, PairTable table) {
    const unsigned int n = *n_def;
    for (unsigned int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint64_t r = deferred[j];
        Ray ray;
        if (triangle_edge_of(V, I, r, ray)) segment_long(ray, T + r / 3, 1, nodes, max_steps, tris, swap, table);
    }
}

// Broad-phase widening (the broad phase below says why it covers every hit).
constexpr float kCullAbs = 1e-4f;
constexpr float kCullRel = 4e-6f;

__device__ __forceinline__ float cull_margin(float l, float h) {
    return kCullRel * (fmaxf(fabsf(l), fabsf(h)) + (h - l));
}

__device__ __forceinline__ int f2ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// The box of edge i's segment widened like a broad-phase query box: kCullAbs plus the
// relative margin of the box, per axis.
__device__ __forceinline__ void edge_query_box(const EdgePayload& p, uint64_t i, float* qlo, float* qhi) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = p.starts[3 * i + k], b = p.ends[3 * i + k];
        const float l = fminf(a, b), h = fmaxf(a, b);
        const float m = kCullAbs + cull_margin(l, h);
        qlo[k] = l - m;
        qhi[k] = h + m;
    }
}

// An object box (ordered ints, min xyz then max xyz) widened by its margin overlaps the
// (already widened) query box.
__device__ __forceinline__ bool box_overlaps(const int* __restrict__ ob, const float* qlo, const float* qhi) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float l = ord2f(__ldg(&ob[k])), h = ord2f(__ldg(&ob[3 + k]));
        const float m = cull_margin(l, h);
        ok = ok && (l - m <= qhi[k]) && (h + m >= qlo[k]);
    }
    return ok;
}

// The edges of one source set traced against the other set's BVH, with the source
// objects' broad-phase flags and the job's work lists.
struct EdgeJob {
    EdgePayload p;
    uint64_t nE;
    const uint8_t* cull;  // flag (or partner count) per source object below n_cull
    uint64_t n_cull;
    const int32_t* part;  // partner lists (nullable), as EdgeCull
    const int* pbox;      // the target set's object boxes
    uint64_t n_pbox;
    uint32_t* live;       // live edges, in arrival order
    uint32_t* rank;       // rank of each live edge within its cell; then the deferred edges
    uint32_t* order;      // live edges by cell (binned jobs)
    uint32_t* cells;      // kCells counts, then their exclusive prefix sums (binned jobs)
    // Entry nodes (nullable, as EdgeCull): per source object, then per edge of live and of
    // order -- the node an edge's traversal starts from.
    const uint32_t* entry;
    uint32_t* live_entry;
    uint32_t* order_entry;
    // Slab index (nullable, as EdgeCull): the payload's slab keys, the source objects' own
    // boxes, and one flag per slab (zeroed) for the slabs that may hold a live edge.
    const long long* xindex;
    const int* sbox;
    uint8_t* covered;
    uint64_t n_slab;
    unsigned int* n_live;
    unsigned int* n_def;
    const BNode* nodes;
    uint32_t max_steps;
    const float4* tris;
    int swap;
};

__device__ __forceinline__ uint32_t spread5(uint32_t v) {  // 5 bits -> every third bit
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton cell (32^3 over the target BVH's root box) of edge i's midpoint.  Written with
// rounded intrinsics so every kernel that calls it computes the same cell.
__device__ __forceinline__ uint32_t edge_cell(const EdgeJob& j, uint64_t i) {
    const float4 na = __ldg(&j.nodes[0].a), nb = __ldg(&j.nodes[0].b), nc = __ldg(&j.nodes[0].c);
    const float lo[3] = {fminf(na.x, nb.z), fminf(na.y, nb.w), fminf(na.z, nc.x)};
    const float hi[3] = {fmaxf(na.w, nc.y), fmaxf(nb.x, nc.z), fmaxf(nb.y, nc.w)};
    uint32_t code = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float m = __fmul_rn(__fadd_rn(j.p.starts[3 * i + k], j.p.ends[3 * i + k]), 0.5f);
        const float ext = __fsub_rn(hi[k], lo[k]);
        float q = ext > 0.0f ? __fmul_rn(__fdiv_rn(__fsub_rn(m, lo[k]), ext), (float)(1 << kCellBits)) : 0.0f;
        q = fminf(fmaxf(q, 0.0f), (float)((1 << kCellBits) - 1));
        code |= spread5((uint32_t)q) << k;
    }
    return code;
}

// Whether edge i of job j is live, given its source count ns, its source list sp, and its
// first source so0 with that object's flag c0 (loaded by the caller).
__device__ __forceinline__ bool edge_is_live(const EdgeJob& j, uint64_t i, int ns, const int32_t* sp, int32_t so0,
                                             uint8_t c0) {
    float qlo[3], qhi[3];
    bool have_box = false;
    for (int q = 0; q < ns; ++q) {
        const int32_t so = q == 0 ? so0 : sp[q];
        if (so < 0 || (uint64_t)so >= j.n_cull) return true;
        const uint8_t c = q == 0 ? c0 : j.cull[so];
        if (c == 0) continue;
        if (!j.part || c == kCandAll) return true;
        // The edge is live when its own widened box reaches a partner's widened box.
        if (!have_box) {
            edge_query_box(j.p, i, qlo, qhi);
            have_box = true;
        }
        const int32_t* pl = j.part + (uint64_t)so * kPartners;
        for (int k = 0; k < (int)c; ++k) {
            const int32_t b = pl[k];
            if (b < 0 || (uint64_t)b >= j.n_pbox || box_overlaps(j.pbox + 6 * (uint64_t)b, qlo, qhi)) return true;
        }
    }
    return false;
}

// Broad phase: the edges with at least one candidate source object (k_cull_flag /
// k_cull_query) are appended to their job's `live` list; in binned jobs each also takes a
// rank within its cell (one warp-aggregated atomic per cell and warp).  Each thread takes
// kLiveEdges edges (a block's edges are contiguous, kLiveEdges rounds of blockDim) and
// issues the dependent loads of all of them together -- count and offset, first source,
// its flag -- so that a wave of threads keeps several chains in flight.  Blocks below
// blocks0 run job j0, the others j1.
constexpr int kLiveEdges = 4;

// Appends edge i to its job's live list when `any` (warp-collective: every lane calls it):
// one atomic per warp, the entry node beside it, and in binned jobs the edge's rank within
// its cell.
__device__ __forceinline__ void live_append(const EdgeJob& j, uint64_t i, bool any, uint32_t en, int lane) {
    const unsigned int below = (1u << lane) - 1u;
    const unsigned int m = __ballot_sync(0xffffffffu, any);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    unsigned int pos0 = 0;
    if (lane == leader) pos0 = atomicAdd(j.n_live, (unsigned int)__popc(m));
    pos0 = __shfl_sync(0xffffffffu, pos0, leader);
    const unsigned int pos = pos0 + __popc(m & below);
    if (any) j.live[pos] = (uint32_t)i;
    if (any && j.live_entry) j.live_entry[pos] = en;
    if (j.order) {
        // Every lane takes part in the match (lanes without a live edge with a cell of
        // their own, kCells + lane), so that the mask is the full warp.
        const uint32_t cell = any ? edge_cell(j, i) : (uint32_t)kCells + lane;
        const unsigned int peers = __match_any_sync(0xffffffffu, cell);
        const int first = __ffs(peers) - 1;
        unsigned int r0 = 0;
        if (any && lane == first) r0 = atomicAdd(&j.cells[cell], (unsigned int)__popc(peers));
        r0 = __shfl_sync(0xffffffffu, r0, first);
        if (any) j.rank[pos] = r0 + __popc(peers & below);
    }
}

__global__ void __launch_bounds__(256) k_edge_live(EdgeJob j0, EdgeJob j1, unsigned int blocks0) {
    const bool second = blockIdx.x >= blocks0;
    const EdgeJob& j = second ? j1 : j0;
    const uint64_t base = (uint64_t)(blockIdx.x - (second ? blocks0 : 0u)) * blockDim.x * kLiveEdges + threadIdx.x;
    int ns[kLiveEdges], off[kLiveEdges];
    int32_t so0[kLiveEdges];
    uint8_t c0[kLiveEdges];
    uint32_t en[kLiveEdges];
#pragma unroll
    for (int u = 0; u < kLiveEdges; ++u) {
        const uint64_t i = base + (uint64_t)u * blockDim.x;
        const bool valid = i < j.nE;
        ns[u] = valid ? j.p.counts[i] : 0;
        off[u] = valid ? j.p.offsets[i] : 0;
    }
#pragma unroll
    for (int u = 0; u < kLiveEdges; ++u) so0[u] = ns[u] > 0 ? j.p.sources[off[u]] : -1;
#pragma unroll
    for (int u = 0; u < kLiveEdges; ++u) {
        const bool in = ns[u] > 0 && so0[u] >= 0 && (uint64_t)so0[u] < j.n_cull;
        c0[u] = in ? j.cull[so0[u]] : (uint8_t)0;
        // One source: its entry node (its partner query ran when its flag is set); more
        // sources: the root.
        en[u] = (j.entry && in && ns[u] == 1) ? j.entry[so0[u]] : 0u;
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int u = 0; u < kLiveEdges; ++u) {
        const uint64_t i = base + (uint64_t)u * blockDim.x;
        const bool any = ns[u] > 0 && edge_is_live(j, i, ns[u], j.p.sources + off[u], so0[u], c0[u]);
        live_append(j, i, any, en[u], lane);
    }
}

// Slab index of an edge payload (rs_edge_index).  The reference's payload is in std::map
// order of its edges' quantised endpoint pairs, lower endpoint first
// (EdgePreprocessor.cpp:41-119: llround(x * 1e5) per coordinate), so it is sorted by the
// quantised x of each edge's lower endpoint -- the smaller of its two quantised x.  Slab b
// holds edges [b * kSlab, (b + 1) * kSlab); index[3 + b] is the key of its first edge.
// index[0] = 1 when the keys never decrease and no source id is negative (else 0),
// index[1] = the largest source id, index[2] = the edge count it was built for.  The
// live-edge check then visits only the slabs whose key range meets the quantised x range
// of an object with a partner: every edge of an object lies between its box's quantised x
// bounds (llround is monotone), and every live edge has such a source.
constexpr uint64_t kSlab = 256;

__device__ __forceinline__ long long edge_key_x(const EdgePayload& p, uint64_t e) {
    return min(llround((double)p.starts[3 * e] * 1e5), llround((double)p.ends[3 * e] * 1e5));
}

// word[0]: 1 once a key decreases or a source id is negative; word[1]: the largest source id.
__global__ void __launch_bounds__(256) k_edge_index(EdgePayload p, uint64_t nE, uint64_t nS,
                                                    long long* __restrict__ index, int* __restrict__ word) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nE; e += stride) {
        const long long x = edge_key_x(p, e);
        if (e % kSlab == 0) index[3 + e / kSlab] = x;
        if (e + 1 < nE && edge_key_x(p, e + 1) < x) bad = true;
    }
    int mx = -1;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nS; k += stride) {
        const int src = p.sources[k];
        bad |= src < 0;
        mx = max(mx, src);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&word[0], 1);
    if ((threadIdx.x & 31) == 0) atomicMax(&word[1], mx);
}

__global__ void k_edge_index_head(long long* __restrict__ index, const int* __restrict__ word, uint64_t nE) {
    index[0] = word[0] ? 0 : 1;
    index[1] = word[1];
    index[2] = (long long)nE;
}

// Slabs of each job that may hold a live edge, one warp per source object: an object with
// a partner (flag set) covers the slabs whose keys can fall in its box's quantised x range.
// A payload whose index says it is not in key order, was built for another edge count, or
// whose source ids reach past the flags, covers every slab (each edge is then checked, as
// without an index).  Blocks below blocks0 run job j0, the others j1.
constexpr int kMarkWarps = 8;

__global__ void __launch_bounds__(32 * kMarkWarps) k_slab_mark(EdgeJob j0, EdgeJob j1, unsigned int blocks0) {
    const bool second = blockIdx.x >= blocks0;
    const EdgeJob& j = second ? j1 : j0;
    const int lane = threadIdx.x & 31;
    const uint64_t o = (uint64_t)(blockIdx.x - (second ? blocks0 : 0u)) * kMarkWarps + (threadIdx.x >> 5);
    const long long* xq = j.xindex + 3;
    const bool ordered =
        j.xindex[0] == 1 && j.xindex[1] < (long long)j.n_cull && j.xindex[2] == (long long)j.nE;
    if (!ordered) {
        if (o == 0)
            for (uint64_t b = lane; b < j.n_slab; b += 32) j.covered[b] = 1;
        return;
    }
    if (o >= j.n_cull || j.cull[o] == 0) return;
    const float lo = ord2f(j.sbox[6 * o]), hi = ord2f(j.sbox[6 * o + 3]);
    if (!(lo <= hi)) return;  // no triangles, hence no edges
    const long long qlo = llround((double)lo * 1e5), qhi = llround((double)hi * 1e5);
    // first slab whose first key is >= qlo (the one before it may hold keys >= qlo too), and
    // the last slab whose first key is <= qhi.
    uint64_t a = 0, b = j.n_slab;
    while (a < b) {
        const uint64_t m = (a + b) / 2;
        if (xq[m] < qlo) a = m + 1;
        else b = m;
    }
    const uint64_t first = a > 0 ? a - 1 : 0;
    a = 0;
    b = j.n_slab;
    while (a < b) {
        const uint64_t m = (a + b) / 2;
        if (xq[m] <= qhi) a = m + 1;
        else b = m;
    }
    if (a == 0) return;  // every key is above qhi
    for (uint64_t s = first + lane; s < a; s += 32) j.covered[s] = 1;
}

// The live-edge check of k_edge_live over the covered slabs only, one block (kSlab threads)
// per slab.  Blocks below blocks0 run job j0, the others j1.
__global__ void __launch_bounds__(kSlab) k_edge_live_slab(EdgeJob j0, EdgeJob j1, unsigned int blocks0) {
    const bool second = blockIdx.x >= blocks0;
    const EdgeJob& j = second ? j1 : j0;
    const uint64_t sl = blockIdx.x - (second ? blocks0 : 0u);
    if (sl >= j.n_slab || !j.covered[sl]) return;  // block-uniform
    const uint64_t i = sl * kSlab + threadIdx.x;
    const bool valid = i < j.nE;
    const int ns = valid ? j.p.counts[i] : 0;
    const int off = valid ? j.p.offsets[i] : 0;
    const int32_t so0 = ns > 0 ? j.p.sources[off] : -1;
    const bool in = ns > 0 && so0 >= 0 && (uint64_t)so0 < j.n_cull;
    const uint8_t c0 = in ? j.cull[so0] : (uint8_t)0;
    const uint32_t en = (j.entry && in && ns == 1) ? j.entry[so0] : 0u;
    const bool any = ns > 0 && edge_is_live(j, i, ns, j.p.sources + off, so0, c0);
    live_append(j, i, any, en, threadIdx.x & 31);
}

// Exclusive prefix sums of the kCells cell counts of each binned job, in place (one block
// of 1024 threads per job, 32 cells per thread).
__global__ void __launch_bounds__(1024) k_cell_scan(uint32_t* c0, uint32_t* c1, const unsigned int* __restrict__ n0,
                                                   const unsigned int* __restrict__ n1) {
    __shared__ uint32_t warp_sum[32];
    uint32_t* c = blockIdx.x ? c1 : c0;
    if (!c || *(blockIdx.x ? n1 : n0) < kBinMinLive) return;
    constexpr int kPer = kCells / 1024;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t v[kPer];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        v[k] = c[t * kPer + k];
        sum += v[k];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sum[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t x = warp_sum[lane], xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        warp_sum[lane] = xi - x;
    }
    __syncthreads();
    uint32_t run = warp_sum[w] + inc - sum;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        c[t * kPer + k] = run;
        run += v[k];
    }
}

// Live edges of the binned jobs into cell order.  Blocks below blocks0 run j0, the others
// j1, each job's blocks striding over its live list.
__global__ void __launch_bounds__(256) k_edge_order(EdgeJob j0, EdgeJob j1, unsigned int blocks0,
                                                    unsigned int blocks1) {
    const bool second = blockIdx.x >= blocks0;
    const EdgeJob& j = second ? j1 : j0;
    if (!j.order) return;
    const unsigned int nb = second ? blocks1 : blocks0;
    const unsigned int n = *j.n_live;
    if (n < kBinMinLive) return;
    for (unsigned int k = (blockIdx.x - (second ? blocks0 : 0u)) * blockDim.x + threadIdx.x; k < n;
         k += nb * blockDim.x) {
        const uint32_t e = j.live[k];
        const uint32_t pos = j.cells[edge_cell(j, e)] + j.rank[k];
        if (pos < n) {  // always: the cell is recomputed with the same arithmetic
            j.order[pos] = e;
            if (j.order_entry) j.order_entry[pos] = j.live_entry[k];
        }
    }
}

// A stream per device for the second direction's rays, forked from and joined back into
// the join's stream, with its two events, created once.  The caller holds *lock (the
// device's mutex) from recording the fork event until the join's stream waits on the
// joined event, so that host threads never record over each other's events.  False when
// they cannot be had: both directions then run on the join's stream.
bool ray_side_stream(cudaStream_t* st_out, cudaEvent_t* fork, cudaEvent_t* joined, std::unique_lock<std::mutex>* lock) {
    struct Side {
        cudaStream_t st = nullptr;
        cudaEvent_t fork = nullptr, joined = nullptr;
        bool ok = false;
        std::mutex mu;
    };
    static Side side[64];
    static std::mutex create_mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return false;
    Side& x = side[dev];
    std::lock_guard<std::mutex> g(create_mu);
    if (!x.ok) {
        x.ok = cudaStreamCreateWithFlags(&x.st, cudaStreamNonBlocking) == cudaSuccess &&
               cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming) == cudaSuccess &&
               cudaEventCreateWithFlags(&x.joined, cudaEventDisableTiming) == cudaSuccess;
        if (!x.ok) {
            cudaGetLastError();
            return false;
        }
    }
    *st_out = x.st;
    *fork = x.fork;
    *joined = x.joined;
    *lock = std::unique_lock<std::mutex>(x.mu);
    return true;
}

__global__ void k_first_tri_init(int32_t* __restrict__ first, uint64_t nObj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < nObj) first[i] = INT_MAX;
}

__global__ void k_first_tri(const int32_t* __restrict__ t2o, uint64_t nF, int32_t* __restrict__ first, uint64_t nObj) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    const int32_t o = t2o[t];
    if (o >= 0 && (uint64_t)o < nObj) atomicMin(&first[o], (int32_t)t);
}

__global__ void k_max_obj(const int32_t* __restrict__ t2o, uint64_t nF, int* __restrict__ mx) {
    int m = -1;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nF; t += (uint64_t)gridDim.x * blockDim.x)
        m = max(m, t2o[t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

// --- broad phase of the overlap join ---------------------------------------------------
//
// If the slab test of an edge ray passes for a triangle box, each coordinate range of
// the ray's segment [1e-6, len + 1e-6] comes within 1.1e-6 + 7u*L of that box (u =
// 2^-24, L = edge length; the slab, direction and length arithmetic rounds at most
// seven times relative to L).  The segment lies in the box of every source object of
// the edge up to the edge payload's 1e-5 endpoint quantisation (a shared edge carries
// its first object's endpoints).  Boxes are therefore compared widened: the triangle
// box by kCullRel * (largest |coordinate| + extent) per axis, the object box by that
// and kCullAbs; the sum covers 1.2e-5 + 7u*L more than five times over (L <= the
// object box's extent).  An object whose widened box overlaps no widened triangle box
// of the other set cannot be the source of a pair, so its edges are not traced.  Each
// set's flags come from its own objects' queries against the other set's BVH.


__global__ void k_obj_box_init(int* __restrict__ box, uint64_t n_obj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < 6 * n_obj) box[i] = (i % 6) < 3 ? 0x7fffffff : (int)0x80000000;
}

// Object boxes from the leaf-ordered triangles (consecutive leaves mostly share an
// object, so lanes with equal objects reduce first and one lane updates the box).
__global__ void k_obj_boxes(const float4* __restrict__ tris, uint64_t n, int* __restrict__ box, uint64_t n_obj) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 p = __ldg(&tris[3 * k]), q = __ldg(&tris[3 * k + 1]), r = __ldg(&tris[3 * k + 2]);
    const int32_t obj = __float_as_int(q.w);
    int v[6] = {f2ord(fminf(fminf(p.x, q.x), r.x)), f2ord(fminf(fminf(p.y, q.y), r.y)),
                f2ord(fminf(fminf(p.z, q.z), r.z)), f2ord(fmaxf(fmaxf(p.x, q.x), r.x)),
                f2ord(fmaxf(fmaxf(p.y, q.y), r.y)), f2ord(fmaxf(fmaxf(p.z, q.z), r.z))};
    const unsigned int peers = __match_any_sync(__activemask(), obj);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = __reduce_min_sync(peers, v[c]);
        v[3 + c] = __reduce_max_sync(peers, v[3 + c]);
    }
    if ((int)(threadIdx.x & 31) != __ffs(peers) - 1) return;
    if (obj < 0 || (uint64_t)obj >= n_obj) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        atomicMin(&box[6 * (uint64_t)obj + c], v[c]);
        atomicMax(&box[6 * (uint64_t)obj + 3 + c], v[3 + c]);
    }
}

// [l, h] widened by its margin overlaps the (already widened) query box.
__device__ __forceinline__ bool cull_overlap(float l0, float l1, float l2, float h0, float h1, float h2,
                                             const float* qlo, const float* qhi) {
    const float m0 = cull_margin(l0, h0), m1 = cull_margin(l1, h1), m2 = cull_margin(l2, h2);
    return l0 - m0 <= qhi[0] && h0 + m0 >= qlo[0] && l1 - m1 <= qhi[1] && h1 + m1 >= qlo[1] &&
           l2 - m2 <= qhi[2] && h2 + m2 >= qlo[2];
}

// The objects of one set (their boxes) queried against the other set's BVH.
struct CullJob {
    const int* box;  // ordered-int min xyz, max xyz per object
    uint64_t n_obj;
    const BNode* nodes;
    uint32_t max_steps;
    const float4* tris;
    uint8_t* cand;
    int32_t* part;    // nullable: partner lists (kPartners per object)
    uint32_t* entry;  // nullable (partner mode): entry node per object queried
};

// Flag pass, one thread per object of one set: does its widened box overlap any widened
// triangle box of the other set's BVH?  cand[o] = 1 on the first overlap, or when the query
// runs out of its node budget or stack; 0 otherwise.  Node boxes contain their triangles'
// boxes and the widening grows with the box, so node culling is conservative.  Most
// objects of a sparse join overlap nothing, and a lone thread answers that in one descent.
// Blocks below blocks0 run job j0, the others j1 (both directions of a join in one launch).
constexpr uint32_t kFlagBudget = 256;  // node visits of a flag query

__global__ void __launch_bounds__(kT) k_cull_flag(CullJob j0, CullJob j1, unsigned int blocks0) {
    const bool second = blockIdx.x >= blocks0;
    const CullJob j = second ? j1 : j0;
    const uint64_t a = (uint64_t)(blockIdx.x - (second ? blocks0 : 0u)) * blockDim.x + threadIdx.x;
    if (a >= j.n_obj) return;
    const BNode* __restrict__ nodes = j.nodes;
    const float4* __restrict__ tris = j.tris;
    float qlo[3], qhi[3];
    bool empty = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float l = ord2f(j.box[6 * a + c]), h = ord2f(j.box[6 * a + 3 + c]);
        empty |= !(l <= h);
        const float m = kCullAbs + cull_margin(l, h);
        qlo[c] = l - m;
        qhi[c] = h + m;
    }
    if (empty) {  // no triangle of this object, hence no edges
        j.cand[a] = 0;
        return;
    }
    int stack[kStack];
    int sp = 0, node = 0;
    uint8_t result = 0;
    const uint32_t budget = min(j.max_steps, kFlagBudget);
    for (uint32_t step = 0;; ++step) {
        if (step > budget) {
            result = 1;
            break;
        }
        const float4 na = __ldg(&nodes[node].a), nb = __ldg(&nodes[node].b), nc = __ldg(&nodes[node].c);
        const int4 nd = __ldg(&nodes[node].d);
        bool h0 = cull_overlap(na.x, na.y, na.z, na.w, nb.x, nb.y, qlo, qhi);
        bool h1 = cull_overlap(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, qlo, qhi);
#pragma unroll 1
        for (int side = 0; side < 2 && !result; ++side) {
            const bool h = side == 0 ? h0 : h1;
            const int first = side == 0 ? nd.x : nd.z, cnt = side == 0 ? nd.y : nd.w;
            if (!h || cnt == 0) continue;
            for (int k = first; k < first + cnt; ++k) {
                const float4 p = __ldg(&tris[3 * (size_t)k]), q = __ldg(&tris[3 * (size_t)k + 1]),
                             r = __ldg(&tris[3 * (size_t)k + 2]);
                if (cull_overlap(fminf(fminf(p.x, q.x), r.x), fminf(fminf(p.y, q.y), r.y),
                                 fminf(fminf(p.z, q.z), r.z), fmaxf(fmaxf(p.x, q.x), r.x),
                                 fmaxf(fmaxf(p.y, q.y), r.y), fmaxf(fmaxf(p.z, q.z), r.z), qlo, qhi)) {
                    result = 1;
                    break;
                }
            }
        }
        if (result) break;
        if (nd.y > 0) h0 = false;
        if (nd.w > 0) h1 = false;
        if (h0 && h1) {
            if (sp == kStack) {
                result = 1;
                break;
            }
            stack[sp++] = nd.z;
            node = nd.x;
        } else if (h0) {
            node = nd.x;
        } else if (h1) {
            node = nd.z;
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    j.cand[a] = result;
}

// Partner pass, one warp per object that the flag pass marked (the others keep cand 0):
// the distinct objects of the other set's triangles whose widened boxes overlap the
// object's widened box go to part[o * kPartners ...] and cand[o] = their number, or
// kCandAll when there are more than kPartners or the query ran out of its budget or stack.
//
// The 32 lanes walk the tree together: each step pops up to 32 nodes from the warp's
// shared-memory stack (one per lane), tests both children of each, tests the triangles of
// the leaves hit, and pushes the inner children hit (ballot prefix sums give the slots).
// Partners found in a step are deduplicated across lanes with ballots and appended to a
// list every lane holds.  A query's latency is therefore its depth plus its node count
// over 32, not its node count.  Blocks below blocks0 run job j0, the others j1 (both
// directions of a join in one launch).
//
// The query also records the object's entry node: the deepest node of the walk's opening
// chain, where each step holds one node, hits no leaf and hits one inner child.  Every
// triangle whose widened box overlaps the object's widened box lies under it, so the rays
// of the object's edges (whose boxes lie inside that box) may start there instead of at
// the root and still meet every triangle they can hit.
constexpr int kCullWarps = 4;             // warps (objects) per block
constexpr int kCullStack = 256;           // entries of a warp's stack
constexpr uint32_t kPartnerBudget = 8192;  // node visits of a partner query

__global__ void __launch_bounds__(32 * kCullWarps) k_cull_query(CullJob j0, CullJob j1, unsigned int blocks0) {
    __shared__ int s_stack[kCullWarps][kCullStack];
    const bool second = blockIdx.x >= blocks0;
    const CullJob j = second ? j1 : j0;
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const uint64_t a = (uint64_t)(blockIdx.x - (second ? blocks0 : 0u)) * kCullWarps + wi;
    if (a >= j.n_obj || j.cand[a] == 0) return;  // warp-uniform
    int* stack = s_stack[wi];
    const BNode* __restrict__ nodes = j.nodes;
    const float4* __restrict__ tris = j.tris;
    float qlo[3], qhi[3];
    bool empty = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float l = ord2f(j.box[6 * a + c]), h = ord2f(j.box[6 * a + 3 + c]);
        empty |= !(l <= h);
        const float m = kCullAbs + cull_margin(l, h);
        qlo[c] = l - m;
        qhi[c] = h + m;
    }
    if (empty) {  // never: the flag pass gave such an object cand 0
        if (lane == 0) j.cand[a] = 0;
        return;
    }
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t budget = min(j.max_steps, kPartnerBudget);
    int32_t pl[kPartners];  // the partner list, the same in every lane
    int np = 0;
    bool all = false;  // flag 1 (flag mode) or kCandAll (partner mode)
    if (lane == 0) stack[0] = 0;
    __syncwarp();
    int sp = 1;
    uint32_t visits = 0;
    int entry = 0;      // under it: every triangle the query can find
    bool chain = true;  // every step so far held one node, hit no leaf and one inner child
    while (sp > 0 && !all) {
        const int take = min(sp, 32);
        const int node = lane < take ? stack[sp - take + lane] : -1;
        if (chain) {
            if (take == 1) entry = __shfl_sync(0xffffffffu, node, 0);
            else chain = false;
        }
        __syncwarp();
        sp -= take;
        visits += (uint32_t)take;
        if (visits > budget) {
            all = true;
            break;
        }
        bool h[2] = {false, false};
        int first[2] = {0, 0}, cnt[2] = {0, 0};
        if (node >= 0) {
            const float4 na = __ldg(&nodes[node].a), nb = __ldg(&nodes[node].b), nc = __ldg(&nodes[node].c);
            const int4 nd = __ldg(&nodes[node].d);
            h[0] = cull_overlap(na.x, na.y, na.z, na.w, nb.x, nb.y, qlo, qhi);
            h[1] = cull_overlap(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, qlo, qhi);
            first[0] = nd.x;
            cnt[0] = nd.y;
            first[1] = nd.z;
            cnt[1] = nd.w;
        }
        if (chain && __any_sync(0xffffffffu, (h[0] && cnt[0] > 0) || (h[1] && cnt[1] > 0))) chain = false;
        // Leaves hit: their triangles, one per lane and round, in warp-uniform rounds.
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int mine = (h[side] && cnt[side] > 0) ? cnt[side] : 0;
            const int rounds = __reduce_max_sync(0xffffffffu, mine);
            for (int k = 0; k < rounds && !all; ++k) {
                bool found = false;
                int32_t pobj = 0;
                if (k < mine) {
                    const int t = first[side] + k;
                    const float4 q = __ldg(&tris[3 * (size_t)t + 1]);
                    pobj = __float_as_int(q.w);
                    bool known = false;
#pragma unroll
                    for (int u = 0; u < kPartners; ++u) known |= (u < np && pl[u] == pobj);
                    if (!known) {
                        const float4 p = __ldg(&tris[3 * (size_t)t]), r = __ldg(&tris[3 * (size_t)t + 2]);
                        found = cull_overlap(fminf(fminf(p.x, q.x), r.x), fminf(fminf(p.y, q.y), r.y),
                                             fminf(fminf(p.z, q.z), r.z), fmaxf(fmaxf(p.x, q.x), r.x),
                                             fmaxf(fmaxf(p.y, q.y), r.y), fmaxf(fmaxf(p.z, q.z), r.z), qlo, qhi);
                    }
                }
                unsigned m = __ballot_sync(0xffffffffu, found);
                while (m && !all) {
                    const int32_t o = __shfl_sync(0xffffffffu, pobj, __ffs(m) - 1);
                    if (np == kPartners) {
                        all = true;
                        break;
                    }
#pragma unroll
                    for (int u = 0; u < kPartners; ++u)
                        if (u == np) pl[u] = o;
                    ++np;
                    m &= ~__ballot_sync(0xffffffffu, found && pobj == o);
                }
            }
        }
        if (all) break;
        // Inner children hit go on the stack.
        const bool p0 = h[0] && cnt[0] == 0, p1 = h[1] && cnt[1] == 0;
        const unsigned b0 = __ballot_sync(0xffffffffu, p0), b1 = __ballot_sync(0xffffffffu, p1);
        const int total = __popc(b0) + __popc(b1);
        if (sp + total > kCullStack) {
            all = true;
            break;
        }
        int pos = sp + __popc(b0 & lt) + __popc(b1 & lt);
        if (p0) stack[pos++] = first[0];
        if (p1) stack[pos] = first[1];
        __syncwarp();
        sp += total;
    }
    if (lane != 0) return;
    if (j.entry) j.entry[a] = (uint32_t)entry;
    j.cand[a] = all ? kCandAll : (uint8_t)np;
    if (!all) {
#pragma unroll
        for (int u = 0; u < kPartners; ++u)
            if (u < np) j.part[a * kPartners + u] = pl[u];
    }
}

// Optional per-source outputs of the containment pass (the reference's pair-hit and
// containment-tracking buffers, query/src/utilities/PairHitTracking.h,
// ContainmentTracking.h): distinct targets crossed, and the odd-parity targets with
// their crossing counts (traversal order within each pass).
struct Tracking {
    int max_targets;
    int32_t* target_ids;      // [nObj * max_targets], -1 where unused
    uint32_t* target_hits;    // [nObj * max_targets]
    uint32_t* candidates;     // [nObj]
};

template <bool TRACK>
__global__ void __launch_bounds__(kT) k_containment(const float* __restrict__ V, uint64_t nV,
                                                    const uint32_t* __restrict__ I,
                                                    const int32_t* __restrict__ first, uint64_t nObj,
                                                    const BNode* __restrict__ nodes, uint32_t max_steps,
                                                    const float4* __restrict__ tris, int swap, PairTable table,
                                                    Tracking trk) {
    const uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (o >= nObj) return;
    if (TRACK) {
        trk.candidates[o] = 0;
        for (int q = 0; q < trk.max_targets; ++q) {
            trk.target_ids[o * trk.max_targets + q] = -1;
            trk.target_hits[o * trk.max_targets + q] = 0;
        }
    }
    const int32_t ft = first[o];
    if (ft == INT_MAX) return;
    const uint32_t vi = I[3 * (uint64_t)ft];
    if (vi >= nV) return;
    const Ray r = make_ray(V[3 * (uint64_t)vi], V[3 * (uint64_t)vi + 1], V[3 * (uint64_t)vi + 2], 0.0f, 0.0f, 1.0f,
                           1e-4f, 1e10f);
    // Parity per target object in passes of at most kTargets objects: pass p tracks the
    // kTargets smallest object ids (as uint32) above the largest id of pass p-1.  A list
    // member is inserted at its first crossing and never evicted (evictions only drop the
    // largest member for a smaller newcomer, and the largest only decreases), so every
    // tracked parity is complete; a pass that had to turn an id away runs another pass.
    uint32_t tgt[kTargets];
    uint32_t hits[TRACK ? kTargets : 1];
    uint32_t lo = 0;
    bool bounded = false;
    unsigned int crossings = 0, candidates = 0, tests = 0;
    int out = 0;
    for (;;) {
        uint32_t par = 0;  // parity bit per list entry
        int nt = 0;
        bool more = false;
        const bool ok = traverse<2>(nodes, max_steps, r, [&](int f, int cnt) {
            for (int k = f; k < f + cnt; ++k) {
                float a[3], b[3], c[3];
                uint32_t tid;
                int32_t obj;
                load_tri(tris, k, a, b, c, tid, obj);
                const uint32_t id = (uint32_t)obj;
                if (bounded && id <= lo) continue;
                if (more && nt == kTargets && (bounded || !table.stats)) {  // above every member of a full list
                    uint32_t mx = 0;
                    for (int j = 0; j < nt; ++j) mx = max(mx, tgt[j]);
                    if (id > mx) continue;
                }
                float t;
                ++tests;
                if (!hit_triangle<2>(r, a, b, c, t)) continue;
                if (!bounded) ++crossings;
                int j = 0;
                for (; j < nt; ++j)
                    if (tgt[j] == id) break;
                if (j < nt) {
                    par ^= 1u << j;
                    if (TRACK) ++hits[j];
                } else if (nt < kTargets) {
                    tgt[nt] = id;
                    if (TRACK) hits[nt] = 1;
                    par |= 1u << nt;
                    ++nt;
                } else {
                    more = true;
                    int jm = 0;
                    for (int q = 1; q < nt; ++q)
                        if (tgt[q] > tgt[jm]) jm = q;
                    if (id < tgt[jm]) {
                        tgt[jm] = id;
                        if (TRACK) hits[jm] = 1;
                        par |= 1u << jm;
                    }
                }
            }
        });
        if (!ok) {
            atomicOr(table.status, ST_STACK_OVERFLOW);
            return;
        }
        candidates += (unsigned int)nt;
        uint32_t mx = 0;
        for (int j = 0; j < nt; ++j) {
            mx = max(mx, tgt[j]);
            if (!((par >> j) & 1u)) continue;
            const unsigned long long key = swap ? (((unsigned long long)tgt[j] << 32) | (uint32_t)o)
                                                : (((unsigned long long)(uint32_t)o << 32) | tgt[j]);
            table_insert(table, key);
            if (TRACK && out < trk.max_targets) {
                trk.target_ids[o * trk.max_targets + out] = (int32_t)tgt[j];
                trk.target_hits[o * trk.max_targets + out] = hits[j];
                ++out;
            }
        }
        if (!more) break;
        lo = mx;
        bounded = true;
    }
    add_tests(tests);
    if (table.stats) {
        atomicAdd(&table.stats[4], 1ull);
        if (crossings) atomicAdd(&table.stats[5], (unsigned long long)crossings);
        if (candidates) atomicAdd(&table.stats[6], (unsigned long long)candidates);
    }
    if (TRACK) trk.candidates[o] = candidates;
}

}  // namespace

int recheck_join(int op, unsigned long long* out) { return recheck_op(op, out); }

PairTable table_view(rs_pairset* ps) {
    ps->known_count = -1;  // a launch is about to insert
    PairTable t;
    t.slots = ps->slots;
    t.capacity = ps->capacity;
    t.pow2 = ps->pow2;
    t.max_probes = ps->max_probes;
    t.status = reinterpret_cast<unsigned int*>(ps->meta);
    t.count = ps->meta + 1;
    t.stats = ps->track ? ps->meta + 2 : nullptr;
    t.max_hits = ps->edge_max_hits;
    t.next_float = ps->edge_next_float;
    t.over = ps->over;
    t.over_mask = kOverSlots - 1;
    t.over_count = ps->meta + kOverWord;
    t.spill_at = std::max<unsigned long long>(1, ps->capacity / 4 * 3 + (ps->capacity % 4) * 3 / 4);
    if (ps->over) ps->over_dirty = true;
    return t;
}

}  // namespace rs

using namespace rs;

namespace rs {
// Launches one edge-ray direction without waiting for it (status lands in the table's meta word).
cudaError_t edge_jobs_async(EdgeJob* job, int n_jobs, rs_pairset* ps, cudaStream_t s);

// Every edge of a payload, in payload order (no broad phase), in chunks of 2^31 edges so
// that edge ids fit the 32-bit deferred list (a chunk's payload pointers are offset; the
// offsets still index the whole sources array).
static cudaError_t edge_all_async(const rs_bvh* target, EdgePayload p, uint64_t nE, int swap, rs_pairset* ps,
                                  cudaStream_t s) {
    constexpr uint64_t kChunk = 1ull << 31;
    const uint64_t cap = std::min(nE, kChunk);
    uint32_t* deferred = nullptr;
    unsigned int* n_def = nullptr;
    cudaError_t e = dmalloc((void**)&deferred, std::max<uint64_t>(cap, 1) * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = dmalloc((void**)&n_def, sizeof(unsigned int), s);
    const PairTable table = table_view(ps);
    const int ptok = prof_begin(P_EDGE_JOIN, s);
    for (uint64_t base = 0; base < nE && e == cudaSuccess; base += kChunk) {
        const uint64_t n = std::min(kChunk, nE - base);
        const EdgePayload q{p.starts + 3 * base, p.ends + 3 * base, p.offsets + base, p.counts + base, p.sources};
        e = cudaMemsetAsync(n_def, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) break;
        const unsigned grid = (unsigned)std::min<uint64_t>((n + kT - 1) / kT, 8ull * sm_count());
        launch(k_edge_rays, grid, kT, 0, s, q, (const uint32_t*)nullptr, (const uint32_t*)nullptr,
               (const unsigned int*)nullptr, n,
               (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap, table, deferred,
               n_def, (const uint32_t*)nullptr, (const uint32_t*)nullptr);
        launch(k_edge_long_warp, (unsigned)std::min<uint64_t>((n + kLongWarps - 1) / kLongWarps, 4ull * sm_count()),
               32 * kLongWarps, 0, s, q, (const uint32_t*)deferred, (const unsigned int*)n_def,
               (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap, table);
        e = cudaGetLastError();
    }
    prof_end(P_EDGE_JOIN, s, ptok);
    if (deferred) cudaFreeAsync(deferred, s);
    if (n_def) cudaFreeAsync(n_def, s);
    return e;
}

cudaError_t edge_join_async(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources, uint64_t nE,
                            int swap, rs_pairset* ps, cudaStream_t s, const EdgeCull& cull) {
    if (nE == 0 || target->n_tris == 0) return cudaSuccess;
    const EdgePayload p{d_starts, d_ends, d_offsets, d_counts, d_sources};
    if (!cull.cand || nE > 0xffffffffull) return edge_all_async(target, p, nE, swap, ps, s);
    EdgeJob job{};
    job.p = p;
    job.nE = nE;
    job.cull = cull.cand;
    job.n_cull = cull.n_obj;
    job.part = cull.part;
    job.pbox = cull.pbox;
    job.n_pbox = cull.n_pbox;
    job.entry = cull.part ? cull.entry : nullptr;
    job.xindex = cull.part ? cull.xindex : nullptr;
    job.sbox = cull.sbox;
    job.nodes = (const BNode*)target->nodes;
    job.max_steps = max_steps(target);
    job.tris = (const float4*)target->tris;
    job.swap = swap;
    return edge_jobs_async(&job, 1, ps, s);
}

// Live edges first, then rays for them only: the live checks of all jobs in one launch,
// the binning of their live edges by cell in two more, then each job's rays (the second
// job's on a side stream) and its deferred edges.  Each job's nE < 2^32 and its cull flags
// set.
cudaError_t edge_jobs_async(EdgeJob* job, int n_jobs, rs_pairset* ps, cudaStream_t s) {
    // One zeroed block: n_live[2], n_def[2], the cell counts of the binned jobs, then (slab
    // mode) each job's slab flags.
    uint32_t* zeroed = nullptr;
    EdgeJob jobs[2] = {};
    uint64_t blocks[2] = {0, 0}, total_e = 0;
    int n_bin = 0;
    // Slab mode when every job has a slab index (and partner lists): the live-edge check
    // visits only the slabs of objects with partners.
    bool slab = n_jobs > 0;
    for (int d = 0; d < n_jobs; ++d) {
        jobs[d] = job[d];
        if (jobs[d].nE <= kBinMaxEdges) ++n_bin;
        slab = slab && jobs[d].xindex && jobs[d].sbox && jobs[d].part;
    }
    auto a256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t cbytes = a256((4 + (size_t)n_bin * kCells) * sizeof(uint32_t));
    size_t zbytes = cbytes;
    for (int d = 0; d < n_jobs && slab; ++d) {
        jobs[d].n_slab = (jobs[d].nE + kSlab - 1) / kSlab;
        zbytes += a256(std::max<uint64_t>(jobs[d].n_slab, 1));
    }
    // One allocation: the zeroed block, then each job's live, rank and (binned jobs) order
    // lists, each 256-byte aligned; one memset clears the zeroed block.
    size_t total = a256(zbytes);
    for (int d = 0; d < n_jobs; ++d) {
        const size_t bytes = a256(std::max<uint64_t>(jobs[d].nE, 1) * sizeof(uint32_t));
        const bool bin = jobs[d].nE <= kBinMaxEdges;
        total += ((bin ? 3 : 2) + (jobs[d].entry ? (bin ? 2 : 1) : 0)) * bytes;
    }
    cudaError_t e = dmalloc((void**)&zeroed, total, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(zeroed, 0, zbytes, s);
    uint32_t* next_cells = zeroed + 4;
    char* next_flags = reinterpret_cast<char*>(zeroed) + cbytes;
    char* next = reinterpret_cast<char*>(zeroed) + a256(zbytes);
    for (int d = 0; d < n_jobs && e == cudaSuccess; ++d) {
        EdgeJob& j = jobs[d];
        const size_t bytes = a256(std::max<uint64_t>(j.nE, 1) * sizeof(uint32_t));
        j.n_live = zeroed + d;
        j.n_def = zeroed + 2 + d;
        j.live = reinterpret_cast<uint32_t*>(next);
        j.rank = reinterpret_cast<uint32_t*>(next + bytes);
        next += 2 * bytes;
        if (j.nE <= kBinMaxEdges) {
            j.order = reinterpret_cast<uint32_t*>(next);
            next += bytes;
            j.cells = next_cells;
            next_cells += kCells;
        }
        if (j.entry) {
            j.live_entry = reinterpret_cast<uint32_t*>(next);
            next += bytes;
            if (j.order) {
                j.order_entry = reinterpret_cast<uint32_t*>(next);
                next += bytes;
            }
        }
        if (slab) {
            j.covered = reinterpret_cast<uint8_t*>(next_flags);
            next_flags += a256(std::max<uint64_t>(j.n_slab, 1));
        }
        blocks[d] = (j.nE + 256 * kLiveEdges - 1) / (256 * kLiveEdges);
        total_e += j.nE;
    }
    if (e == cudaSuccess && total_e) {
        const int ptok = prof_begin(P_EDGE_JOIN, s);
        if (slab) {
            uint64_t mb[2] = {0, 0};
            for (int d = 0; d < n_jobs; ++d) mb[d] = std::max<uint64_t>((jobs[d].n_cull + kMarkWarps - 1) / kMarkWarps, 1);
            launch(k_slab_mark, (unsigned)(mb[0] + mb[1]), 32 * kMarkWarps, 0, s, jobs[0], jobs[1], (unsigned)mb[0]);
            launch(k_edge_live_slab, (unsigned)(jobs[0].n_slab + jobs[1].n_slab), (unsigned)kSlab, 0, s, jobs[0],
                   jobs[1], (unsigned)jobs[0].n_slab);
        } else {
            launch(k_edge_live, (unsigned)(blocks[0] + blocks[1]), 256, 0, s, jobs[0], jobs[1], (unsigned)blocks[0]);
        }
        if (n_bin) {
            launch(k_cell_scan, 2, 1024, 0, s, jobs[0].cells, n_jobs > 1 ? jobs[1].cells : (uint32_t*)nullptr,
                   (const unsigned int*)jobs[0].n_live,
                   (const unsigned int*)(n_jobs > 1 ? jobs[1].n_live : jobs[0].n_live));
            const unsigned ob0 = (unsigned)std::min<uint64_t>(std::max<uint64_t>(blocks[0], 1), 4ull * sm_count());
            const unsigned ob1 = (unsigned)std::min<uint64_t>(blocks[1], 4ull * sm_count());
            launch(k_edge_order, ob0 + ob1, 256, 0, s, jobs[0], jobs[1], ob0, ob1);
        }
        // The rays of the second job on a side stream, concurrent with the first's: each
        // list's rays are latency-bound chains when the lists are short, and a full list
        // keeps the GPU busy either way.
        const PairTable table = table_view(ps);
        cudaStream_t side = nullptr;
        cudaEvent_t fork = nullptr, joined = nullptr;
        std::unique_lock<std::mutex> side_lock;
        if (n_jobs == 2 && ray_side_stream(&side, &fork, &joined, &side_lock) &&
            (cudaEventRecord(fork, s) != cudaSuccess || cudaStreamWaitEvent(side, fork, 0) != cudaSuccess)) {
            cudaGetLastError();
            side = nullptr;  // both on s
        }
        for (int d = 0; d < n_jobs; ++d) {
            const EdgeJob& j = jobs[d];
            cudaStream_t st = d == 1 && side ? side : s;
            launch(k_edge_rays_warp,
                   (unsigned)std::min<uint64_t>((std::min<uint64_t>(j.nE, kWarpRayMax) + kWarpRayWarps - 1) /
                                                    kWarpRayWarps, 4ull * sm_count()),
                   32 * kWarpRayWarps, 0, st, j.p, (const uint32_t*)j.live, (const unsigned int*)j.n_live, j.nE,
                   j.nodes, j.max_steps, j.tris, j.swap, table, j.rank, j.n_def, (const uint32_t*)j.live_entry);
            launch(k_edge_rays, (unsigned)std::min<uint64_t>((j.nE + kT - 1) / kT, 8ull * sm_count()), kT, 0, st, j.p,
                   (const uint32_t*)j.order, (const uint32_t*)j.live, (const unsigned int*)j.n_live, j.nE, j.nodes,
                   j.max_steps, j.tris, j.swap, table, j.rank, j.n_def, (const uint32_t*)j.order_entry,
                   (const uint32_t*)j.live_entry);
            launch(k_edge_long_warp,
                   (unsigned)std::min<uint64_t>((j.nE + kLongWarps - 1) / kLongWarps, 4ull * sm_count()),
                   32 * kLongWarps, 0, st, j.p, (const uint32_t*)j.rank, (const unsigned int*)j.n_def, j.nodes,
                   j.max_steps, j.tris, j.swap, table);
        }
        if (side) {
            e = cudaEventRecord(joined, side);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, joined, 0);
            if (e != cudaSuccess) cudaStreamSynchronize(side);  // the lists are freed on s below
        }
        prof_end(P_EDGE_JOIN, s, ptok);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (zeroed) cudaFreeAsync(zeroed, s);
    return e;
}

// Both edge directions of a join with both broad-phase flag sets: A's edges against B's
// BVH (swap 0) and B's edges against A's BVH (swap 1), rays of both in flight together.
cudaError_t edge_join_pair_async(const rs_bvh* A, const float* startsA, const float* endsA, const int32_t* offsetsA,
                                 const int32_t* countsA, const int32_t* sourcesA, uint64_t nEA, const EdgeCull& cullA,
                                 const rs_bvh* B, const float* startsB, const float* endsB, const int32_t* offsetsB,
                                 const int32_t* countsB, const int32_t* sourcesB, uint64_t nEB, const EdgeCull& cullB,
                                 rs_pairset* ps, cudaStream_t s) {
    EdgeJob job[2] = {};
    int n = 0;
    auto add = [&](const rs_bvh* target, EdgePayload p, uint64_t nE, const EdgeCull& c, int swap) {
        EdgeJob& j = job[n++];
        j.p = p;
        j.nE = nE;
        j.cull = c.cand;
        j.n_cull = c.n_obj;
        j.part = c.part;
        j.pbox = c.pbox;
        j.n_pbox = c.n_pbox;
        j.entry = c.part ? c.entry : nullptr;
        j.xindex = c.part ? c.xindex : nullptr;
        j.sbox = c.sbox;
        j.nodes = (const BNode*)target->nodes;
        j.max_steps = max_steps(target);
        j.tris = (const float4*)target->tris;
        j.swap = swap;
    };
    if (nEA && B->n_tris) add(B, EdgePayload{startsA, endsA, offsetsA, countsA, sourcesA}, nEA, cullA, 0);
    if (nEB && A->n_tris) add(A, EdgePayload{startsB, endsB, offsetsB, countsB, sourcesB}, nEB, cullB, 1);
    return n ? edge_jobs_async(job, n, ps, s) : cudaSuccess;
}

// Broad phase of both directions in one launch: set d's objects (A for d = 0, B for d = 1)
// are queried against the other set's BVH when cand[d] is given (either null: that
// direction is skipped), in partner mode when part[d] is given too.  Object boxes come from
// the build (k_morton) when they cover the set, else from its leaf triangles into
// temporaries.  With boxes_out, both sets' boxes are made and returned (the partner filter
// of the edge rays reads them) and the temporaries go to tmps_out, for the caller to free
// after those rays; otherwise they are freed here.
cudaError_t cull_impl(const rs_bvh* A, const rs_bvh* B, uint8_t* candA, uint8_t* candB, int32_t* partA,
                      int32_t* partB, uint32_t* entryA, uint32_t* entryB, const int** boxes_out, int** tmps_out,
                      cudaStream_t s) {
    const rs_bvh* src[2] = {A, B};
    const rs_bvh* other[2] = {B, A};
    uint8_t* cand[2] = {candA, candB};
    int32_t* part[2] = {partA, partB};
    uint32_t* entry[2] = {entryA, entryB};
    int* tmp[2] = {nullptr, nullptr};
    const int* boxes[2] = {nullptr, nullptr};
    CullJob job[2] = {};
    unsigned int blocks[2] = {0, 0};
    cudaError_t e = cudaSuccess;
    for (int d = 0; d < 2 && e == cudaSuccess; ++d) {
        const rs_bvh* h = src[d];
        if ((!cand[d] && !boxes_out) || h->n_obj == 0) continue;
        const int* box = h->obox;
        if (!box || h->n_obj > h->obox_cap) {
            e = dmalloc((void**)&tmp[d], 6 * h->n_obj * sizeof(int), s);
            if (e != cudaSuccess) break;
            launch(k_obj_box_init, (unsigned)((6 * h->n_obj + 255) / 256), 256, 0, s, tmp[d], h->n_obj);
            launch(k_obj_boxes, (unsigned)((h->n_tris + 255) / 256), 256, 0, s, (const float4*)h->tris, h->n_tris,
                   tmp[d], h->n_obj);
            box = tmp[d];
        }
        boxes[d] = box;
    }
    unsigned int wblocks[2] = {0, 0};
    for (int d = 0; d < 2 && e == cudaSuccess; ++d) {
        const rs_bvh* h = src[d];
        if (!cand[d] || h->n_obj == 0) continue;
        job[d] = CullJob{boxes[d], h->n_obj, (const BNode*)other[d]->nodes, max_steps(other[d]),
                         (const float4*)other[d]->tris, cand[d], part[d], part[d] ? entry[d] : nullptr};
        blocks[d] = (unsigned int)((h->n_obj + kT - 1) / kT);
        if (part[d]) wblocks[d] = (unsigned int)((h->n_obj + kCullWarps - 1) / kCullWarps);
    }
    if (e == cudaSuccess && blocks[0] + blocks[1] > 0)
        launch(k_cull_flag, blocks[0] + blocks[1], kT, 0, s, job[0], job[1], blocks[0]);
    // The partner pass of a direction without partner lists has no blocks.
    if (e == cudaSuccess && wblocks[0] + wblocks[1] > 0)
        launch(k_cull_query, wblocks[0] + wblocks[1], 32 * kCullWarps, 0, s, job[0], job[1], wblocks[0]);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (boxes_out && e == cudaSuccess) {
        boxes_out[0] = boxes[0];
        boxes_out[1] = boxes[1];
        tmps_out[0] = tmp[0];
        tmps_out[1] = tmp[1];
    } else {
        for (int* p : tmp)
            if (p) cudaFreeAsync(p, s);
    }
    return e;
}

// Broad-phase flags of A's objects against B's BVH into candA and of B's objects against
// A's BVH into candB (either null: that direction is skipped), both in one launch.
cudaError_t cull_pair_async(const rs_bvh* A, const rs_bvh* B, uint8_t* candA, uint8_t* candB, cudaStream_t s) {
    return cull_impl(A, B, candA, candB, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, s);
}

// Broad-phase flags of `src`'s objects against `other`'s BVH.
cudaError_t cull_async(const rs_bvh* src, const rs_bvh* other, uint8_t* cand, cudaStream_t s) {
    return cull_pair_async(src, other, cand, nullptr, s);
}

// The distinct-key count read with the status is kept for rs_pairset_finalize/info.
int table_status(rs_pairset* ps, cudaStream_t s, cudaError_t e) {
    constexpr uint32_t kHard = ST_TABLE_FULL | ST_STACK_OVERFLOW | ST_ITER_LIMIT | ST_TARGET_OVERFLOW;
    for (int round = 0;; ++round) {
        unsigned long long m[kOverWord + 1] = {};
        if (e == cudaSuccess) e = cudaMemcpyAsync(m, ps->meta, sizeof(m), cudaMemcpyDeviceToHost, s);
        cudaError_t e2 = cudaStreamSynchronize(s);
        prof_collect();
        if (e == cudaSuccess) e = e2;
        if (e != cudaSuccess) return to_status(e);
        const uint32_t bits = (uint32_t)m[0];
        if ((bits & ST_SPILLED) && !(bits & kHard) && round < 4) {
            e = table_regrow(ps, m[1], m[kOverWord], s);
            continue;
        }
        // No spill: nothing went to the overflow table (a key goes there only after
        // ST_SPILLED is raised).  Otherwise the result is an error: empty it.
        if (!(bits & ST_SPILLED)) ps->over_dirty = false;
        else if ((e = over_clear(ps, s)) == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return to_status(e);
        const int st = status_from_bits(bits);
        ps->known_count = st == RS_OK ? (long long)m[1] : -1;
        return st;
    }
}
}  // namespace rs

extern "C" int rs_edge_index(const float* d_starts, const float* d_ends, const int32_t* d_sources, uint64_t nE,
                             uint64_t nS, int64_t* d_index, int* h_ordered, void* stream) {
    if (!d_index || (nE && (!d_starts || !d_ends)) || (nS && !d_sources)) return RS_ERR_INVALID;
    const void* q[4] = {d_starts, d_ends, d_sources, d_index};
    for (const void*& x : q)
        if (rs_kernel_pointer(x, &x) != RS_OK) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    int* word = nullptr;
    cudaError_t e = dmalloc((void**)&word, 2 * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(word, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(word + 1, 0xff, sizeof(int), s);  // -1
    long long* index = reinterpret_cast<long long*>(const_cast<void*>(q[3]));
    if (e == cudaSuccess) {
        const EdgePayload p{static_cast<const float*>(q[0]), static_cast<const float*>(q[1]), nullptr, nullptr,
                            static_cast<const int32_t*>(q[2])};
        const uint64_t n = std::max<uint64_t>(std::max(nE, nS), 1);
        launch(k_edge_index, (unsigned)std::min<uint64_t>((n + 255) / 256, 4ull * sm_count()), 256, 0, s, p, nE, nS,
               index, word);
        launch(k_edge_index_head, 1, 1, 0, s, index, (const int*)word, nE);
        e = cudaGetLastError();
    }
    long long head = 0;
    if (e == cudaSuccess && h_ordered) {
        e = cudaMemcpyAsync(&head, index, sizeof(head), cudaMemcpyDefault, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) *h_ordered = head == 1 ? 1 : 0;
    }
    if (word) cudaFreeAsync(word, s);
    return to_status(e);
}

extern "C" int rs_edge_join(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources,
                            uint64_t nE, int swap, rs_pairset* ps, void* stream) {
    if (!target || !ps || (nE && (!d_starts || !d_ends || !d_offsets || !d_counts || !d_sources)))
        return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const int st = bvh_use(target, s);
    if (st != RS_OK) return st;
    cudaError_t e = edge_join_async(target, d_starts, d_ends, d_offsets, d_counts, d_sources, nE, swap, ps, s,
                                    EdgeCull{});
    return table_status(ps, s, e);
}

extern "C" int rs_triangle_join(const rs_bvh* target, const float* d_vertices, uint64_t nV, const uint32_t* d_indices,
                                uint64_t nF, const int32_t* d_tri2obj, int swap, rs_pairset* ps, void* stream) {
    if (!target || !ps || (nF && (!d_vertices || !d_indices || !d_tri2obj))) return RS_ERR_INVALID;
    const uint64_t m = 3 * nF;
    if (m == 0 || target->n_tris == 0) return RS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int st = bvh_use(target, s);
    if (st != RS_OK) return st;
    // bad flag and deferred count in one zeroed pair; records as 32-bit ids when they fit
    // (else every record runs the long path in the first kernel).
    unsigned int* flags = nullptr;
    uint32_t* deferred = nullptr;
    unsigned int hbad = 0;
    cudaError_t e = dmalloc((void**)&flags, 2 * sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned int), s);
    if (e == cudaSuccess && m <= 0xffffffffull) e = dmalloc((void**)&deferred, m * sizeof(uint32_t), s);
    if (e == cudaSuccess) {
        const PairTable table = table_view(ps);
        const int ptok = prof_begin(P_EDGE_JOIN, s);
        launch(k_tri_edge_join, (unsigned)((m + kT - 1) / kT), kT, 0, s, d_vertices, nV, d_indices, d_tri2obj, m,
               (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap, table, flags,
               deferred, flags + 1);
        if (deferred)
            launch(k_tri_edge_long, (unsigned)std::min<uint64_t>((m + kT - 1) / kT, 2ull * sm_count()), kT, 0, s,
                   d_vertices, d_indices, d_tri2obj, (const uint32_t*)deferred, (const unsigned int*)(flags + 1),
                   (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap, table);
        prof_end(P_EDGE_JOIN, s, ptok);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, flags, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    if (flags) cudaFreeAsync(flags, s);
    if (deferred) cudaFreeAsync(deferred, s);
    const int r = table_status(ps, s, e);
    if (r == RS_OK && hbad) return RS_ERR_INVALID;
    return r;
}

static int containment_impl(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                            const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj, int swap,
                            rs_pairset* ps, const Tracking* trk, uint64_t trk_capacity, cudaStream_t s) {
    if (!target || !ps || (src_nF && (!d_src_vertices || !d_src_indices || !d_src_tri2obj))) return RS_ERR_INVALID;
    if (src_nF == 0 || target->n_tris == 0) return RS_OK;
    const int st = bvh_use(target, s);
    if (st != RS_OK) return st;
    int* dmx = nullptr;
    int32_t* first = nullptr;
    int hmx = -1;
    cudaError_t e = dmalloc((void**)&dmx, sizeof(int), s);
    if (e == cudaSuccess) {
        cudaMemsetAsync(dmx, 0xff, sizeof(int), s);
        launch(k_max_obj, 2 * sm_count(), 256, 0, s, d_src_tri2obj, src_nF, dmx);
        e = cudaMemcpyAsync(&hmx, dmx, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    // Objects 0..max id (the reference sizes its launch by the number of distinct ids,
    // which is the same for the contiguous ids preprocess_dataset writes).
    const uint64_t nObj = hmx >= 0 ? (uint64_t)hmx + 1 : 0;
    if (trk && nObj > trk_capacity) {
        if (dmx) cudaFreeAsync(dmx, s);
        cudaStreamSynchronize(s);
        return RS_ERR_OUTPUT_OVERFLOW;
    }
    if (e == cudaSuccess && nObj) {
        e = dmalloc((void**)&first, nObj * sizeof(int32_t), s);
        if (e == cudaSuccess) {
            launch(k_first_tri_init, (unsigned)((nObj + 255) / 256), 256, 0, s, first, nObj);
            launch(k_first_tri, (unsigned)((src_nF + 255) / 256), 256, 0, s, d_src_tri2obj, src_nF, first, nObj);
            const unsigned grid = (unsigned)((nObj + kT - 1) / kT);
            const int ptok = prof_begin(P_CONTAINMENT, s);
            if (trk)
                launch(k_containment<true>, grid, kT, 0, s, d_src_vertices, src_nV, d_src_indices, (const int32_t*)first,
                       nObj, (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap,
                       table_view(ps), *trk);
            else
                launch(k_containment<false>, grid, kT, 0, s, d_src_vertices, src_nV, d_src_indices, (const int32_t*)first,
                       nObj, (const BNode*)target->nodes, max_steps(target), (const float4*)target->tris, swap,
                       table_view(ps), Tracking{0, nullptr, nullptr, nullptr});
            prof_end(P_CONTAINMENT, s, ptok);
            e = cudaGetLastError();
        }
    }
    if (dmx) cudaFreeAsync(dmx, s);
    if (first) cudaFreeAsync(first, s);
    return table_status(ps, s, e);
}

extern "C" int rs_containment(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                              const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj,
                              int swap, rs_pairset* ps, void* stream) {
    return containment_impl(target, d_src_vertices, src_nV, d_src_indices, src_nF, d_src_tri2obj, swap, ps, nullptr,
                            0, (cudaStream_t)stream);
}

extern "C" int rs_containment_tracked(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                                      const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj,
                                      int swap, rs_pairset* ps, int max_targets, int32_t* d_target_ids,
                                      uint32_t* d_target_hits, uint32_t* d_candidate_counts, uint64_t capacity,
                                      void* stream) {
    if (max_targets <= 0 || !d_target_ids || !d_target_hits || !d_candidate_counts) return RS_ERR_INVALID;
    const Tracking trk{max_targets, d_target_ids, d_target_hits, d_candidate_counts};
    return containment_impl(target, d_src_vertices, src_nV, d_src_indices, src_nF, d_src_tri2obj, swap, ps, &trk,
                            capacity, (cudaStream_t)stream);
}
