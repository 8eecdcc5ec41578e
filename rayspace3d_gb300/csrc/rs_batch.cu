// rs_batch.cu -- many point-in-mesh queries and edge-ray joins in one persistent launch.
//
// The reference launches one OptiX pipeline per query (RayLauncher::launch,
// query/src/raytracing/RayLauncher.cpp:39-64; MeshIntersectionLauncher,
// query/src/raytracing/MeshIntersectionLauncher.cpp:279-328) and synchronises after
// each.  A batch instead lists every query's rays as fixed-size chunks; one persistent
// kernel (a few CTAs per SM) has each warp pull the next chunk from a global atomic
// counter and trace its rays with the same per-ray bodies as the single-query kernels
// (rs_query_core.cuh), so queries of very uneven sizes share the GPU without a launch
// or a tail per query.  Axis-aligned point-in-mesh queries read the handle's column
// grid (built at the first submit), others traverse the BVH.  Points whose rays cross
// more than 8 triangles, and edges with more than 4 crossings or a deep traversal, go to
// one overflow list that a second launch resolves exactly.  The launches of an unchanged
// batch are captured once as a CUDA graph and replayed.  rs_batch_autotune times the
// batch over BVH leaf sizes, chunk sizes and traversal stack depths and keeps the best.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "rs_engine.h"
#include "rs_prims.cuh"
#include "rs_query_core.cuh"

namespace rs {
namespace {

constexpr int kBT = 128;                      // threads per CTA of the persistent kernel
constexpr uint64_t kOverflowCap = 1ull << 22;  // rays queued for the exact fallback per submit

struct BatchQuery {
    const BNode* nodes;
    const float4* tris;
    uint32_t max_steps;
    int kind;  // 0 point in mesh, 1 edge rays
    int axis;  // -1 any direction, else the axis of a +e_axis ray
    float dx, dy, dz;
    const float* pts;
    int32_t* obj;
    uint8_t* in;
    const float* starts;
    const float* ends;
    const int32_t* offsets;
    const int32_t* counts;
    const int32_t* sources;
    int swap;
    PairTable table;
    uint64_t n;
    uint64_t first_chunk;
    unsigned int* status;
    int use_grid;  // axis-aligned point-in-mesh through the handle's column grid
    GridView grid;
};

__device__ __forceinline__ int find_query(const BatchQuery* __restrict__ q, int nq, uint64_t chunk) {
    int lo = 0, hi = nq - 1;  // last query whose first_chunk <= chunk
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (q[mid].first_chunk <= chunk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int AXIS, int STACK>
__device__ __forceinline__ void batch_pim_ray(const BatchQuery& Q, int qi, uint64_t i, uint2* __restrict__ ovf,
                                              unsigned long long* __restrict__ ovf_count) {
    const Ray r = make_ray(Q.pts[3 * i], Q.pts[3 * i + 1], Q.pts[3 * i + 2], Q.dx, Q.dy, Q.dz, kEps, kTmax);
    HitList hl;
    unsigned int tests = 0;
    const bool ok = pim_collect<AXIS, STACK>(Q.nodes, Q.max_steps, Q.tris, r, hl, tests);
    add_tests(tests);
    if (!ok) {
        atomicOr(Q.status, ST_STACK_OVERFLOW);
        return;
    }
    if (hl.ovf) {
        const unsigned long long slot = atomicAdd(ovf_count, 1ull);
        if (slot < kOverflowCap) ovf[slot] = make_uint2((uint32_t)qi, (uint32_t)i);
        else atomicOr(Q.status, ST_HIT_OVERFLOW);
        return;
    }
    write_result(hl.finish(), i, Q.obj, Q.in);
}

template <int STACK>
__global__ void __launch_bounds__(kBT) k_batch(const BatchQuery* __restrict__ q, int nq, uint64_t total_chunks,
                                               int chunk, unsigned long long* __restrict__ next,
                                               uint2* __restrict__ ovf, unsigned long long* __restrict__ ovf_count) {
    __shared__ GridWarpSlots slots[kBT / 32];
    __shared__ EdgeSmem<kBT, STACK> esm;  // edge rays' stacks and crossings, one column per thread
    const int lane = threadIdx.x & 31;
    GridWarpSlots& sl = slots[threadIdx.x >> 5];
    for (;;) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(next, 1ull);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= total_chunks) return;
        const int qi = find_query(q, nq, c);
        const BatchQuery& Q = q[qi];
        const uint64_t r0 = (c - Q.first_chunk) * (uint64_t)chunk;
        const uint64_t r1 = min(r0 + (uint64_t)chunk, Q.n);
        if (Q.kind == 0 && Q.use_grid) {
            // Warp-cooperative rounds of 32 points: every lane takes part in each round.
            for (uint64_t base = r0; base < r1; base += 32) {
                const uint64_t i = base + lane;
                const bool valid = i < r1;
                float p[3] = {0.0f, 0.0f, 0.0f};
                if (valid) {
                    p[0] = Q.pts[3 * i];
                    p[1] = Q.pts[3 * i + 1];
                    p[2] = Q.pts[3 * i + 2];
                }
                auto spill = [&]() {
                    const unsigned long long slot = atomicAdd(ovf_count, 1ull);
                    if (slot < kOverflowCap) ovf[slot] = make_uint2((uint32_t)qi, (uint32_t)i);
                    else atomicOr(Q.status, ST_HIT_OVERFLOW);
                };
                if (Q.axis == 0) pim_grid_warp<0>(Q.grid, Q.tris, p, valid, valid, i, Q.obj, Q.in, sl, spill);
                else if (Q.axis == 1) pim_grid_warp<1>(Q.grid, Q.tris, p, valid, valid, i, Q.obj, Q.in, sl, spill);
                else pim_grid_warp<2>(Q.grid, Q.tris, p, valid, valid, i, Q.obj, Q.in, sl, spill);
                __syncwarp();
            }
            continue;
        }
        for (uint64_t i = r0 + lane; i < r1; i += 32) {
            if (Q.kind == 1) {
                const EdgePayload p{Q.starts, Q.ends, Q.offsets, Q.counts, Q.sources};
                if (!edge_ray_fast<STACK>(esm.column(threadIdx.x), p, i, Q.nodes, Q.max_steps, Q.tris, Q.swap,
                                          Q.table)) {
                    const unsigned long long slot = atomicAdd(ovf_count, 1ull);
                    if (slot < kOverflowCap) ovf[slot] = make_uint2((uint32_t)qi, (uint32_t)i);
                    else atomicOr(Q.status, ST_HIT_OVERFLOW);
                }
            } else if (Q.axis == 0) {
                batch_pim_ray<0, STACK>(Q, qi, i, ovf, ovf_count);
            } else if (Q.axis == 1) {
                batch_pim_ray<1, STACK>(Q, qi, i, ovf, ovf_count);
            } else if (Q.axis == 2) {
                batch_pim_ray<2, STACK>(Q, qi, i, ovf, ovf_count);
            } else {
                batch_pim_ray<-1, STACK>(Q, qi, i, ovf, ovf_count);
            }
        }
    }
}

template <int STACK>
__global__ void __launch_bounds__(kBT) k_batch_fallback(const BatchQuery* __restrict__ q,
                                                        const uint2* __restrict__ ovf,
                                                        const unsigned long long* __restrict__ ovf_count) {
    const unsigned long long cnt = min(*ovf_count, (unsigned long long)kOverflowCap);
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < cnt;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 item = ovf[e];
        const BatchQuery& Q = q[item.x];
        const uint64_t i = item.y;
        if (Q.kind == 1) {
            edge_ray_long(EdgePayload{Q.starts, Q.ends, Q.offsets, Q.counts, Q.sources}, i, Q.nodes, Q.max_steps,
                          Q.tris, Q.swap, Q.table);
            continue;
        }
        const Ray r = make_ray(Q.pts[3 * i], Q.pts[3 * i + 1], Q.pts[3 * i + 2], Q.dx, Q.dy, Q.dz, kEps, kTmax);
        if (Q.axis == 0) pim_fallback_ray<0, STACK>(Q.nodes, Q.max_steps, Q.tris, r, Q.status, Q.obj, Q.in, i);
        else if (Q.axis == 1) pim_fallback_ray<1, STACK>(Q.nodes, Q.max_steps, Q.tris, r, Q.status, Q.obj, Q.in, i);
        else if (Q.axis == 2) pim_fallback_ray<2, STACK>(Q.nodes, Q.max_steps, Q.tris, r, Q.status, Q.obj, Q.in, i);
        else pim_fallback_ray<-1, STACK>(Q.nodes, Q.max_steps, Q.tris, r, Q.status, Q.obj, Q.in, i);
    }
}

}  // namespace

PairTable table_view(rs_pairset* ps);

int recheck_batch(int op, unsigned long long* out) { return recheck_op(op, out); }

}  // namespace rs

using namespace rs;

struct rs_batch_item {
    int kind = 0;
    const rs_bvh* bvh = nullptr;
    const float* pts = nullptr;
    uint64_t n = 0;
    float d[3] = {0, 0, 1};
    int32_t* obj = nullptr;
    uint8_t* in = nullptr;
    const float* starts = nullptr;
    const float* ends = nullptr;
    const int32_t* offsets = nullptr;
    const int32_t* counts = nullptr;
    const int32_t* sources = nullptr;
    int swap = 0;
    rs_pairset* ps = nullptr;
    uint64_t gen = 0;  // ps->generation when the batch was committed
};

struct rs_batch {
    std::vector<rs_batch_item> items;
    int chunk = 64;
    int stack = 64;
    int use_graph = 1;
    // Device state of the committed batch.
    bool dirty = true;
    BatchQuery* d_q = nullptr;
    unsigned int* d_status = nullptr;
    unsigned long long* d_counters = nullptr;  // [0] next chunk, [1] overflow count
    uint2* d_ovf = nullptr;
    uint64_t total_chunks = 0;
    int grid = 0;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t last_stream = nullptr;
    // BVHs the autotuner rebuilt with another leaf size, by the caller's handle.
    std::map<const rs_bvh*, rs_bvh*> own;
    int device = 0;
};

namespace {

const rs_bvh* effective(const rs_batch* b, const rs_bvh* h) {
    auto it = b->own.find(h);
    return it == b->own.end() ? h : it->second;
}

void release_device(rs_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    if (b->d_q) cudaFree(b->d_q);
    if (b->d_status) cudaFree(b->d_status);
    if (b->d_counters) cudaFree(b->d_counters);
    if (b->d_ovf) cudaFree(b->d_ovf);
    b->d_q = nullptr;
    b->d_status = nullptr;
    b->d_counters = nullptr;
    b->d_ovf = nullptr;
    b->dirty = true;
}

int commit(rs_batch* b, cudaStream_t s) {
    if (!b->dirty) return RS_OK;
    release_device(b);
    const int nq = (int)b->items.size();
    std::vector<BatchQuery> hq(nq);
    uint64_t chunks = 0;
    bool any_pim = false;
    for (int i = 0; i < nq; ++i) {
        rs_batch_item& it = b->items[i];
        if (it.ps) it.gen = it.ps->generation;
        const rs_bvh* h = effective(b, it.bvh);
        const int st = bvh_ready(h);
        if (st != RS_OK) return st;
        BatchQuery& q = hq[i];
        std::memset(&q, 0, sizeof(q));
        q.nodes = h->nodes;
        q.tris = (const float4*)h->tris;
        q.max_steps = max_steps(h);
        q.kind = it.kind;
        q.n = h->n_tris ? it.n : 0;  // nothing to hit: outputs are set below
        q.first_chunk = chunks;
        chunks += (q.n + b->chunk - 1) / b->chunk;
        if (it.kind == 0) {
            any_pim = true;
            q.dx = it.d[0];
            q.dy = it.d[1];
            q.dz = it.d[2];
            const bool zx = it.d[0] == 0.0f, zy = it.d[1] == 0.0f, zz = it.d[2] == 0.0f;
            q.axis = (it.d[2] == 1.0f && zx && zy) ? 2 : (it.d[0] == 1.0f && zy && zz) ? 0
                                                         : (it.d[1] == 1.0f && zx && zz) ? 1 : -1;
            q.pts = it.pts;
            q.obj = it.obj;
            q.in = it.in;
            if (q.axis >= 0 && h->n_tris > 0) {
                const int g = ensure_grid(h, q.axis, s);
                if (g != RS_OK) return g;
                const rs_column_grid& cg = h->cgrid[q.axis];
                q.use_grid = 1;
                q.grid = GridView{cg.u0, cg.v0, cg.su, cg.sv, cg.u1, cg.v1, cg.gu, cg.gv, cg.start, cg.list};
            }
        } else {
            q.axis = -1;
            q.starts = it.starts;
            q.ends = it.ends;
            q.offsets = it.offsets;
            q.counts = it.counts;
            q.sources = it.sources;
            q.swap = it.swap;
            q.table = table_view(it.ps);
        }
    }
    cudaError_t e = cudaMalloc((void**)&b->d_q, std::max(nq, 1) * sizeof(BatchQuery));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_status, std::max(nq, 1) * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_counters, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess && nq) e = cudaMalloc((void**)&b->d_ovf, kOverflowCap * sizeof(uint2));
    for (int i = 0; i < nq && e == cudaSuccess; ++i) {
        const rs_batch_item& it = b->items[i];
        hq[i].status = it.kind == 1 ? hq[i].table.status : b->d_status + i;
    }
    if (e == cudaSuccess && nq) e = cudaMemcpy(b->d_q, hq.data(), nq * sizeof(BatchQuery), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        release_device(b);
        return to_status(e);
    }
    b->total_chunks = chunks;
    int per_sm = 0;
    if (b->stack == 32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<32>, kBT, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<64>, kBT, 0);
    b->grid = std::max(1, per_sm) * sm_count();
    b->dirty = false;
    return RS_OK;
}

// One fallback thread per possible overflow entry, up to the list's capacity (the count
// is only known on the device; threads past it return at once).
unsigned fallback_grid(const rs_batch* b) {
    uint64_t rays = 0;
    for (const rs_batch_item& it : b->items) rays += it.n;
    return (unsigned)std::max<uint64_t>(1, (std::min(rays, kOverflowCap) + kBT - 1) / kBT);
}

// The launches of one submit: counters, per-query statuses, outputs of queries against
// empty meshes, the persistent kernel and the overflow fallback.
cudaError_t enqueue(rs_batch* b, cudaStream_t s) {
    const int nq = (int)b->items.size();
    cudaError_t e = cudaMemsetAsync(b->d_counters, 0, 2 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_status, 0, std::max(nq, 1) * sizeof(unsigned int), s);
    for (int i = 0; i < nq && e == cudaSuccess; ++i) {
        const rs_batch_item& it = b->items[i];
        if (it.kind != 0 || effective(b, it.bvh)->n_tris || it.n == 0) continue;
        if (it.obj) e = cudaMemsetAsync(it.obj, 0xff, it.n * sizeof(int32_t), s);
        if (e == cudaSuccess && it.in) e = cudaMemsetAsync(it.in, 0, it.n, s);
    }
    if (e != cudaSuccess) return e;
    if (b->total_chunks) {
        if (b->stack == 32) {
            launch(k_batch<32>, b->grid, kBT, 0, s, (const BatchQuery*)b->d_q, nq, b->total_chunks, b->chunk,
                   b->d_counters, b->d_ovf, b->d_counters + 1);
            if (b->d_ovf) launch(k_batch_fallback<32>, fallback_grid(b), kBT, 0, s, (const BatchQuery*)b->d_q,
                                 (const uint2*)b->d_ovf, (const unsigned long long*)b->d_counters + 1);
        } else {
            launch(k_batch<64>, b->grid, kBT, 0, s, (const BatchQuery*)b->d_q, nq, b->total_chunks, b->chunk,
                   b->d_counters, b->d_ovf, b->d_counters + 1);
            if (b->d_ovf) launch(k_batch_fallback<64>, fallback_grid(b), kBT, 0, s, (const BatchQuery*)b->d_q,
                                 (const uint2*)b->d_ovf, (const unsigned long long*)b->d_counters + 1);
        }
    }
    return cudaGetLastError();
}

}  // namespace

extern "C" int rs_batch_create(rs_batch** out) {
    if (!out) return RS_ERR_INVALID;
    *out = new rs_batch();
    cudaGetDevice(&(*out)->device);
    return RS_OK;
}

extern "C" int rs_batch_destroy(rs_batch* b) {
    if (!b) return RS_OK;
    if (b->last_stream) cudaStreamSynchronize(b->last_stream);
    release_device(b);
    for (auto& kv : b->own) rs_bvh_destroy(kv.second);
    delete b;
    return RS_OK;
}

extern "C" int rs_batch_add_pim(rs_batch* b, const rs_bvh* bvh, const float* d_points, uint64_t n, float dx,
                                float dy, float dz, int32_t* d_obj, uint8_t* d_inside, int* index) {
    if (!b || !bvh || (n && !d_points) || n > 0xffffffffull) return RS_ERR_INVALID;
    rs_batch_item it;
    it.kind = 0;
    it.bvh = bvh;
    it.pts = d_points;
    it.n = n;
    it.d[0] = dx;
    it.d[1] = dy;
    it.d[2] = dz;
    it.obj = d_obj;
    it.in = d_inside;
    b->items.push_back(it);
    b->dirty = true;
    if (index) *index = (int)b->items.size() - 1;
    return RS_OK;
}

extern "C" int rs_batch_add_edges(rs_batch* b, const rs_bvh* target, const float* d_starts, const float* d_ends,
                                  const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources,
                                  uint64_t nE, int swap, rs_pairset* ps, int* index) {
    if (!b || !target || !ps || (nE && (!d_starts || !d_ends || !d_offsets || !d_counts || !d_sources)))
        return RS_ERR_INVALID;
    rs_batch_item it;
    it.kind = 1;
    it.bvh = target;
    it.n = nE;
    it.starts = d_starts;
    it.ends = d_ends;
    it.offsets = d_offsets;
    it.counts = d_counts;
    it.sources = d_sources;
    it.swap = swap;
    it.ps = ps;
    b->items.push_back(it);
    b->dirty = true;
    if (index) *index = (int)b->items.size() - 1;
    return RS_OK;
}

extern "C" int rs_batch_set_options(rs_batch* b, int chunk, int stack_depth, int use_graph) {
    if (!b) return RS_ERR_INVALID;
    if (chunk == 0) chunk = 64;
    if (stack_depth == 0) stack_depth = 64;
    if (chunk < 32 || chunk > 4096 || (chunk & 31) || (stack_depth != 32 && stack_depth != 64)) return RS_ERR_INVALID;
    if (chunk != b->chunk || stack_depth != b->stack) b->dirty = true;
    b->chunk = chunk;
    b->stack = stack_depth;
    b->use_graph = use_graph != 0;
    if (!b->use_graph && b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return RS_OK;
}

extern "C" int rs_batch_submit(rs_batch* b, void* stream) {
    if (!b) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    for (const rs_batch_item& it : b->items)
        if (it.ps && it.ps->generation != it.gen) b->dirty = true;  // its slots were reallocated
    const int st = commit(b, s);
    if (st != RS_OK) return st;
    for (const rs_batch_item& it : b->items) {
        const int u = bvh_use(effective(b, it.bvh), s);
        if (u != RS_OK) return u;
        if (it.ps) it.ps->known_count = -1;  // a replayed graph inserts without table_view()
    }
    b->last_stream = s;
    if (!b->use_graph || s == nullptr) return to_status(enqueue(b, s));  // the legacy stream cannot be captured
    if (!b->exec) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return to_status(e);
        const cudaError_t e1 = enqueue(b, s);
        e = cudaStreamEndCapture(s, &g);
        if (e1 != cudaSuccess) e = e1;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return to_status(e);
        }
    }
    return to_status(cudaGraphLaunch(b->exec, s));
}

extern "C" int rs_batch_wait(rs_batch* b, int* h_status) {
    if (!b) return RS_ERR_INVALID;
    cudaError_t e = b->last_stream ? cudaStreamSynchronize(b->last_stream) : cudaDeviceSynchronize();
    if (e != cudaSuccess) return to_status(e);
    const int nq = (int)b->items.size();
    if (nq == 0 || b->dirty) return RS_OK;
    std::vector<unsigned int> st(nq, 0);
    e = cudaMemcpy(st.data(), b->d_status, nq * sizeof(unsigned int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return to_status(e);
    int first = RS_OK;
    for (int i = 0; i < nq; ++i) {
        unsigned int bits = st[i];
        if (b->items[i].kind == 1) {
            unsigned long long m = 0;
            e = cudaMemcpy(&m, b->items[i].ps->meta, sizeof(m), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return to_status(e);
            bits = (unsigned int)m;
        }
        int ts = status_from_bits(bits);
        if (b->items[i].kind == 1 && (bits & ST_SPILLED))  // regrow from the overflow table, or empty it
            ts = table_status(b->items[i].ps, b->last_stream, cudaSuccess);
        const int s = bits & ST_HIT_OVERFLOW ? RS_ERR_OUTPUT_OVERFLOW : ts;
        if (h_status) h_status[i] = s;
        if (first == RS_OK) first = s;
    }
    return first;
}

extern "C" int rs_batch_autotune(rs_batch* b, int* h_leaf, int* h_chunk, int* h_stack, double* h_ms, void* stream) {
    if (!b) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    // The caller's BVHs and the geometry they were built from.
    std::vector<const rs_bvh*> orig;
    for (const rs_batch_item& it : b->items)
        if (std::find(orig.begin(), orig.end(), it.bvh) == orig.end()) orig.push_back(it.bvh);
    const int leaves[4] = {2, 4, 8, 16};
    const int chunks[3] = {32, 64, 128};
    const int stacks[2] = {32, 64};
    const int graph = b->use_graph;
    double best = -1.0;
    int best_leaf = 4, best_chunk = b->chunk, best_stack = b->stack;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int result = RS_OK;
    for (int leaf : leaves) {
        // Rebuild every BVH of the batch with this leaf size.
        for (auto& kv : b->own) rs_bvh_destroy(kv.second);
        b->own.clear();
        for (const rs_bvh* h : orig) {
            rs_bvh* nb = nullptr;
            const int st = rs_bvh_build(h->V, h->nV, h->I, h->nF, h->t2o, leaf, &nb, s);
            if (st != RS_OK) {
                result = st;
                break;
            }
            b->own[h] = nb;
        }
        if (result != RS_OK) break;
        b->dirty = true;
        for (int ch : chunks) {
            for (int sd : stacks) {
                rs_batch_set_options(b, ch, sd, 0);
                double ms_sum = 0.0;
                bool ok = true;
                for (int rep = 0; rep < 3 && ok; ++rep) {
                    cudaEventRecord(e0, s);
                    ok = rs_batch_submit(b, s) == RS_OK;
                    cudaEventRecord(e1, s);
                    ok = ok && rs_batch_wait(b, nullptr) == RS_OK;
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) ms_sum += ms;  // the first run warms up
                }
                if (ok && (best < 0.0 || ms_sum / 2.0 < best)) {
                    best = ms_sum / 2.0;
                    best_leaf = leaf;
                    best_chunk = ch;
                    best_stack = sd;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // Keep the best configuration (leaf size 4 is the caller's own BVHs' default).
    for (auto& kv : b->own) rs_bvh_destroy(kv.second);
    b->own.clear();
    if (result == RS_OK && best >= 0.0) {
        for (const rs_bvh* h : orig) {
            if (best_leaf == h->leaf_size) continue;
            rs_bvh* nb = nullptr;
            const int st = rs_bvh_build(h->V, h->nV, h->I, h->nF, h->t2o, best_leaf, &nb, s);
            if (st != RS_OK) {
                result = st;
                break;
            }
            b->own[h] = nb;
        }
    }
    rs_batch_set_options(b, best_chunk, best_stack, graph);
    b->dirty = true;
    if (h_leaf) *h_leaf = best_leaf;
    if (h_chunk) *h_chunk = best_chunk;
    if (h_stack) *h_stack = best_stack;
    if (h_ms) *h_ms = best;
    if (result == RS_OK && best < 0.0) result = RS_ERR_ITER_LIMIT;  // no configuration completed
    return result;
}
