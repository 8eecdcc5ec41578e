// rs_join.cu -- edge-ray overlap and the containment fallback.
//
// Edge rays replace __raygen__mesh_overlap_edges / trace_edge_multi_hits_edges
// (query/src/cuda/mesh_overlap_edges.cu:106-216) and __raygen__mesh_overlap
// (mesh_intersection.cu:16-91,288-334): one thread per unique edge traces the
// segment once (the reference re-traces per hit and, in the intersection variant,
// per source object) and inserts (source, target) pairs straight into the pair
// table.  Containment replaces __raygen__mesh_containment_anyhit +
// __anyhit__ah_containment (mesh_intersection_anyhit.cu:46-240): one +Z ray per
// source object, parity per target object kept in registers instead of a
// 256-slot global scratch per object.
#include <climits>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kT = 128;
constexpr int kTargets = 32;

__global__ void __launch_bounds__(kT) k_edge_join(const float* __restrict__ starts, const float* __restrict__ ends,
                                                  const int32_t* __restrict__ offsets,
                                                  const int32_t* __restrict__ counts,
                                                  const int32_t* __restrict__ sources, uint64_t nE,
                                                  const BNode* __restrict__ nodes, uint32_t max_steps,
                                                  const float4* __restrict__ tris, int swap, PairTable table) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= nE) return;
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
    const bool ok = traverse<-1>(nodes, max_steps, r, [&](int first, int cnt) {
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
    PairTable t;
    t.slots = ps->slots;
    t.capacity = ps->capacity;
    t.pow2 = ps->pow2;
    t.max_probes = ps->max_probes;
    t.status = reinterpret_cast<unsigned int*>(ps->meta);
    t.count = ps->meta + 1;
    t.stats = ps->track ? ps->meta + 2 : nullptr;
    return t;
}

}  // namespace rs

using namespace rs;

namespace rs {
// Launches one edge-ray direction without waiting for it (status lands in the table's meta word).
cudaError_t edge_join_async(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources, uint64_t nE,
                            int swap, rs_pairset* ps, cudaStream_t s) {
    if (nE == 0 || target->n_tris == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((nE + kT - 1) / kT);
    const int ptok = prof_begin(P_EDGE_JOIN, s);
    launch(k_edge_join, grid, kT, 0, s, d_starts, d_ends, d_offsets, d_counts, d_sources, nE, target->nodes,
           max_steps(target), target->tris, swap, table_view(ps));
    prof_end(P_EDGE_JOIN, s, ptok);
    return cudaGetLastError();
}

// Waits for the stream and turns the table's status bits into an rs_status.
int table_status(rs_pairset* ps, cudaStream_t s, cudaError_t e) {
    unsigned long long st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, ps->meta, sizeof(st), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    prof_collect();
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return to_status(e);
    return status_from_bits((uint32_t)st);
}
}  // namespace rs

extern "C" int rs_edge_join(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources,
                            uint64_t nE, int swap, rs_pairset* ps, void* stream) {
    if (!target || !ps || (nE && (!d_starts || !d_ends || !d_offsets || !d_counts || !d_sources)))
        return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = edge_join_async(target, d_starts, d_ends, d_offsets, d_counts, d_sources, nE, swap, ps, s);
    return table_status(ps, s, e);
}

static int containment_impl(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                            const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj, int swap,
                            rs_pairset* ps, const Tracking* trk, uint64_t trk_capacity, cudaStream_t s) {
    if (!target || !ps || (src_nF && (!d_src_vertices || !d_src_indices || !d_src_tri2obj))) return RS_ERR_INVALID;
    if (src_nF == 0 || target->n_tris == 0) return RS_OK;
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
