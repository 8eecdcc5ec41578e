// rs_pairs.cu -- pair tables, deterministic finalisation and the join drivers.
//
// Replaces the hash-table lifecycle of executeHashQuery
// (query/src/applications/raytracer_overlap_estimated_main.cpp:39-112,
// raytracer_intersection_estimated_main.cpp:77-176), compact_hash_table_pairs and
// merge_and_deduplicate_pairs_gpu (query/src/cuda/mesh_query_deduplication.cu:56-144).
// Differences by design: no key is dropped (the reference drops one after 5000 / 1000
// probes).  A table past 3/4 load sends keys that do not settle at their first slot to
// the pair set's overflow table, and the status read after the launches regrows the
// table from both; only a key that finds no slot in either raises RS_ERR_TABLE_FULL,
// after which the drivers grow the table and rerun.  The finalised output is sorted, so
// it does not depend on slot order or atomic timing.
#include <algorithm>
#include <cstring>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
PairTable table_view(rs_pairset* ps);
cudaError_t edge_join_async(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources, uint64_t nE,
                            int swap, rs_pairset* ps, cudaStream_t s, const EdgeCull& cull);
cudaError_t cull_pair_async(const rs_bvh* A, const rs_bvh* B, uint8_t* candA, uint8_t* candB, cudaStream_t s);
cudaError_t cull_impl(const rs_bvh* A, const rs_bvh* B, uint8_t* candA, uint8_t* candB, int32_t* partA,
                      int32_t* partB, uint32_t* entryA, uint32_t* entryB, const int** boxes_out, int** tmps_out,
                      cudaStream_t s);
cudaError_t edge_join_pair_async(const rs_bvh* A, const float* startsA, const float* endsA, const int32_t* offsetsA,
                                 const int32_t* countsA, const int32_t* sourcesA, uint64_t nEA, const EdgeCull& cullA,
                                 const rs_bvh* B, const float* startsB, const float* endsB, const int32_t* offsetsB,
                                 const int32_t* countsB, const int32_t* sourcesB, uint64_t nEB, const EdgeCull& cullB,
                                 rs_pairset* ps, cudaStream_t s);
bool g_overlap_cull = true;

namespace {

__global__ void k_swap_halves(uint64_t* __restrict__ k, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) k[i] = (k[i] << 32) | (k[i] >> 32);
}

uint64_t next_pow2(uint64_t v) {
    if (v == 0) return 1;
    --v;
    v |= v >> 1;
    v |= v >> 2;
    v |= v >> 4;
    v |= v >> 8;
    v |= v >> 16;
    v |= v >> 32;
    return v + 1;
}

}  // namespace

cudaError_t alloc_slots(rs_pairset* ps, uint64_t capacity, cudaStream_t s) {
    ps->known_count = -1;
    if (ps->slots) cudaFreeAsync(ps->slots, s);
    ps->slots = nullptr;
    ps->capacity = capacity;
    ps->max_probes = (unsigned)std::min<uint64_t>(capacity, 8192);
    ++ps->generation;
    return dmalloc((void**)&ps->slots, capacity * sizeof(unsigned long long), s);
}

namespace {
// Reinserts the keys of a spilled table's old slots (n_slots) and of its overflow table
// (n_over slots) into the regrown table, skipping empty slots.
__global__ void __launch_bounds__(256) k_rehash(PairTable t, const unsigned long long* __restrict__ keys,
                                                const unsigned long long* __restrict__ over, uint64_t n_slots,
                                                uint64_t n_over) {
    const uint64_t n = n_slots + n_over;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = i < n_slots ? keys[i] : over[i - n_slots];
        if (k != kEmptyKey) table_insert(t, k);
    }
}
}  // namespace

cudaError_t over_clear(rs_pairset* ps, cudaStream_t s) {
    if (!ps->over || !ps->over_dirty) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(ps->over, 0xff, kOverSlots * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ps->meta + kOverWord, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) ps->over_dirty = false;
    return e;
}

cudaError_t table_regrow(rs_pairset* ps, uint64_t count, uint64_t over, cudaStream_t s) {
    // Room for every key at load 1/2 or less (a key may be in both tables, so this is
    // generous), and at least four times the old slots.
    const uint64_t need = 2 * (count + over);
    uint64_t cap = ps->capacity * 4;
    while (cap < need) cap *= 2;
    if (!ps->pow2 && cap % 2 == 0) cap += 1;
    if (cap > (1ull << 34)) return cudaErrorMemoryAllocation;
    unsigned long long* old = ps->slots;
    const uint64_t old_cap = ps->capacity;
    // The overflow table is rehashed from a copy: the regrown table may overflow into it.
    unsigned long long* over_copy = nullptr;
    cudaError_t e = cudaSuccess;
    if (over) {
        e = dmalloc((void**)&over_copy, kOverSlots * sizeof(unsigned long long), s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(over_copy, ps->over, kOverSlots * sizeof(unsigned long long), cudaMemcpyDeviceToDevice,
                                s);
        if (e == cudaSuccess) e = over_clear(ps, s);
    }
    ps->slots = nullptr;  // the old slots stay allocated until the rehash has read them
    if (e == cudaSuccess) e = alloc_slots(ps, cap, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ps->slots, 0xff, cap * sizeof(unsigned long long), s);
    // Status and count start over.
    if (e == cudaSuccess) e = cudaMemsetAsync(ps->meta, 0, 2 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        PairTable t = table_view(ps);
        t.stats = nullptr;
        const uint64_t n = old_cap + (over ? kOverSlots : 0);
        const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 4u * sm_count());
        launch(k_rehash, grid, 256, 0, s, t, (const unsigned long long*)old, (const unsigned long long*)over_copy,
               old_cap, over ? kOverSlots : 0);
        e = cudaGetLastError();
    }
    if (old) cudaFreeAsync(old, s);
    if (over_copy) cudaFreeAsync(over_copy, s);
    return e;
}
}  // namespace rs

using namespace rs;

extern "C" int rs_kernel_pointer(const void* p, const void** out) {
    if (!out) return RS_ERR_INVALID;
    *out = nullptr;
    if (!p) return RS_OK;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return RS_ERR_INVALID;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        *out = p;
        return RS_OK;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) {
        *out = a.devicePointer;
        return RS_OK;
    }
    return RS_ERR_INVALID;  // pageable host memory: no kernel may read it
}

extern "C" uint64_t rs_hash_size_pow2(int64_t est) {
    uint64_t size = 16777216ull;
    if (est > 0) {
        uint64_t target = (uint64_t)(est / 0.5);
        if (target < 1024) target = 1024;
        if (target > 1073741824ull) target = 1073741824ull;
        size = next_pow2(target);
    }
    return size;
}

extern "C" uint64_t rs_hash_size_odd(int64_t est, float load_factor) {
    int64_t size = 16777216;
    if (est > 0) {
        uint64_t target = (uint64_t)(est / load_factor);
        if (target < 1024) target = 1024;
        if (target > 1073741824ull) target = 1073741824ull;
        size = (int64_t)target;
        if (size % 2 == 0) size += 1;
    }
    return (uint64_t)size;
}

extern "C" int rs_pairset_create(uint64_t capacity, int pow2, rs_pairset** out, void* stream) {
    if (!out || capacity == 0 || capacity > (1ull << 36)) return RS_ERR_INVALID;
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    rs_pairset* ps = new rs_pairset();
    cudaGetDevice(&ps->device);
    ps->pow2 = pow2 ? 1 : 0;
    if (ps->pow2) capacity = next_pow2(capacity);
    cudaError_t e = dmalloc((void**)&ps->meta, (kMetaWords + kOverSlots) * sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        ps->over = ps->meta + kMetaWords;
        ps->over_dirty = true;  // cleared below
        e = over_clear(ps, s);
    }
    if (e == cudaSuccess) e = alloc_slots(ps, capacity, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        if (ps->meta) cudaFree(ps->meta);
        if (ps->slots) cudaFree(ps->slots);
        delete ps;
        return to_status(e);
    }
    *out = ps;
    return rs_pairset_clear(ps, stream);
}

extern "C" int rs_pairset_clear(rs_pairset* ps, void* stream) {
    if (!ps) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    ps->known_count = -1;
    cudaError_t e = cudaMemsetAsync(ps->slots, 0xff, ps->capacity * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ps->meta, 0, kMetaWords * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = over_clear(ps, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) ps->known_count = 0;
    return to_status(e);
}

extern "C" int rs_pairset_destroy(rs_pairset* ps) {
    if (!ps) return RS_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(ps->device);
    if (ps->slots) cudaFree(ps->slots);
    if (ps->meta) cudaFree(ps->meta);
    cudaSetDevice(prev);
    delete ps;
    return RS_OK;
}

extern "C" int rs_pairset_info(const rs_pairset* ps, uint64_t* capacity, uint64_t* count, void* stream) {
    if (!ps) return RS_ERR_INVALID;
    if (capacity) *capacity = ps->capacity;
    if (count && ps->known_count >= 0) {
        *count = (uint64_t)ps->known_count;
    } else if (count) {
        cudaStream_t s = (cudaStream_t)stream;
        unsigned long long c = 0;
        cudaError_t e = cudaMemcpyAsync(&c, ps->meta + 1, sizeof(c), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return to_status(e);
        *count = c;
    }
    return RS_OK;
}

extern "C" int rs_pairset_finalize(rs_pairset* ps, int order, uint64_t* d_keys, uint64_t capacity,
                                   uint64_t* h_count, void* stream) {
    const bool no_wait = (order & RS_FINALIZE_NO_WAIT) != 0;
    order &= ~RS_FINALIZE_NO_WAIT;
    if (!ps || !h_count || (capacity && !d_keys)) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    *h_count = 0;
    cudaError_t e = cudaSuccess;
    // The status and count: from the last read when no launch has touched the table since.
    uint64_t n = 0;
    if (ps->known_count >= 0) {
        n = (uint64_t)ps->known_count;
    } else {
        const int st = table_status(ps, s, cudaSuccess);  // regrows a spilled table first
        if (st != RS_OK) return st;
        n = (uint64_t)ps->known_count;
    }
    if (n == 0) return RS_OK;
    if (n <= kSmallTableSort && n <= capacity) {
        // Gather and one-block sort straight into d_keys; nothing to read back.
        const int ptok = prof_begin(P_FINALIZE, s);
        e = table_keys_sorted_small(reinterpret_cast<const uint64_t*>(ps->slots), ps->capacity, kEmptyKey,
                                    order == 1 ? 1 : 0, d_keys, n, ps->meta + kGatherWord, s);
        prof_end(P_FINALIZE, s, ptok);
        if (e == cudaSuccess && !no_wait) e = cudaStreamSynchronize(s);
        if (!no_wait) prof_collect();
        if (e != cudaSuccess) return to_status(e);
        *h_count = n;
        return RS_OK;
    }
    uint64_t* tmp = nullptr;
    uint64_t* dcount = nullptr;
    const int ptok = prof_begin(P_FINALIZE, s);
    e = dmalloc((void**)&tmp, n * sizeof(uint64_t), s);
    if (e == cudaSuccess) e = dmalloc((void**)&dcount, sizeof(uint64_t), s);
    if (e == cudaSuccess) e = compact_u64(reinterpret_cast<const uint64_t*>(ps->slots), ps->capacity, kEmptyKey, tmp,
                                          dcount, s);
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (e == cudaSuccess && order == 1) launch(k_swap_halves, grid, 256, 0, s, tmp, n);
    if (e == cudaSuccess) e = sort_u64_any(tmp, n, s);
    if (e == cudaSuccess && order == 1) launch(k_swap_halves, grid, 256, 0, s, tmp, n);
    const uint64_t ncopy = std::min<uint64_t>(n, capacity);
    if (e == cudaSuccess && ncopy)
        e = cudaMemcpyAsync(d_keys, tmp, ncopy * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
    prof_end(P_FINALIZE, s, ptok);
    if (tmp) cudaFreeAsync(tmp, s);
    if (dcount) cudaFreeAsync(dcount, s);
    uint32_t sort_err = 0;
    if (e == cudaSuccess) e = sort_error_read(&sort_err, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    prof_collect();
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return to_status(e);
    if (sort_err) {
        sort_error_clear(s);
        return RS_ERR_ITER_LIMIT;
    }
    *h_count = n;
    return n > capacity ? RS_ERR_OUTPUT_OVERFLOW : RS_OK;
}

// *p replaced by the address kernels read it through (rs_kernel_pointer); false when none.
template <class T>
static bool kernel_ptr(const T** p) {
    const void* q = nullptr;
    if (rs_kernel_pointer(*p, &q) != RS_OK) return false;
    *p = static_cast<const T*>(q);
    return true;
}

static int overlap_join_impl(const rs_bvh* A, const float* d_startsA, const float* d_endsA,
                             const int32_t* d_offsetsA, const int32_t* d_countsA, const int32_t* d_sourcesA,
                             uint64_t nEA, const rs_bvh* B, const float* d_startsB, const float* d_endsB,
                             const int32_t* d_offsetsB, const int32_t* d_countsB, const int32_t* d_sourcesB,
                             uint64_t nEB, int direction, int with_containment, rs_pairset* ps, void* stream,
                             cudaEvent_t edges_a_ready, cudaEvent_t edges_b_ready,
                             const long long* indexA = nullptr, const long long* indexB = nullptr) {
    if (!A || !B || !ps || direction < 0 || direction > 2) return RS_ERR_INVALID;
    const bool a2b = direction == 0 || direction == 1;
    const bool b2a = direction == 0 || direction == 2;
    cudaStream_t s = (cudaStream_t)stream;
    // Payloads in pinned host memory are read in place through their mapped addresses.
    if (!kernel_ptr(&d_startsA) || !kernel_ptr(&d_endsA) || !kernel_ptr(&d_offsetsA) || !kernel_ptr(&d_countsA) ||
        !kernel_ptr(&d_sourcesA) || !kernel_ptr(&d_startsB) || !kernel_ptr(&d_endsB) || !kernel_ptr(&d_offsetsB) ||
        !kernel_ptr(&d_countsB) || !kernel_ptr(&d_sourcesB) || !kernel_ptr(&indexA) || !kernel_ptr(&indexB))
        return RS_ERR_INVALID;
    {
        int st = bvh_ready(A);  // the broad phase needs the object counts
        if (st == RS_OK) st = bvh_ready(B);
        if (st == RS_OK) st = bvh_use(A, s);
        if (st == RS_OK) st = bvh_use(B, s);
        if (st != RS_OK) return st;
    }
    // Broad phase once per call (it does not depend on the table, so reruns after growth
    // reuse it): object boxes of each set against the other set's triangle boxes, listing
    // each object's partner objects, so that only edges whose own box reaches a partner's
    // box are traced.
    uint8_t* cand = nullptr;    // [A objects | B objects]
    int32_t* part = nullptr;    // kPartners per object, same order
    uint32_t* entry = nullptr;  // entry node per object, same order
    const int* boxes[2] = {nullptr, nullptr};
    int* tmps[2] = {nullptr, nullptr};
    EdgeCull cullA, cullB;
    if (g_overlap_cull && A->n_obj && B->n_obj && A->n_tris && B->n_tris) {
        const uint64_t n_obj = A->n_obj + B->n_obj;
        // One allocation: the partner lists, the entry nodes, then the flags.
        cudaError_t e = dmalloc((void**)&part, n_obj * (kPartners + 1) * sizeof(int32_t) + n_obj, s);
        if (e == cudaSuccess) {
            entry = reinterpret_cast<uint32_t*>(part + n_obj * kPartners);
            cand = reinterpret_cast<uint8_t*>(entry + n_obj);
        }
        if (e == cudaSuccess)
            e = cull_impl(A, B, a2b ? cand : nullptr, b2a ? cand + A->n_obj : nullptr, part,
                          part + A->n_obj * kPartners, entry, entry + A->n_obj, boxes, tmps, s);
        if (e == cudaSuccess) {
            if (a2b) cullA = EdgeCull{cand, A->n_obj, part, boxes[1], B->n_obj, entry, indexA, boxes[0]};
            if (b2a)
                cullB = EdgeCull{cand + A->n_obj, B->n_obj, part + A->n_obj * kPartners, boxes[0], A->n_obj,
                                 entry + A->n_obj, indexB, boxes[1]};
        } else {
            cudaGetLastError();  // culling is an optimisation: run without it
        }
    }
    auto release = [&]() {
        if (part) cudaFreeAsync(part, s);
        for (int* p : tmps)
            if (p) cudaFreeAsync(p, s);
    };
    for (int attempt = 0; attempt < 8; ++attempt) {
        // Order of executeHashQuery (raytracer_intersection_estimated_main.cpp:107-158): overlap A->B,
        // overlap B->A, containment A->B, containment B->A.  The two edge directions are queued
        // back to back and checked with one status read.
        ps->known_count = -1;
        cudaError_t e = cudaMemsetAsync(ps->slots, 0xff, ps->capacity * sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ps->meta, 0, kMetaWords * sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = over_clear(ps, s);
        // Both directions with their broad phase and no events: one live-edge launch for both,
        // and the two directions' rays concurrently.  Otherwise each direction reads its
        // source edges only after the caller's event for them.
        const bool together = a2b && b2a && !edges_a_ready && !edges_b_ready && cullA.cand && cullB.cand &&
                              nEA <= 0xffffffffull && nEB <= 0xffffffffull;
        if (e == cudaSuccess && together) {
            e = edge_join_pair_async(A, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, cullA, B, d_startsB,
                                     d_endsB, d_offsetsB, d_countsB, d_sourcesB, nEB, cullB, ps, s);
        } else {
            if (e == cudaSuccess && a2b && edges_a_ready) e = cudaStreamWaitEvent(s, edges_a_ready, 0);
            if (e == cudaSuccess && a2b)
                e = edge_join_async(B, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, 0, ps, s, cullA);
            if (e == cudaSuccess && b2a && edges_b_ready) e = cudaStreamWaitEvent(s, edges_b_ready, 0);
            if (e == cudaSuccess && b2a)
                e = edge_join_async(A, d_startsB, d_endsB, d_offsetsB, d_countsB, d_sourcesB, nEB, 1, ps, s, cullB);
        }
        int st = table_status(ps, s, e);
        if (with_containment) {
            if (st == RS_OK && a2b) st = rs_containment(B, A->V, A->nV, A->I, A->nF, A->t2o, 0, ps, stream);
            if (st == RS_OK && b2a) st = rs_containment(A, B->V, B->nV, B->I, B->nF, B->t2o, 1, ps, stream);
        }
        if (st != RS_ERR_TABLE_FULL) {
            release();
            return st;
        }
        // Grow and rerun: the table keeps the hashing variant, with four times the slots.
        uint64_t cap = ps->capacity * 4;
        if (!ps->pow2 && cap % 2 == 0) cap += 1;
        if (cap > (1ull << 34)) break;
        e = alloc_slots(ps, cap, s);
        if (e != cudaSuccess) {
            release();
            return to_status(e);
        }
    }
    release();
    return RS_ERR_TABLE_FULL;
}

extern "C" int rs_overlap_join(const rs_bvh* A, const float* d_startsA, const float* d_endsA,
                               const int32_t* d_offsetsA, const int32_t* d_countsA, const int32_t* d_sourcesA,
                               uint64_t nEA, const rs_bvh* B, const float* d_startsB, const float* d_endsB,
                               const int32_t* d_offsetsB, const int32_t* d_countsB, const int32_t* d_sourcesB,
                               uint64_t nEB, int direction, int with_containment, rs_pairset* ps, void* stream) {
    return overlap_join_impl(A, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, B, d_startsB, d_endsB,
                             d_offsetsB, d_countsB, d_sourcesB, nEB, direction, with_containment, ps, stream, nullptr,
                             nullptr);
}

extern "C" int rs_overlap_join_after(const rs_bvh* A, const float* d_startsA, const float* d_endsA,
                                     const int32_t* d_offsetsA, const int32_t* d_countsA, const int32_t* d_sourcesA,
                                     uint64_t nEA, const rs_bvh* B, const float* d_startsB, const float* d_endsB,
                                     const int32_t* d_offsetsB, const int32_t* d_countsB,
                                     const int32_t* d_sourcesB, uint64_t nEB, int direction, int with_containment,
                                     rs_pairset* ps, void* edges_a_ready, void* edges_b_ready, void* stream) {
    return overlap_join_impl(A, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, B, d_startsB, d_endsB,
                             d_offsetsB, d_countsB, d_sourcesB, nEB, direction, with_containment, ps, stream,
                             (cudaEvent_t)edges_a_ready, (cudaEvent_t)edges_b_ready);
}

extern "C" int rs_overlap_join_indexed(const rs_bvh* A, const float* d_startsA, const float* d_endsA,
                                       const int32_t* d_offsetsA, const int32_t* d_countsA,
                                       const int32_t* d_sourcesA, uint64_t nEA, const int64_t* d_indexA,
                                       const rs_bvh* B, const float* d_startsB, const float* d_endsB,
                                       const int32_t* d_offsetsB, const int32_t* d_countsB,
                                       const int32_t* d_sourcesB, uint64_t nEB, const int64_t* d_indexB,
                                       int direction, int with_containment, rs_pairset* ps, void* edges_a_ready,
                                       void* edges_b_ready, void* stream) {
    return overlap_join_impl(A, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, B, d_startsB, d_endsB,
                             d_offsetsB, d_countsB, d_sourcesB, nEB, direction, with_containment, ps, stream,
                             (cudaEvent_t)edges_a_ready, (cudaEvent_t)edges_b_ready,
                             reinterpret_cast<const long long*>(d_indexA),
                             reinterpret_cast<const long long*>(d_indexB));
}

extern "C" int rs_set_overlap_cull(int on) {
    g_overlap_cull = on != 0;
    return RS_OK;
}

extern "C" int rs_pairset_set_tracking(rs_pairset* ps, int on) {
    if (!ps) return RS_ERR_INVALID;
    ps->track = on != 0;
    return RS_OK;
}

extern "C" int rs_pairset_set_edge_rule(rs_pairset* ps, int max_hits, int next_float) {
    if (!ps) return RS_ERR_INVALID;
    ps->edge_max_hits = max_hits > 0 ? max_hits : 100;  // mesh_intersection.cu:25-28
    ps->edge_next_float = next_float != 0;
    ps->known_count = -1;
    return RS_OK;
}

extern "C" int rs_pairset_counters(const rs_pairset* ps, uint64_t* h_out8, void* stream) {
    if (!ps || !h_out8) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long m[kMetaWords];
    cudaError_t e = cudaMemcpyAsync(m, ps->meta, sizeof(m), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return to_status(e);
    for (int k = 0; k < 8; ++k) h_out8[k] = m[2 + k];
    return RS_OK;
}

extern "C" const char* rs_status_string(int status) {
    switch (status) {
        case RS_OK: return "ok";
        case RS_ERR_CUDA: return "CUDA runtime error";
        case RS_ERR_INVALID: return "invalid argument";
        case RS_ERR_TABLE_FULL: return "pair table full";
        case RS_ERR_OUTPUT_OVERFLOW: return "output buffer too small";
        case RS_ERR_ITER_LIMIT: return "iteration or stack budget exhausted";
        case RS_ERR_FORMAT: return "malformed input";
        case RS_ERR_OOM: return "out of device memory";
        case RS_ERR_TARGET_OVERFLOW: return "containment ray crossed too many distinct targets";
        case RS_ERR_TOO_LARGE: return "input larger than the entry point's fixed capacity";
        default: return "unknown status";
    }
}

extern "C" const char* rs_version(void) { return "rayspace3d-gb300 0.1 (sm_103a)"; }
