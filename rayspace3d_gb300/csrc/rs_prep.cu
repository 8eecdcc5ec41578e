// rs_prep.cu -- the query path's input preparation on the GPU: the unique-edge payload of
// EdgePreprocessor::extractEdges (preprocess/src/EdgePreprocessor.cpp:41-119), byte for
// byte.
//
// Every edge of every valid triangle (triangle order; edges v0v1, v1v2, v2v0) is a record
// r = 3 t + e.  Its key is the ordered pair (k0 <= k1) of its endpoints quantised with
// llround(double(x) * 1e5), and the reference's std::map orders keys lexicographically.
// Here the six quantised coordinates are offset by their per-axis minimum and packed, most
// significant first, into one wide integer of just the bits the data needs, with a top bit
// that sends records of skipped triangles last.  A stable LSD radix sort over its 64-bit
// words, started from record order, sorts the records by (key, record).  Each run of equal
// keys is one unique edge: its first record gives the endpoints in that record's own
// orientation, and a second stable sort by (run, object) marks each object's first record
// in the run, so the sources come out deduplicated in first-seen order -- the reference's
// first-occurrence rules.
#include <algorithm>
#include <climits>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kPT = 256;

__device__ __forceinline__ void quantise(const float* __restrict__ V, uint32_t v, long long q[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = llround((double)V[3 * (uint64_t)v + k] * 1e5);
}

__device__ __forceinline__ bool less3(const long long* a, const long long* b) {
    return a[0] < b[0] || (a[0] == b[0] && (a[1] < b[1] || (a[1] == b[1] && a[2] < b[2])));
}

// Key endpoints of record r; false when its triangle has an index >= nV (the reference
// skips such triangles, EdgePreprocessor.cpp:64-66).
__device__ __forceinline__ bool record_key(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                                           uint32_t r, long long k0[3], long long k1[3]) {
    const uint64_t t = r / 3;
    const int e = (int)(r % 3);
    const uint32_t v[3] = {I[3 * t], I[3 * t + 1], I[3 * t + 2]};
    if (v[0] >= nV || v[1] >= nV || v[2] >= nV) return false;
    long long q0[3], q1[3];
    quantise(V, v[e], q0);
    quantise(V, v[e == 2 ? 0 : e + 1], q1);
    const bool sw = less3(q1, q0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        k0[k] = sw ? q1[k] : q0[k];
        k1[k] = sw ? q0[k] : q1[k];
    }
    return true;
}

// Per-axis range of the quantised coordinates over valid records, and their number.
__global__ void k_q_bounds(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t m,
                           long long* __restrict__ b, unsigned long long* __restrict__ n_valid) {
    long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    unsigned long long cnt = 0;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < m; r += (uint64_t)gridDim.x * blockDim.x) {
        long long k0[3], k1[3];
        if (!record_key(V, nV, I, (uint32_t)r, k0, k1)) continue;
        ++cnt;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = min(mn[k], min(k0[k], k1[k]));
            mx[k] = max(mx[k], max(k0[k], k1[k]));
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        atomicMin(&b[k], mn[k]);
        atomicMax(&b[3 + k], mx[k]);
    }
    if (cnt) atomicAdd(n_valid, cnt);
}

// Field layout of the packed key, least significant first:
// k1.z, k1.y, k1.x, k0.z, k0.y, k0.x, skipped-triangle flag.
struct Packing {
    long long mn[3];
    int width[3];
    int total;
};

__device__ __forceinline__ uint64_t packed_word(const float* __restrict__ V, uint64_t nV,
                                                const uint32_t* __restrict__ I, uint32_t r, const Packing& p,
                                                int word) {
    long long k0[3], k1[3];
    const bool ok = record_key(V, nV, I, r, k0, k1);
    const uint64_t f[7] = {ok ? (uint64_t)(k1[2] - p.mn[2]) : 0, ok ? (uint64_t)(k1[1] - p.mn[1]) : 0,
                           ok ? (uint64_t)(k1[0] - p.mn[0]) : 0, ok ? (uint64_t)(k0[2] - p.mn[2]) : 0,
                           ok ? (uint64_t)(k0[1] - p.mn[1]) : 0, ok ? (uint64_t)(k0[0] - p.mn[0]) : 0,
                           ok ? 0ull : 1ull};
    const int w[7] = {p.width[2], p.width[1], p.width[0], p.width[2], p.width[1], p.width[0], 1};
    const int lo = 64 * word, hi = lo + 64;
    uint64_t out = 0;
    int pos = 0;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        const int a = pos, b = pos + w[i];  // the field holds bits [a, b)
        if (w[i] > 0 && b > lo && a < hi) {
            const int s0 = max(a, lo), s1 = min(b, hi);
            const int n = s1 - s0;
            const uint64_t mask = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
            out |= ((f[i] >> (s0 - a)) & mask) << (s0 - lo);
        }
        pos = b;
    }
    return out;
}

__global__ void k_iota(uint32_t* __restrict__ p, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}

// keys[j] = the given word of the packed key of record perm[j].
__global__ void k_word(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                       const uint32_t* __restrict__ perm, uint64_t m, Packing p, int word,
                       uint64_t* __restrict__ keys) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j < m) keys[j] = packed_word(V, nV, I, perm[j], p, word);
}

// head[j] = 1 when sorted record j starts a run of equal keys.
__global__ void k_heads(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                        const uint32_t* __restrict__ perm, uint64_t mv, uint32_t* __restrict__ head) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= mv) return;
    if (j == 0) {
        head[0] = 1;
        return;
    }
    long long a0[3], a1[3], b0[3], b1[3];
    record_key(V, nV, I, perm[j], a0, a1);
    record_key(V, nV, I, perm[j - 1], b0, b1);
    bool same = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) same = same && a0[k] == b0[k] && a1[k] == b1[k];
    head[j] = same ? 0u : 1u;
}

// (run, object) keys of the sorted records; the run of record j is gid[j] + head[j] - 1
// (gid = exclusive scan of the heads).
__global__ void k_run_obj(const int32_t* __restrict__ T, const uint32_t* __restrict__ perm,
                          const uint32_t* __restrict__ head, const uint32_t* __restrict__ gid, uint64_t mv,
                          uint64_t* __restrict__ key2, uint32_t* __restrict__ val2) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= mv) return;
    const uint32_t run = gid[j] + head[j] - 1;
    key2[j] = ((uint64_t)run << 32) | (uint32_t)T[perm[j] / 3];
    val2[j] = (uint32_t)j;
}

// keep[j] = 1 for the first record (in record order) of each (run, object).
__global__ void k_keep(const uint64_t* __restrict__ key2, const uint32_t* __restrict__ val2, uint64_t mv,
                       uint32_t* __restrict__ keep) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= mv) return;
    keep[val2[i]] = (i == 0 || key2[i] != key2[i - 1]) ? 1u : 0u;
}

// The payload: each kept record writes its object at its rank among kept records and
// counts itself in its run; each run's first record (always kept) writes the endpoints in
// its own orientation and the run's offset.
__global__ void k_emit(const float* __restrict__ V, const uint32_t* __restrict__ I, const int32_t* __restrict__ T,
                       const uint32_t* __restrict__ perm, const uint32_t* __restrict__ head,
                       const uint32_t* __restrict__ gid, const uint32_t* __restrict__ keep,
                       const uint32_t* __restrict__ kpos, uint64_t mv, float* __restrict__ starts,
                       float* __restrict__ ends, int32_t* __restrict__ offsets, int32_t* __restrict__ counts,
                       int32_t* __restrict__ sources) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= mv) return;
    const uint32_t r = perm[j];
    const uint32_t run = gid[j] + head[j] - 1;
    if (keep[j]) {
        sources[kpos[j]] = T[r / 3];
        atomicAdd(&counts[run], 1);
    }
    if (!head[j]) return;
    const uint64_t t = r / 3;
    const int e = (int)(r % 3);
    const uint32_t a = I[3 * t + e], b = I[3 * t + (e == 2 ? 0 : e + 1)];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        starts[3 * (uint64_t)run + k] = V[3 * (uint64_t)a + k];
        ends[3 * (uint64_t)run + k] = V[3 * (uint64_t)b + k];
    }
    offsets[run] = (int32_t)kpos[j];
}



}  // namespace
}  // namespace rs

using namespace rs;

extern "C" int rs_extract_edges(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                                const int32_t* d_tri2obj, float* d_starts, float* d_ends, int32_t* d_offsets,
                                int32_t* d_counts, int32_t* d_sources, uint64_t capacity, uint64_t* h_nE,
                                uint64_t* h_nS, void* stream) {
    if (!h_nE || !h_nS) return RS_ERR_INVALID;
    *h_nE = *h_nS = 0;
    if ((nF && (!d_indices || !d_tri2obj)) || (nV && !d_vertices)) return RS_ERR_INVALID;
    const uint64_t m = 3 * nF;
    if (m == 0 || nV == 0) return RS_OK;
    if (m > 0x7fffffffull) return RS_ERR_TOO_LARGE;  // int32 offsets, u32 record ids
    if (!d_starts || !d_ends || !d_offsets || !d_counts || !d_sources) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    long long hb[6];
    unsigned long long hv = 0;
    uint32_t htot[2] = {0, 0};
    {
        Scratch sc{s};
        long long* qb = nullptr;
        uint32_t *perm = nullptr, *head = nullptr, *gid = nullptr, *keep = nullptr, *kpos = nullptr,
                 *val2 = nullptr;
        uint64_t* keys = nullptr;
        e = sc.get(&qb, 8 * sizeof(long long));
        if (e == cudaSuccess) e = sc.get(&perm, m * 4);
        if (e == cudaSuccess) e = sc.get(&keys, m * 8);
        if (e != cudaSuccess) return to_status(e);
        unsigned long long* nvalid = reinterpret_cast<unsigned long long*>(qb + 6);
        const long long init[7] = {LLONG_MAX, LLONG_MAX, LLONG_MAX, LLONG_MIN, LLONG_MIN, LLONG_MIN, 0};
        e = cudaMemcpyAsync(qb, init, sizeof(init), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            launch(k_q_bounds, 4 * sm_count(), kPT, 0, s, d_vertices, nV, d_indices, m, qb, nvalid);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(hb, qb, sizeof(hb), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hv, nvalid, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess || hv == 0) return to_status(e);

        Packing p;
        p.total = 1;
        for (int k = 0; k < 3; ++k) {
            p.mn[k] = hb[k];
            p.width[k] = bits_for((unsigned long long)hb[3 + k] - (unsigned long long)hb[k]);
            p.total += 2 * p.width[k];
        }
        const int nwords = (p.total + 63) / 64;
        const unsigned nb = (unsigned)((m + kPT - 1) / kPT);
        launch(k_iota, nb, kPT, 0, s, perm, m);
        for (int w = 0; w < nwords && e == cudaSuccess; ++w) {
            launch(k_word, nb, kPT, 0, s, d_vertices, nV, d_indices, (const uint32_t*)perm, m, p, w, keys);
            e = radix_sort_u64(keys, perm, m, std::min(64, p.total - 64 * w), s);
        }
        // Valid records sort first (flag bit 0); runs and sources over those alone.
        const uint64_t mv = hv;
        const unsigned nbv = (unsigned)((mv + kPT - 1) / kPT);
        uint32_t* tot = reinterpret_cast<uint32_t*>(qb);
        if (e == cudaSuccess) e = sc.get(&head, mv * 4);
        if (e == cudaSuccess) e = sc.get(&gid, mv * 4);
        if (e == cudaSuccess) e = sc.get(&keep, mv * 4);
        if (e == cudaSuccess) e = sc.get(&kpos, mv * 4);
        if (e == cudaSuccess) e = sc.get(&val2, mv * 4);
        if (e == cudaSuccess) {
            launch(k_heads, nbv, kPT, 0, s, d_vertices, nV, d_indices, (const uint32_t*)perm, mv, head);
            e = exclusive_scan_u32(head, gid, mv, tot, s);
        }
        if (e == cudaSuccess) {
            launch(k_run_obj, nbv, kPT, 0, s, d_tri2obj, (const uint32_t*)perm, (const uint32_t*)head,
                   (const uint32_t*)gid, mv, keys, val2);
            e = radix_sort_u64(keys, val2, mv, 32 + bits_for(mv), s);  // run < mv
        }
        if (e == cudaSuccess) {
            launch(k_keep, nbv, kPT, 0, s, (const uint64_t*)keys, (const uint32_t*)val2, mv, keep);
            e = exclusive_scan_u32(keep, kpos, mv, tot + 1, s);
        }
        uint32_t sort_err = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(htot, tot, 8, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = sort_error_read(&sort_err, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return to_status(e);
        if (sort_err) {
            sort_error_clear(s);
            return RS_ERR_ITER_LIMIT;
        }
        *h_nE = htot[0];
        *h_nS = htot[1];
        if (htot[0] > capacity || htot[1] > capacity) return RS_ERR_OUTPUT_OVERFLOW;
        e = cudaMemsetAsync(d_counts, 0, (size_t)htot[0] * sizeof(int32_t), s);
        if (e == cudaSuccess) {
            launch(k_emit, nbv, kPT, 0, s, d_vertices, d_indices, d_tri2obj, (const uint32_t*)perm,
                   (const uint32_t*)head, (const uint32_t*)gid, (const uint32_t*)keep, (const uint32_t*)kpos, mv,
                   d_starts, d_ends, d_offsets, d_counts, d_sources);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return to_status(e);
}
