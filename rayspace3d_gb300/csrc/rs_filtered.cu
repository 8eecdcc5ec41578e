// rs_filtered.cu -- overlap / intersection join over raw geometry with an object-level
// filter before the builds (no counterpart in the reference, whose launchers build one GAS
// over every triangle of each set: query/src/optix/OptixAccelerationStructure.cpp:22-68,
// query/src/applications/rayspace_mesh_overlap_main.cpp:42-146).
//
// An edge of source object a can only cross a triangle of target object b when a's box and
// b's box overlap (the edge lies in a's box, the triangle in b's box), and a containment ray
// of b can only see an odd crossing count for a when b's first vertex lies in a's box.  So
// the join first computes every object's box, builds a small BVH over one box-diagonal
// triangle per object (its leaf boxes are the object boxes), marks the objects whose
// widened box overlaps a widened box of the other set (the broad phase's own test and
// margins), and builds each set's BVH over the triangles of its marked objects only.  The
// edge rays of marked source objects are then traced as in rs_overlap_join; the pair set
// is the same, and a join of sparse sets builds and traces a small fraction of the data.
#include <algorithm>
#include <climits>
#include <mutex>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
PairTable table_view(rs_pairset* ps);
cudaError_t edge_join_async(const rs_bvh* target, const float* d_starts, const float* d_ends,
                            const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources, uint64_t nE,
                            int swap, rs_pairset* ps, cudaStream_t s, const EdgeCull& cull);
cudaError_t cull_async(const rs_bvh* src, const rs_bvh* other, uint8_t* cand, cudaStream_t s);
cudaError_t alloc_slots(rs_pairset* ps, uint64_t capacity, cudaStream_t s);

namespace {

constexpr int kFT = 256;

__device__ __forceinline__ int f_ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float f_unord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// Largest object id over the triangles (words[0], starts at -1) and an out-of-range index
// flag (words[1]).
__global__ void k_fj_scan(const uint32_t* __restrict__ I, uint64_t nF, uint64_t nV, const int32_t* __restrict__ T,
                          int* __restrict__ words) {
    int mo = -1, bad = 0;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nF; t += (uint64_t)gridDim.x * blockDim.x) {
        mo = max(mo, T[t]);
        bad |= (I[3 * t] >= nV || I[3 * t + 1] >= nV || I[3 * t + 2] >= nV) ? 1 : 0;
    }
    mo = __reduce_max_sync(0xffffffffu, mo);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        if (mo >= 0) atomicMax(&words[0], mo);
        if (bad) atomicOr(&words[1], 1);
    }
}

__global__ void k_fj_box_init(int* __restrict__ box, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < 6 * n) box[i] = (i % 6) < 3 ? f_ord(INFINITY) : f_ord(-INFINITY);
}

// Object boxes (ordered-int min xyz, max xyz) from the triangles; objects outside
// [0, n_obj) are ignored.  The triangles of an object are usually stored together, so the
// lanes of a warp holding the same object reduce first and one of them does the atomics.
__global__ void k_fj_boxes(const float* __restrict__ V, const uint32_t* __restrict__ I, uint64_t nF,
                           const int32_t* __restrict__ T, uint64_t n_obj, int* __restrict__ box) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    const int32_t o = T[t];
    int v[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = V[3 * (uint64_t)I[3 * t] + k], b = V[3 * (uint64_t)I[3 * t + 1] + k],
                    c = V[3 * (uint64_t)I[3 * t + 2] + k];
        v[k] = f_ord(fminf(fminf(a, b), c));
        v[3 + k] = f_ord(fmaxf(fmaxf(a, b), c));
    }
    const unsigned int peers = __match_any_sync(__activemask(), o);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] = __reduce_min_sync(peers, v[k]);
        v[3 + k] = __reduce_max_sync(peers, v[3 + k]);
    }
    if ((int)(threadIdx.x & 31) != __ffs(peers) - 1 || o < 0 || (uint64_t)o >= n_obj) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        atomicMin(&box[6 * (uint64_t)o + k], v[k]);
        atomicMax(&box[6 * (uint64_t)o + 3 + k], v[3 + k]);
    }
}

// Each object's box widened by the broad phase's margins (both of its query and of its
// targets: 1e-4 + 4e-6 * (largest |coordinate| + extent) per axis); an object without
// triangles gets an empty box.
__global__ void k_fj_widen(const int* __restrict__ box, uint64_t n_obj, float* __restrict__ wbox) {
    const uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (o >= n_obj) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float l = f_unord(box[6 * o + k]), h = f_unord(box[6 * o + 3 + k]);
        float wl = INFINITY, wh = -INFINITY;
        if (l <= h) {
            const float m = 1e-4f + 4e-6f * (fmaxf(fabsf(l), fabsf(h)) + (h - l));
            wl = l - m;
            wh = h + m;
        }
        wbox[6 * o + k] = wl;
        wbox[6 * o + 3 + k] = wh;
    }
}

// All pairs of widened boxes, A objects against tiles of B objects in shared memory: both
// objects of an overlapping pair are marked.
constexpr int kPairTile = 1024;
__global__ void __launch_bounds__(kFT) k_fj_pairs(const float* __restrict__ wa, uint64_t na, const float* __restrict__ wb,
                                                 uint64_t nb, uint8_t* __restrict__ ca, uint8_t* __restrict__ cb) {
    __shared__ float tile[6][kPairTile];
    const uint64_t a = blockIdx.x * (uint64_t)kFT + threadIdx.x;
    const uint64_t b0 = (uint64_t)blockIdx.y * kPairTile;
    const int nt = (int)min((uint64_t)kPairTile, nb - b0);
    for (int i = threadIdx.x; i < nt; i += kFT)
#pragma unroll
        for (int k = 0; k < 6; ++k) tile[k][i] = wb[6 * (b0 + i) + k];
    __syncthreads();
    if (a >= na) return;
    float lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = wa[6 * a + k];
        hi[k] = wa[6 * a + 3 + k];
    }
    if (!(lo[0] <= hi[0])) return;
    bool any = false;
    for (int i = 0; i < nt; ++i) {
        if (tile[0][i] <= hi[0] && tile[3][i] >= lo[0] && tile[1][i] <= hi[1] && tile[4][i] >= lo[1] &&
            tile[2][i] <= hi[2] && tile[5][i] >= lo[2]) {
            any = true;
            cb[b0 + i] = 1;
        }
    }
    if (any) ca[a] = 1;
}

// One box-diagonal triangle (min corner, max corner, min corner) per object with
// triangles, appended at an atomic slot (the order does not matter: the box BVH only
// answers box-overlap queries).
__global__ void k_fj_box_tris(const int* __restrict__ box, uint64_t n_obj, float* __restrict__ Vb,
                              uint32_t* __restrict__ Ib, int32_t* __restrict__ Tb, unsigned int* __restrict__ count) {
    const uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (o >= n_obj) return;
    const float lo0 = f_unord(box[6 * o]);
    if (!(lo0 <= f_unord(box[6 * o + 3]))) return;  // no triangle
    const unsigned int j = atomicAdd(count, 1u);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        Vb[6 * (uint64_t)j + k] = f_unord(box[6 * o + k]);
        Vb[6 * (uint64_t)j + 3 + k] = f_unord(box[6 * o + 3 + k]);
    }
    Ib[3 * (uint64_t)j] = 2 * j;
    Ib[3 * (uint64_t)j + 1] = 2 * j + 1;
    Ib[3 * (uint64_t)j + 2] = 2 * j;
    Tb[j] = (int32_t)o;
}

__global__ void k_fj_flags(const int32_t* __restrict__ T, uint64_t nF, const uint8_t* __restrict__ cand, uint64_t n_obj,
                           uint32_t* __restrict__ flag) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    const int32_t o = T[t];
    flag[t] = (o >= 0 && (uint64_t)o < n_obj && cand[o]) ? 1u : 0u;
}

// Ordered compaction of the marked triangles (index triple and object id).
__global__ void k_fj_gather(const uint32_t* __restrict__ I, const int32_t* __restrict__ T, uint64_t nF,
                            const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                            uint32_t* __restrict__ Is, int32_t* __restrict__ Ts) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF || !flag[t]) return;
    const uint32_t j = pos[t];
    Is[3 * (uint64_t)j] = I[3 * t];
    Is[3 * (uint64_t)j + 1] = I[3 * t + 1];
    Is[3 * (uint64_t)j + 2] = I[3 * t + 2];
    Ts[j] = T[t];
}

struct Set {
    const float* V;
    uint64_t nV;
    const uint32_t* I;
    uint64_t nF;
    const int32_t* T;
    uint64_t n_obj = 0;
    int* box = nullptr;      // ordered-int object boxes
    float* wbox = nullptr;   // widened object boxes
    uint8_t* cand = nullptr; // marks
    // box BVH (many objects): one box-diagonal triangle per object
    float* Vb = nullptr;
    uint32_t* Ib = nullptr;
    int32_t* Tb = nullptr;
    rs_bvh* box_bvh = nullptr;
    // the marked objects' triangles and their BVH
    uint32_t* flag = nullptr;
    uint32_t* pos = nullptr;
    uint32_t* Is = nullptr;
    int32_t* Ts = nullptr;
    uint64_t ns = 0;
    rs_bvh* bvh = nullptr;
};

void release(Set& x, cudaStream_t s) {
    if (x.box_bvh) rs_bvh_destroy(x.box_bvh);
    if (x.bvh) rs_bvh_destroy(x.bvh);
    for (void* p : {(void*)x.box, (void*)x.wbox, (void*)x.cand, (void*)x.Vb, (void*)x.Ib, (void*)x.Tb, (void*)x.flag,
                    (void*)x.pos, (void*)x.Is, (void*)x.Ts})
        if (p) cudaFreeAsync(p, s);
    x = Set{x.V, x.nV, x.I, x.nF, x.T};
}

// Above this many object pairs the marks come from a BVH over the object boxes instead of
// the all-pairs kernel.
constexpr uint64_t kPairLimit = 1ull << 32;

// Marks through box BVHs: one box-diagonal triangle per object (its triangle box is the
// object box), then the broad phase's per-object query of each set against the other's.
cudaError_t marks_by_bvh(Set& A, Set& B, cudaStream_t s) {
    unsigned int* cnt = nullptr;
    unsigned int hc[2] = {0, 0};
    cudaError_t e = dmalloc((void**)&cnt, 2 * sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned int), s);
    Set* sets[2] = {&A, &B};
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        Set& x = *sets[i];
        e = dmalloc((void**)&x.Vb, 6 * x.n_obj * sizeof(float), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.Ib, 3 * x.n_obj * sizeof(uint32_t), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.Tb, x.n_obj * sizeof(int32_t), s);
        if (e == cudaSuccess)
            launch(k_fj_box_tris, (unsigned)((x.n_obj + kFT - 1) / kFT), kFT, 0, s, (const int*)x.box, x.n_obj, x.Vb,
                   x.Ib, x.Tb, cnt + i);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (cnt) cudaFreeAsync(cnt, s);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < 2; ++i) {
        Set& x = *sets[i];
        if (rs_bvh_build_async(x.Vb, 2 * (uint64_t)hc[i], x.Ib, hc[i], x.Tb, 0, &x.box_bvh, s) != RS_OK)
            return cudaErrorUnknown;
    }
    if (bvh_ready(A.box_bvh) != RS_OK || bvh_ready(B.box_bvh) != RS_OK) return cudaErrorUnknown;
    if (bvh_use(A.box_bvh, s) != RS_OK || bvh_use(B.box_bvh, s) != RS_OK) return cudaErrorUnknown;
    e = cull_async(A.box_bvh, B.box_bvh, A.cand, s);
    if (e == cudaSuccess) e = cull_async(B.box_bvh, A.box_bvh, B.cand, s);
    return e;
}

// Two streams per device for the builds of the filtered sets.
cudaStream_t side_stream(int which) {
    static cudaStream_t st[64][2] = {};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!st[dev][which] && cudaStreamCreateWithFlags(&st[dev][which], cudaStreamNonBlocking) != cudaSuccess)
        st[dev][which] = nullptr;
    return st[dev][which];
}

}  // namespace
}  // namespace rs

using namespace rs;

extern "C" int rs_overlap_join_filtered(const float* d_VA, uint64_t nVA, const uint32_t* d_IA, uint64_t nFA,
                                        const int32_t* d_TA, const float* d_startsA, const float* d_endsA,
                                        const int32_t* d_offsetsA, const int32_t* d_countsA,
                                        const int32_t* d_sourcesA, uint64_t nEA, const float* d_VB, uint64_t nVB,
                                        const uint32_t* d_IB, uint64_t nFB, const int32_t* d_TB,
                                        const float* d_startsB, const float* d_endsB, const int32_t* d_offsetsB,
                                        const int32_t* d_countsB, const int32_t* d_sourcesB, uint64_t nEB,
                                        int direction, int with_containment, int leaf_size, rs_pairset* ps,
                                        void* stream) {
    if (!ps || direction < 0 || direction > 2) return RS_ERR_INVALID;
    if ((nFA && (!d_VA || !d_IA || !d_TA)) || (nFB && (!d_VB || !d_IB || !d_TB))) return RS_ERR_INVALID;
    if ((nEA && (!d_startsA || !d_endsA || !d_offsetsA || !d_countsA || !d_sourcesA)) ||
        (nEB && (!d_startsB || !d_endsB || !d_offsetsB || !d_countsB || !d_sourcesB)))
        return RS_ERR_INVALID;
    if (nFA >= 0xffffffffull || nFB >= 0xffffffffull) return RS_ERR_TOO_LARGE;
    const bool a2b = direction == 0 || direction == 1;
    const bool b2a = direction == 0 || direction == 2;
    cudaStream_t s = (cudaStream_t)stream;
    Set A{d_VA, nVA, d_IA, nFA, d_TA}, B{d_VB, nVB, d_IB, nFB, d_TB};
    Set* sets[2] = {&A, &B};
    int* words = nullptr;
    cudaEvent_t ev = nullptr;
    auto finish = [&](int st) {
        cudaStreamSynchronize(s);
        if (words) cudaFreeAsync(words, s);
        if (ev) cudaEventDestroy(ev);
        release(A, s);
        release(B, s);
        cudaStreamSynchronize(s);
        return st;
    };
    // 1. Object counts and the index check of both sets (one synchronisation).
    int hw[4] = {-1, 0, -1, 0};
    cudaError_t e = dmalloc((void**)&words, sizeof(hw), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(words, hw, sizeof(hw), cudaMemcpyHostToDevice, s);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        if (sets[i]->nF)
            launch(k_fj_scan, 4 * sm_count(), kFT, 0, s, sets[i]->I, sets[i]->nF, sets[i]->nV, sets[i]->T,
                   words + 2 * i);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hw, words, sizeof(hw), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return finish(to_status(e));
    if (hw[1] || hw[3]) return finish(RS_ERR_INVALID);
    A.n_obj = hw[0] >= 0 ? (uint64_t)hw[0] + 1 : 0;
    B.n_obj = hw[2] >= 0 ? (uint64_t)hw[2] + 1 : 0;
    // 2. Object boxes, widened boxes, marks.
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        Set& x = *sets[i];
        if (!x.n_obj) continue;
        e = dmalloc((void**)&x.box, 6 * x.n_obj * sizeof(int), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.wbox, 6 * x.n_obj * sizeof(float), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.cand, x.n_obj, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(x.cand, 0, x.n_obj, s);
        if (e == cudaSuccess) {
            const unsigned go = (unsigned)((x.n_obj + kFT - 1) / kFT);
            launch(k_fj_box_init, (unsigned)((6 * x.n_obj + kFT - 1) / kFT), kFT, 0, s, x.box, x.n_obj);
            launch(k_fj_boxes, (unsigned)((x.nF + kFT - 1) / kFT), kFT, 0, s, x.V, x.I, x.nF, x.T, x.n_obj, x.box);
            launch(k_fj_widen, go, kFT, 0, s, (const int*)x.box, x.n_obj, x.wbox);
        }
    }
    if (e == cudaSuccess && A.n_obj && B.n_obj) {
        if (A.n_obj * B.n_obj <= kPairLimit && (B.n_obj + kPairTile - 1) / kPairTile <= 65535)
            launch(k_fj_pairs, dim3((unsigned)((A.n_obj + kFT - 1) / kFT), (unsigned)((B.n_obj + kPairTile - 1) / kPairTile)),
                   kFT, 0, s, (const float*)A.wbox, A.n_obj, (const float*)B.wbox, B.n_obj, A.cand, B.cand);
        else
            e = marks_by_bvh(A, B, s);
    }
    if (e != cudaSuccess) return finish(to_status(e));
    // 3. The marked objects' triangles, in order (one synchronisation for both counts).
    uint32_t* tot = reinterpret_cast<uint32_t*>(words);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        Set& x = *sets[i];
        if (!x.nF || !x.cand) continue;
        e = dmalloc((void**)&x.flag, x.nF * sizeof(uint32_t), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.pos, x.nF * sizeof(uint32_t), s);
        if (e == cudaSuccess) {
            launch(k_fj_flags, (unsigned)((x.nF + kFT - 1) / kFT), kFT, 0, s, x.T, x.nF, (const uint8_t*)x.cand,
                   x.n_obj, x.flag);
            e = exclusive_scan_u32(x.flag, x.pos, x.nF, tot + i, s);
        }
    }
    uint32_t ht[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(ht, tot, sizeof(ht), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return finish(to_status(e));
    for (int i = 0; i < 2; ++i) sets[i]->ns = (sets[i]->nF && sets[i]->cand) ? ht[i] : 0;
    // 4. Gather and build both BVHs concurrently on the two side streams.
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        Set& x = *sets[i];
        if (!x.ns) continue;
        e = dmalloc((void**)&x.Is, 3 * x.ns * sizeof(uint32_t), s);
        if (e == cudaSuccess) e = dmalloc((void**)&x.Ts, x.ns * sizeof(int32_t), s);
        if (e == cudaSuccess)
            launch(k_fj_gather, (unsigned)((x.nF + kFT - 1) / kFT), kFT, 0, s, x.I, x.T, x.nF, (const uint32_t*)x.flag,
                   (const uint32_t*)x.pos, x.Is, x.Ts);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev, s);
    if (e != cudaSuccess) return finish(to_status(e));
    for (int i = 0; i < 2; ++i) {
        Set& x = *sets[i];
        cudaStream_t bs = side_stream(i);
        if (!bs) bs = s;
        if (bs != s && cudaStreamWaitEvent(bs, ev, 0) != cudaSuccess) return finish(RS_ERR_CUDA);
        const int st = rs_bvh_build_async(x.V, x.nV, x.Is, x.ns, x.Ts, leaf_size, &x.bvh, bs);
        if (st != RS_OK) return finish(st);
    }
    int st = bvh_use(A.bvh, s);
    if (st == RS_OK) st = bvh_use(B.bvh, s);
    if (st != RS_OK) return finish(st);
    // 5. The join over the filtered BVHs, with the table growth of rs_overlap_join.
    const EdgeCull cullA{A.cand, A.n_obj}, cullB{B.cand, B.n_obj};
    for (int attempt = 0; attempt < 8; ++attempt) {
        ps->known_count = -1;
        e = cudaMemsetAsync(ps->slots, 0xff, ps->capacity * sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ps->meta, 0, kMetaWords * sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = over_clear(ps, s);
        if (e == cudaSuccess && a2b && A.cand)
            e = edge_join_async(B.bvh, d_startsA, d_endsA, d_offsetsA, d_countsA, d_sourcesA, nEA, 0, ps, s, cullA);
        if (e == cudaSuccess && b2a && B.cand)
            e = edge_join_async(A.bvh, d_startsB, d_endsB, d_offsetsB, d_countsB, d_sourcesB, nEB, 1, ps, s, cullB);
        st = table_status(ps, s, e);
        if (with_containment) {
            if (st == RS_OK && a2b) st = rs_containment(B.bvh, d_VA, nVA, d_IA, nFA, d_TA, 0, ps, stream);
            if (st == RS_OK && b2a) st = rs_containment(A.bvh, d_VB, nVB, d_IB, nFB, d_TB, 1, ps, stream);
        }
        if (st != RS_ERR_TABLE_FULL) return finish(st);
        // Grow and rerun: the table keeps the hashing variant, with four times the slots.
        uint64_t cap = ps->capacity * 4;
        if (!ps->pow2 && cap % 2 == 0) cap += 1;
        if (cap > (1ull << 34)) break;
        const cudaError_t ge = alloc_slots(ps, cap, s);
        if (ge != cudaSuccess) return finish(to_status(ge));
    }
    return finish(RS_ERR_TABLE_FULL);
}
