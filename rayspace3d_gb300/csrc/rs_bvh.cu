// rs_bvh.cu -- Morton-code LBVH builder.
//
// Replaces OptixAccelerationStructure::buildInternal
// (query/src/optix/OptixAccelerationStructure.cpp:22-68), which builds one
// triangle GAS over every triangle of a .pre set.  Steps:
//   1. bounds of all vertices;
//   2. keys = 32-bit Morton code of each triangle box's centre (11/11/10 bits, in the
//      vertex bounds) << 32 | triangle id, unique by construction;
//   3. stable radix sort of the 32 Morton bits only (4 passes; ids stay ascending
//      within equal codes);
//   4. groups of leaf_size / 2 consecutive sorted triangles; k_build_tree writes the
//      triangles in leaf order (3 x float4 each) and, per block of 256 groups, every
//      subtree of the binary radix tree over the groups' keys that lies in the block,
//      each from shared-memory range tables (64-byte nodes; subtrees of <= leaf_size
//      triangles become leaves);
//   5. k_build_cross joins the subtrees left open across blocks.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>


#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ int flt_ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord_flt(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// The build's scratch words, in one launch: bounds[0..2] = min (ordered ints), [3..5] =
// max, [6..11] the same for vertices, [12] the error flags = 0, [13] the largest object id
// = -1; the open-subtree count = 0; every cross-block exchange word = -1.
__global__ void k_build_init(int* __restrict__ b, unsigned int* __restrict__ n_open, int* __restrict__ xchg,
                             uint64_t n_xchg) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < 12) b[i] = (i % 6) < 3 ? 0x7fffffff : (int)0x80000000;
    if (i == 12) b[12] = 0;
    if (i == 13) b[13] = -1;
    if (i == 14 && n_open) *n_open = 0;
    for (uint64_t k = i; k < n_xchg; k += (uint64_t)gridDim.x * blockDim.x) xchg[k] = -1;
}

// Block-wide min/max of the three components (and the largest object id), then one atomic
// per value and block: same-address atomics from every warp of the grid would serialise in
// one L2 slice.  Called by every thread of the block.
__device__ __forceinline__ void block_minmax_atomic(float mn[3], float mx[3], int mo, int* out, int* max_obj) {
    __shared__ int s_v[32][7];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int v[7];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] = __reduce_min_sync(0xffffffffu, flt_ord(mn[k]));
        v[3 + k] = __reduce_max_sync(0xffffffffu, flt_ord(mx[k]));
    }
    v[6] = __reduce_max_sync(0xffffffffu, mo);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 7; ++k) s_v[w][k] = v[k];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const int x = lane < nw ? s_v[lane][k] : s_v[0][k];
            v[k] = (k < 3) ? __reduce_min_sync(0xffffffffu, x) : __reduce_max_sync(0xffffffffu, x);
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                atomicMin(&out[k], v[k]);
                atomicMax(&out[3 + k], v[3 + k]);
            }
            if (v[6] >= 0) atomicMax(max_obj, v[6]);
        }
    }
}

// Bounds of all vertices (bounds[6..11]) and the largest object id (max_obj), grid-stride
// with one atomic per warp.  The xyz array is read as float4 when it is 16-byte aligned:
// float f of the flat array is component f % 3, and float4 q starts at component q % 3.
__device__ __forceinline__ void fold_component(float mn[3], float mx[3], int c, float v) {
    // c is 0, 1 or 2; selects keep the three accumulators in registers.
    mn[0] = c == 0 ? fminf(mn[0], v) : mn[0];
    mx[0] = c == 0 ? fmaxf(mx[0], v) : mx[0];
    mn[1] = c == 1 ? fminf(mn[1], v) : mn[1];
    mx[1] = c == 1 ? fmaxf(mx[1], v) : mx[1];
    mn[2] = c == 2 ? fminf(mn[2], v) : mn[2];
    mx[2] = c == 2 ? fmaxf(mx[2], v) : mx[2];
}

__global__ void k_vertex_bounds(const float* __restrict__ V, uint64_t nV, const int32_t* __restrict__ t2o,
                                uint64_t nF, int* bounds, int* max_obj) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t nf = 3 * nV;
    uint64_t done = 0;
    // Four independent loads in flight per thread and iteration; the component of float4
    // q is q % 3, advanced incrementally (4 = 1 mod 3).
    constexpr int U = 4;
    if ((reinterpret_cast<uintptr_t>(V) & 15u) == 0) {
        const float4* V4 = reinterpret_cast<const float4*>(V);
        const uint64_t n4 = nf / 4;
        const int s3 = (int)(stride % 3), step3 = (int)((U * stride) % 3);
        int c0 = (int)(tid % 3);
        for (uint64_t q0 = tid; q0 < n4; q0 += U * stride) {
            float4 v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t q = q0 + u * stride;
                v[u] = q < n4 ? __ldg(&V4[q]) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            int c = c0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (q0 + u * stride < n4) {
                    fold_component(mn, mx, c, v[u].x);
                    fold_component(mn, mx, c == 2 ? 0 : c + 1, v[u].y);
                    fold_component(mn, mx, c == 0 ? 2 : c - 1, v[u].z);
                    fold_component(mn, mx, c, v[u].w);
                }
                c += s3;
                c = c >= 3 ? c - 3 : c;
            }
            c0 += step3;
            c0 = c0 >= 3 ? c0 - 3 : c0;
        }
        done = 4 * n4;
    }
    for (uint64_t f = done + tid; f < nf; f += stride) fold_component(mn, mx, (int)(f % 3), V[f]);
    int mo = -1;
    if ((reinterpret_cast<uintptr_t>(t2o) & 15u) == 0) {
        const int4* T4 = reinterpret_cast<const int4*>(t2o);
        const uint64_t n4 = nF / 4;
        for (uint64_t q0 = tid; q0 < n4; q0 += U * stride) {
            int4 t[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t q = q0 + u * stride;
                t[u] = q < n4 ? __ldg(&T4[q]) : make_int4(-1, -1, -1, -1);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) mo = max(max(mo, max(t[u].x, t[u].y)), max(t[u].z, t[u].w));
        }
        for (uint64_t q = 4 * n4 + tid; q < nF; q += stride) mo = max(mo, t2o[q]);
    } else {
        for (uint64_t q = tid; q < nF; q += stride) mo = max(mo, t2o[q]);
    }
    block_minmax_atomic(mn, mx, mo, bounds + 6, max_obj);
}

// Indices are clamped so a malformed index buffer cannot read out of bounds; the
// build reports RS_ERR_INVALID for such input after the fact.
__device__ __forceinline__ void tri_box(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                                        uint64_t t, float lo[3], float hi[3]) {
    const uint64_t last = nV - 1;
    const uint64_t i0 = min((uint64_t)I[3 * t], last), i1 = min((uint64_t)I[3 * t + 1], last),
                   i2 = min((uint64_t)I[3 * t + 2], last);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = V[3 * (uint64_t)i0 + k], b = V[3 * (uint64_t)i1 + k], c = V[3 * (uint64_t)i2 + k];
        lo[k] = fminf(fminf(a, b), c);
        hi[k] = fmaxf(fmaxf(a, b), c);
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Keys of the triangles: the Morton code of the box centre quantised in the bounds of
// all vertices, << 32 | triangle id.  Also flags out-of-range vertex indices.
// Object boxes of the objects below min(largest id + 1, cap) set to empty (min +inf, max
// -inf as ordered ints); the largest id comes from k_vertex_bounds.
__global__ void k_obox_init(int* __restrict__ box, uint64_t cap, const int* __restrict__ max_obj) {
    const uint64_t n = min((uint64_t)(max(*max_obj, -1) + 1), cap);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < 6 * n; i += (uint64_t)gridDim.x * blockDim.x)
        box[i] = (i % 6) < 3 ? 0x7fffffff : (int)0x80000000;
}

// Morton key of each triangle's box centre (and, into obox, the box of each object below
// obox_cap: triangles of one object are usually stored together, so the lanes of a warp
// with equal objects reduce first and one of them does the atomics).
// Grid-stride over the triangles; also counts the four 8-bit digits of each Morton code
// (the sort's histogram, hist[p * 256 + digit p]) in shared memory, added to `hist` once
// per block, so the sort does not read the keys back for them.
__global__ void __launch_bounds__(kT) k_morton(const float* __restrict__ V, uint64_t nV,
                                              const uint32_t* __restrict__ I, uint64_t nF,
                                              const int32_t* __restrict__ T, const int* __restrict__ bounds,
                                              uint64_t* __restrict__ keys, unsigned int* __restrict__ bad_index,
                                              int* __restrict__ obox, uint64_t obox_cap,
                                              uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_hist[4 * 256];
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x) s_hist[k] = 0;
    __syncthreads();
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nF; t += (uint64_t)gridDim.x * blockDim.x) {
        if (I[3 * t] >= nV || I[3 * t + 1] >= nV || I[3 * t + 2] >= nV) atomicOr(bad_index, 1u);
        float lo[3], hi[3];
        tri_box(V, nV, I, t, lo, hi);
        if (obox) {
            const int32_t o = T[t];
            int v[6] = {flt_ord(lo[0]), flt_ord(lo[1]), flt_ord(lo[2]), flt_ord(hi[0]), flt_ord(hi[1]), flt_ord(hi[2])};
            const unsigned int peers = __match_any_sync(__activemask(), o);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                v[k] = __reduce_min_sync(peers, v[k]);
                v[3 + k] = __reduce_max_sync(peers, v[3 + k]);
            }
            if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && o >= 0 && (uint64_t)o < obox_cap) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    atomicMin(&obox[6 * (uint64_t)o + k], v[k]);
                    atomicMax(&obox[6 * (uint64_t)o + 3 + k], v[3 + k]);
                }
            }
        }
        uint32_t q[3];
        const float scale[3] = {2048.0f, 2048.0f, 1024.0f};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float cmin = ord_flt(bounds[6 + k]), cmax = ord_flt(bounds[9 + k]);
            const float ext = cmax - cmin;
            const float c = 0.5f * lo[k] + 0.5f * hi[k];
            float u = ext > 0.0f ? (c - cmin) / ext : 0.0f;
            u = fminf(fmaxf(u, 0.0f), 1.0f);
            q[k] = (uint32_t)fminf(u * scale[k], scale[k] - 1.0f);
        }
        const uint32_t code = ((q[0] >> 10) << 31) | ((q[1] >> 10) << 30) | (spread10(q[0]) << 2) |
                              (spread10(q[1]) << 1) | spread10(q[2]);
        keys[t] = ((uint64_t)code << 32) | (uint32_t)t;
#pragma unroll
        for (int p = 0; p < 4; ++p) atomicAdd(&s_hist[p * 256 + ((code >> (8 * p)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x)
        if (s_hist[k]) atomicAdd(&hist[k], s_hist[k]);
}

// Length of the common prefix of the keys of groups g and g+1 (the keys of their first
// triangles, distinct by construction).
__device__ __forceinline__ int group_prefix(const uint64_t* __restrict__ keys, int g, int L) {
    return __clzll((long long)(__ldg(&keys[(size_t)g * L]) ^ __ldg(&keys[(size_t)(g + 1) * L])));
}

__device__ __forceinline__ int exchange_acq_rel(int* p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// A node slot holds its two children: side 0 in a.xyzw b.xy (box) and d.xy (entry),
// side 1 in b.zw c.xyzw and d.zw.  The two sides occupy disjoint bytes, so the two
// children of a node can write their halves concurrently.
__device__ __forceinline__ void store_half(BNode* nd, int side, const float lo[3], const float hi[3], int idx,
                                           int cnt) {
    char* b = reinterpret_cast<char*>(nd);
    if (side == 0) {
        *reinterpret_cast<float4*>(b) = make_float4(lo[0], lo[1], lo[2], hi[0]);
        *reinterpret_cast<float2*>(b + 16) = make_float2(hi[1], hi[2]);
        *reinterpret_cast<int2*>(b + 48) = make_int2(idx, cnt);
    } else {
        *reinterpret_cast<float2*>(b + 24) = make_float2(lo[0], lo[1]);
        *reinterpret_cast<float4*>(b + 32) = make_float4(lo[2], hi[0], hi[1], hi[2]);
        *reinterpret_cast<int2*>(b + 56) = make_int2(idx, cnt);
    }
}

__device__ __forceinline__ void load_half(const BNode* nd, int side, float lo[3], float hi[3]) {
    const char* b = reinterpret_cast<const char*>(nd);
    if (side == 0) {
        const float4 a = __ldcg(reinterpret_cast<const float4*>(b));
        const float2 c = __ldcg(reinterpret_cast<const float2*>(b + 16));
        lo[0] = a.x, lo[1] = a.y, lo[2] = a.z, hi[0] = a.w, hi[1] = c.x, hi[2] = c.y;
    } else {
        const float2 a = __ldcg(reinterpret_cast<const float2*>(b + 24));
        const float4 c = __ldcg(reinterpret_cast<const float4*>(b + 32));
        lo[0] = a.x, lo[1] = a.y, lo[2] = c.x, hi[0] = c.y, hi[1] = c.z, hi[2] = c.w;
    }
}

__device__ __forceinline__ void store_node(BNode* nd, const float lo0[3], const float hi0[3], int i0, int c0,
                                           const float lo1[3], const float hi1[3], int i1, int c1) {
    nd->a = make_float4(lo0[0], lo0[1], lo0[2], hi0[0]);
    nd->b = make_float4(hi0[1], hi0[2], lo1[0], lo1[1]);
    nd->c = make_float4(lo1[2], hi1[0], hi1[1], hi1[2]);
    nd->d = make_int4(i0, c0, i1, c1);
}

// Leaf groups of L consecutive sorted triangles.  The entry of the child subtree over
// groups [a, b] with node slot `slot`: a subtree of at most `leaf` triangles is a leaf
// (first triangle, count), a larger one an inner node (slot, 0).
struct Groups {
    int n, L, leaf;
    __device__ __forceinline__ int tris(int a, int b) const { return min(n, (b + 1) * L) - a * L; }
    __device__ __forceinline__ int idx(int a, int b, int slot) const { return tris(a, b) <= leaf ? a * L : slot; }
    __device__ __forceinline__ int cnt(int a, int b) const {
        const int c = tris(a, b);
        return c <= leaf ? c : 0;
    }
};

// A subtree left open by k_build_tree: box, group range, node slot.
struct OpenTree {
    float lo[3], hi[3];
    int l, r, self;
};

// Bottom-up-free construction of the radix tree over the leaf groups of one block of kTB
// groups (the tree Karras' top-down construction gives: Karras 2012, "Maximizing
// Parallelism in the Construction of BVHs, Octrees, and k-d Trees"), fused with the
// emission of the leaf-ordered triangles.  Split p (between groups p and p+1) has the
// prefix length d(p) of their keys; the subtree of split p covers the groups [l, r]
// bounded by the nearest splits on either side with a smaller d (the prefix length
// strictly decreases at a subtree's boundary, and its minimum inside is unique).  A
// subtree [l, r] is the left child of split r when d(r) > d(l-1), else the right child of
// split l-1 (Apetrei 2014).  So every subtree -- the thread's own leaf group and its own
// split -- finds its range, its parent and its box by itself: ranges by binary lifting
// over a shared-memory sparse table of the block's d values (min over 2^k consecutive
// splits), boxes by a query of a shared-memory pyramid of the groups' boxes (aligned
// unions of 2^k groups).  It then writes its box and entry into its half of its parent's
// slot (a parent of <= leaf triangles becomes a leaf of its own parent and gets no slot;
// the root's children write slot 0).  No merge rounds: ten barriers per block in all.
// A subtree whose parent's range leaves the block is handed to k_build_cross; a subtree
// whose own range leaves the block is built there.  Node slot p+1 holds split p.
constexpr int kTB = 256;   // groups per block
constexpr int kLogTB = 8;  // log2(kTB)

// Nearest index j < from (j >= 0) with t[0][j] < v, by binary lifting; -1 when none.
// (A galloping search -- windows of 2^0, 2^1, ... elements, then lifting inside the last
// one -- reads fewer table entries for near boundaries but ran the kernel 10 % slower:
// its data-dependent trip counts diverge where this fixed nine-step loop does not.)
__device__ __forceinline__ int nearest_left(const signed char (*t)[kTB + 1], int from, int v) {
    int pos = from;
#pragma unroll
    for (int lv = kLogTB; lv >= 0; --lv)
        if (pos - (1 << lv) >= 0 && t[lv][pos - (1 << lv)] >= v) pos -= 1 << lv;
    return pos - 1;
}

// Nearest index j > from (j <= kTB) with t[0][j] < v; -1 when none.
__device__ __forceinline__ int nearest_right(const signed char (*t)[kTB + 1], int from, int v) {
    int pos = from + 1;
#pragma unroll
    for (int lv = kLogTB; lv >= 0; --lv)
        if (pos + (1 << lv) - 1 <= kTB && t[lv][pos] >= v) pos += 1 << lv;
    return pos <= kTB ? pos : -1;
}

__global__ void __launch_bounds__(kTB) k_build_tree(const float* __restrict__ V, uint64_t nV,
                                                    const uint32_t* __restrict__ I, const int32_t* __restrict__ t2o,
                                                    const uint64_t* __restrict__ keys, Groups G, int nG,
                                                    float4* __restrict__ tris, BNode* __restrict__ nodes,
                                                    OpenTree* __restrict__ open, unsigned int* __restrict__ n_open) {
    // s_t[lv][j]: min of d over splits bb-1+j .. bb-1+j+2^lv-1 (-1 where no split exists).
    __shared__ signed char s_t[kLogTB + 1][kTB + 1];
    // Box pyramid: level lv holds kTB >> lv unions of 2^lv groups at offset 2kTB - (2kTB >> lv).
    __shared__ float s_b[6][2 * kTB];
    const int tid = threadIdx.x, lane = tid & 31;
    const int bb = blockIdx.x * kTB;
    const int g = bb + tid;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (g < nG) {
        const int j0 = g * G.L, j1 = min(G.n, j0 + G.L);
        const uint64_t last = nV - 1;
        for (int j = j0; j < j1; ++j) {
            // The low word is a triangle id; the clamp only matters after a failed sort.
            const uint32_t t = min((uint32_t)(__ldg(&keys[j]) & 0xffffffffull), (uint32_t)(G.n - 1));
            const uint64_t i0 = min((uint64_t)I[3 * (uint64_t)t], last),
                           i1 = min((uint64_t)I[3 * (uint64_t)t + 1], last),
                           i2 = min((uint64_t)I[3 * (uint64_t)t + 2], last);
            float a[3], b[3], c[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                a[q] = V[3 * i0 + q];
                b[q] = V[3 * i1 + q];
                c[q] = V[3 * i2 + q];
                lo[q] = fminf(lo[q], fminf(fminf(a[q], b[q]), c[q]));
                hi[q] = fmaxf(hi[q], fmaxf(fmaxf(a[q], b[q]), c[q]));
            }
            tris[3 * (uint64_t)j] = make_float4(a[0], a[1], a[2], __uint_as_float(t));
            tris[3 * (uint64_t)j + 1] = make_float4(b[0], b[1], b[2], __int_as_float(t2o[t]));
            tris[3 * (uint64_t)j + 2] = make_float4(c[0], c[1], c[2], 0.0f);
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        s_b[q][tid] = lo[q];
        s_b[3 + q][tid] = hi[q];
    }
    s_t[0][tid + 1] = (signed char)((g < nG - 1) ? group_prefix(keys, g, G.L) : -1);
    if (tid == 0) s_t[0][0] = (signed char)((bb > 0 && bb - 1 < nG - 1) ? group_prefix(keys, bb - 1, G.L) : -1);
    __syncthreads();
#pragma unroll 1
    for (int lv = 1; lv <= kLogTB; ++lv) {
        const int h = 1 << (lv - 1);
        if (tid + (1 << lv) - 1 <= kTB) s_t[lv][tid] = min(s_t[lv - 1][tid], s_t[lv - 1][tid + h]);
        const int n_lv = kTB >> lv;
        if (tid < n_lv) {
            const int src = 2 * kTB - (2 * kTB >> (lv - 1)), dst = 2 * kTB - (2 * kTB >> lv);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                s_b[q][dst + tid] = fminf(s_b[q][src + 2 * tid], s_b[q][src + 2 * tid + 1]);
                s_b[3 + q][dst + tid] = fmaxf(s_b[3 + q][src + 2 * tid], s_b[3 + q][src + 2 * tid + 1]);
            }
        }
        __syncthreads();
    }
    // The thread's two subtrees: its leaf group (k = 0) and its split (k = 1).
    bool emit[2] = {false, false};
    OpenTree ot[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        int l, r, self = 0;
        float blo[3], bhi[3];
        if (k == 0) {
            if (g >= nG) continue;
            l = r = g;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                blo[q] = lo[q];
                bhi[q] = hi[q];
            }
        } else {
            // Split g exists inside the block (the block's last split leaves the block).
            if (g >= nG - 1 || tid >= kTB - 1) continue;
            const int v = s_t[0][tid + 1];
            const int jl = nearest_left(s_t, tid + 1, v);
            const int jr = nearest_right(s_t, tid + 1, v);
            if (jl < 0 || jr < 0) continue;  // the range leaves the block
            l = bb + jl;
            r = bb - 1 + jr;
            self = g + 1;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                blo[q] = INFINITY;
                bhi[q] = -INFINITY;
            }
            int x = l - bb, y = r - bb + 1, off = 0, n_lv = kTB;
            while (x < y) {
                if (x & 1) {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        blo[q] = fminf(blo[q], s_b[q][off + x]);
                        bhi[q] = fmaxf(bhi[q], s_b[3 + q][off + x]);
                    }
                    ++x;
                }
                if (y & 1) {
                    --y;
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        blo[q] = fminf(blo[q], s_b[q][off + y]);
                        bhi[q] = fmaxf(bhi[q], s_b[3 + q][off + y]);
                    }
                }
                x >>= 1;
                y >>= 1;
                off += n_lv;
                n_lv >>= 1;
            }
        }
        // The parent: split r (this is its left child) when d(r) > d(l-1), else split l-1.
        const int dl = s_t[0][l - bb], dr = s_t[0][r - bb + 1];
        if (dl < 0 && dr < 0) continue;  // the root: nothing above it
        const bool left = dr > dl;
        int pl, pr, jp;
        bool inside;
        if (left) {
            jp = r - bb + 1;  // index of split r
            pl = l;
            const int j = jp < kTB ? nearest_right(s_t, jp, dr) : -1;
            inside = j >= 0;
            pr = bb - 1 + j;
        } else {
            jp = l - bb;  // index of split l-1
            pr = r;
            const int j = jp > 0 ? nearest_left(s_t, jp, dl) : -1;
            inside = j >= 0;
            pl = bb + j;
        }
        if (!inside) {
            emit[k] = true;
            OpenTree& o = ot[k];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                o.lo[q] = blo[q];
                o.hi[q] = bhi[q];
            }
            o.l = l;
            o.r = r;
            o.self = self;
            continue;
        }
        const bool root = pl == 0 && pr == nG - 1;
        if (!root && G.tris(pl, pr) <= G.leaf) continue;  // the parent is a leaf of its own parent
        const int p = bb - 1 + jp;
        store_half(nodes + (root ? 0 : p + 1), left ? 0 : 1, blo, bhi, G.idx(l, r, self), G.cnt(l, r));
    }
    // Open subtrees are packed densely for k_build_cross.
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, emit[k]);
        if (!m) continue;
        unsigned int slot = 0;
        if (lane == __ffs(m) - 1) slot = atomicAdd(n_open, (unsigned int)__popc(m));
        slot = __shfl_sync(0xffffffffu, slot, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1u));
        if (emit[k]) open[slot] = ot[k];
    }
}

// Cross-block merges, one open subtree per thread: at split p the child writes its box and
// entry into its half of node slot p+1, then exchanges its outer range bound in xchg[p]
// with acquire-release semantics; the first arrival stops, the second reads its sibling's
// half, merges and continues.  Every split therefore sees exactly one merge.
__global__ void __launch_bounds__(kT) k_build_cross(const uint64_t* __restrict__ keys, Groups G, int nG,
                                                    BNode* __restrict__ nodes, int* __restrict__ xchg,
                                                    const OpenTree* __restrict__ open,
                                                    const unsigned int* __restrict__ n_open) {
    const unsigned int count = *n_open;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        float lo[3], hi[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            lo[q] = open[i].lo[q];
            hi[q] = open[i].hi[q];
        }
        int l = open[i].l, r = open[i].r, self = open[i].self;
        for (;;) {
            if (l == 0 && r == nG - 1) {
                const float4* src = reinterpret_cast<const float4*>(nodes + self);
                float4* dst = reinterpret_cast<float4*>(nodes);
#pragma unroll
                for (int q = 0; q < 4; ++q) dst[q] = __ldcg(src + q);
                break;
            }
            const bool left_child =
                (l == 0) ? true : (r == nG - 1) ? false : group_prefix(keys, r, G.L) > group_prefix(keys, l - 1, G.L);
            const int p = left_child ? r : l - 1;
            BNode* nd = nodes + (p + 1);
            store_half(nd, left_child ? 0 : 1, lo, hi, G.idx(l, r, self), G.cnt(l, r));
            const int other = exchange_acq_rel(&xchg[p], left_child ? l : r);
            if (other < 0) break;
            float olo[3], ohi[3];
            load_half(nd, left_child ? 1 : 0, olo, ohi);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                lo[q] = fminf(lo[q], olo[q]);
                hi[q] = fmaxf(hi[q], ohi[q]);
            }
            if (left_child) r = other;
            else l = other;
            self = p + 1;
        }
    }
}

// Root of a set that is one group (1 <= n <= group size): child 0 is the leaf of all n sorted
// triangles, child 1 an empty box that the slab test always rejects.
__global__ void k_one_group_root(const float4* __restrict__ tris, int n, BNode* nodes) {
    const float inf = INFINITY;
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (int j = 0; j < n; ++j)
        for (int v = 0; v < 3; ++v) {
            const float4 p = tris[3 * j + v];
            lo[0] = fminf(lo[0], p.x), lo[1] = fminf(lo[1], p.y), lo[2] = fminf(lo[2], p.z);
            hi[0] = fmaxf(hi[0], p.x), hi[1] = fmaxf(hi[1], p.y), hi[2] = fmaxf(hi[2], p.z);
        }
    BNode nd;
    nd.a = make_float4(lo[0], lo[1], lo[2], hi[0]);
    nd.b = make_float4(hi[1], hi[2], inf, inf);
    nd.c = make_float4(inf, -inf, -inf, -inf);
    nd.d = make_int4(0, n, 0, 0);
    nodes[0] = nd;
}

// Root of an empty set: two empty children.
__global__ void k_empty_root(BNode* nodes) {
    const float inf = INFINITY;
    BNode nd;
    nd.a = make_float4(inf, inf, inf, -inf);
    nd.b = make_float4(-inf, -inf, inf, inf);
    nd.c = make_float4(inf, -inf, -inf, -inf);
    nd.d = make_int4(0, 0, 0, 0);
    nodes[0] = nd;
}

template <class T>
cudaError_t alloc(T** p, size_t count, cudaStream_t s) {
    return dmalloc((void**)p, (count ? count : 1) * sizeof(T), s);
}

}  // namespace

int to_status(cudaError_t e) {
    if (e == cudaSuccess) return RS_OK;
    if (e == cudaErrorMemoryAllocation) return RS_ERR_OOM;
    return RS_ERR_CUDA;
}

int status_from_bits(uint32_t bits) {
    if (bits & ST_STACK_OVERFLOW) return RS_ERR_ITER_LIMIT;
    if (bits & ST_ITER_LIMIT) return RS_ERR_ITER_LIMIT;
    if (bits & ST_TARGET_OVERFLOW) return RS_ERR_TARGET_OVERFLOW;
    if (bits & (ST_TABLE_FULL | ST_SPILLED)) return RS_ERR_TABLE_FULL;  // spilled: not regrown yet
    return RS_OK;
}

}  // namespace rs

using namespace rs;

namespace rs {

std::mutex g_bvh_mu;

// Reads an asynchronous build's result words once the build has finished: vertex bounds,
// object count and the bad-index flag.  Returns the build's status.
int bvh_ready(const rs_bvh* ch) {
    rs_bvh* h = const_cast<rs_bvh*>(ch);
    std::lock_guard<std::mutex> g(g_bvh_mu);
    if (!h->pending) return h->build_status;
    int hb[14];
    cudaError_t e = cudaEventSynchronize(h->done);
    if (e == cudaSuccess) std::memcpy(hb, h->pending, sizeof(hb));
    pinned_slot_release(h->pending);
    h->pending = nullptr;
    if (e != cudaSuccess) {
        h->build_status = to_status(e);
        return h->build_status;
    }
    for (int k = 0; k < 3; ++k) {
        auto dec = [](int i) {
            int b = i >= 0 ? i : i ^ 0x7fffffff;
            float f;
            std::memcpy(&f, &b, 4);
            return f;
        };
        h->vmin[k] = dec(hb[6 + k]);
        h->vmax[k] = dec(hb[9 + k]);
    }
    h->n_obj = hb[13] >= 0 ? (uint64_t)hb[13] + 1 : 0;
    // [12]: bit 0 an index out of range, bit 1 a failed sort (bounded wait ran out).
    h->build_status = (hb[12] & 2) ? RS_ERR_ITER_LIMIT : hb[12] != 0 ? RS_ERR_INVALID : RS_OK;
    return h->build_status;
}

// Orders work queued on stream s after the handle's build.
int bvh_use(const rs_bvh* h, cudaStream_t s) {
    if (h->build_status != RS_OK) return h->build_status;
    if (h->done && cudaStreamWaitEvent(s, h->done, 0) != cudaSuccess) return RS_ERR_CUDA;
    return RS_OK;
}

static void bvh_free(rs_bvh* h) {
    if (h->done) cudaEventSynchronize(h->done);
    pinned_slot_release(h->pending);
    if (h->mem) cudaFree(h->mem);
    for (auto& g : h->cgrid) {
        if (g.start) cudaFree(g.start);
        if (g.list) cudaFree(g.list);
    }
    if (h->done) cudaEventDestroy(h->done);
    delete h;
}

static int build_impl(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                      const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, cudaStream_t s, bool async) {

    if (!out) return RS_ERR_INVALID;
    *out = nullptr;
    if ((nF && (!d_indices || !d_tri2obj || !d_vertices)) || (nV && !d_vertices)) return RS_ERR_INVALID;
    if (nF && nV == 0) return RS_ERR_INVALID;               // every index would be out of range
    if (nF >= (uint64_t)0x7fffffff) return RS_ERR_INVALID;  // node/leaf indices are int32
    // Default 2: the exact triangle test costs more than a node visit, so small leaves
    // trace fastest on dense joins (4 doubles the edge-ray time at selectivity 1e-4).
    if (leaf_size == 0) leaf_size = 2;
    if (leaf_size < 1 || leaf_size > 16) return RS_ERR_INVALID;
    rs_bvh* h = new rs_bvh();
    h->V = d_vertices;
    h->nV = nV;
    h->I = d_indices;
    h->nF = nF;
    h->t2o = d_tri2obj;
    h->leaf_size = leaf_size;
    cudaGetDevice(&h->device);
    const int n = (int)nF;
    cudaError_t e = cudaSuccess;
    int* slot = nullptr;
    const int grid = 4 * sm_count();
    // Leaf groups of half the leaf size: the radix tree over the groups decides which
    // subtrees of <= leaf_size triangles become leaves.
    const int group = std::max(1, leaf_size / 2);
    const int nG = (n + group - 1) / group;
    h->n_nodes = nG >= 2 ? (uint64_t)nG : 1;  // slot 0 = root, slot p+1 = split p
    h->n_tris = (uint64_t)n;
    // Object boxes for the broad phase of the joins, for up to min(nF, 2^24) objects
    // (dense ids: every object has a triangle); more objects, and the joins compute them.
    h->obox_cap = std::min<uint64_t>(nF, 1ull << 24);
    auto a256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    // The handle's arrays in one allocation: nodes | tris | obox.
    const size_t b_nodes = a256(h->n_nodes * sizeof(BNode)), b_tris = a256(3 * (size_t)n * sizeof(float4));
    const size_t b_obox = a256(6 * h->obox_cap * sizeof(int));
    // The build's scratch in another: 256 bytes of words (bounds[14], the open count) |
    // exchange words | keys | open subtrees (at most two per level of the tree -- 64 key
    // bits -- per block of kTB groups, so nG / 2 + kTB bound them) | the sort's scratch.
    const size_t n_xchg = (size_t)std::max(nG - 1, 1);
    const size_t b_xchg = a256(n_xchg * sizeof(int)), b_keys = a256((size_t)n * sizeof(uint64_t));
    const size_t b_open = a256(((size_t)nG / 2 + kTB) * sizeof(OpenTree));
    const size_t b_sort = radix_sort_scratch_bytes((size_t)n, 64, 32, false);
    char* scratch = nullptr;
    int* bounds = nullptr;  // [6..11] vertex bounds (ordered ints), [12] bad-index flag, [13] max object
    unsigned int* n_open = nullptr;
    int* xchg = nullptr;
    uint64_t* keys = nullptr;
    OpenTree* open = nullptr;
    const int ptok = prof_begin(P_BVH_BUILD, s);
    e = dmalloc(&h->mem, b_nodes + (n ? b_tris + b_obox : 0), s);
    if (e == cudaSuccess) e = dmalloc((void**)&scratch, 256 + (n ? b_xchg + b_keys + b_open + b_sort : 0), s);
    if (e != cudaSuccess) goto fail;
    h->nodes = reinterpret_cast<BNode*>(h->mem);
    if (n) {
        h->tris = reinterpret_cast<float4*>(static_cast<char*>(h->mem) + b_nodes);
        h->obox = reinterpret_cast<int*>(static_cast<char*>(h->mem) + b_nodes + b_tris);
    } else {
        h->obox_cap = 0;
    }
    bounds = reinterpret_cast<int*>(scratch);
    n_open = reinterpret_cast<unsigned int*>(scratch + 64);
    if (n) {
        xchg = reinterpret_cast<int*>(scratch + 256);
        keys = reinterpret_cast<uint64_t*>(scratch + 256 + b_xchg);
        open = reinterpret_cast<OpenTree*>(scratch + 256 + b_xchg + b_keys);
    }
    launch(k_build_init, (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n ? n_xchg : 0) / 256 + 1, grid)), 256, 0,
           s, bounds, n_open, xchg, (uint64_t)(n ? n_xchg : 0));
    if (nV || nF) launch(k_vertex_bounds, grid, kT, 0, s, d_vertices, nV, d_tri2obj, nF, bounds, bounds + 13);
    if (n == 0) {
        launch(k_empty_root, 1, 1, 0, s, h->nodes);
    } else {
        const Groups G{n, group, leaf_size};
        launch(k_obox_init, 2 * sm_count(), kT, 0, s, h->obox, h->obox_cap, (const int*)(bounds + 13));
        char* sort_scratch = scratch + 256 + b_xchg + b_keys + b_open;
        uint32_t* hist = radix_sort_hist(sort_scratch, (size_t)n, false);
        e = cudaMemsetAsync(hist, 0, 4 * 256 * sizeof(uint32_t), s);
        if (e != cudaSuccess) goto fail;
        launch(k_morton, (unsigned)std::min<uint64_t>(((uint64_t)n + kT - 1) / kT, 8ull * sm_count()), kT, 0, s,
               d_vertices, nV, d_indices, nF, d_tri2obj, (const int*)bounds, keys,
               reinterpret_cast<unsigned int*>(bounds + 12), h->obox, h->obox_cap, hist);
        e = radix_sort_u64_in(keys, nullptr, (size_t)n, 64, s, 32, reinterpret_cast<uint32_t*>(bounds + 12), 2u,
                              sort_scratch, true);
        if (e != cudaSuccess) goto fail;
        const int utok = prof_begin(P_BUILD_UP, s);
        launch(k_build_tree, (nG + kTB - 1) / kTB, kTB, 0, s, d_vertices, nV, d_indices, d_tri2obj, (const uint64_t*)keys,
               G, nG, h->tris, h->nodes, open, n_open);
        prof_end(P_BUILD_UP, s, utok);
        if (nG == 1)
            launch(k_one_group_root, 1, 1, 0, s, (const float4*)h->tris, n, h->nodes);
        else
            launch(k_build_cross, 4 * sm_count(), kT, 0, s, (const uint64_t*)keys, G, nG, h->nodes, xchg,
                   (const OpenTree*)open, (const unsigned int*)n_open);
    }
    prof_end(P_BVH_BUILD, s, ptok);
    e = cudaGetLastError();
    // The result words go to a pinned slot, read by bvh_ready() after the build's event.
    if (e == cudaSuccess) {
        slot = pinned_slot_acquire();
        if (!slot) e = cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(slot, bounds, 14 * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(h->done, s);
fail:
    if (scratch) cudaFreeAsync(scratch, s);
    if (e != cudaSuccess) {
        if (h->mem) cudaFreeAsync(h->mem, s);
        h->mem = nullptr;
        h->nodes = nullptr;
        h->tris = nullptr;
        h->obox = nullptr;
        cudaStreamSynchronize(s);
        pinned_slot_release(slot);
        if (h->done) cudaEventDestroy(h->done);
        delete h;
        return to_status(e);
    }
    h->pending = slot;
    if (!async) {
        const int st = bvh_ready(h);
        prof_collect();
        if (st != RS_OK) {
            bvh_free(h);
            return st;
        }
    }
    *out = h;
    return RS_OK;
}

}  // namespace rs

extern "C" int rs_bvh_build(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                            const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, void* stream) {
    return rs::build_impl(d_vertices, nV, d_indices, nF, d_tri2obj, leaf_size, out, (cudaStream_t)stream, false);
}

extern "C" int rs_bvh_build_async(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                                  const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, void* stream) {
    return rs::build_impl(d_vertices, nV, d_indices, nF, d_tri2obj, leaf_size, out, (cudaStream_t)stream, true);
}

extern "C" int rs_bvh_wait(const rs_bvh* bvh) {
    if (!bvh) return RS_ERR_INVALID;
    return rs::bvh_ready(bvh);
}

extern "C" int rs_bvh_destroy(rs_bvh* bvh) {
    if (!bvh) return RS_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(bvh->device);
    rs::bvh_free(bvh);
    cudaSetDevice(prev);
    return RS_OK;
}

extern "C" int rs_bvh_info(const rs_bvh* bvh, uint64_t* n_tri, uint64_t* n_nodes, uint64_t* bytes,
                           float* h_min3, float* h_max3) {
    if (!bvh) return RS_ERR_INVALID;
    const int st = rs::bvh_ready(bvh);
    if (st != RS_OK) return st;
    if (n_tri) *n_tri = bvh->n_tris;
    if (n_nodes) *n_nodes = bvh->n_nodes;
    if (bytes) *bytes = bvh->n_nodes * sizeof(BNode) + bvh->n_tris * 3 * sizeof(float4);
    for (int k = 0; k < 3; ++k) {
        if (h_min3) h_min3[k] = bvh->vmin[k];
        if (h_max3) h_max3[k] = bvh->vmax[k];
    }
    return RS_OK;
}
