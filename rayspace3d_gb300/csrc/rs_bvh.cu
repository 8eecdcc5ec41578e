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
//   4. one bottom-up pass (k_build_up) that writes the triangles in leaf order
//      (3 x float4 each), builds the binary radix tree over the sorted keys
//      agglomeratively and refits its boxes on the way up, emitting 64-byte nodes
//      in which subtrees of <= leaf_size triangles become leaves.
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

// bounds[0..2] = min (ordered ints), [3..5] = max; [6..11] same for vertices.
__global__ void k_init_bounds(int* b) {
    if (threadIdx.x < 12) b[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0x7fffffff : (int)0x80000000;
}

__device__ __forceinline__ void block_minmax_atomic(float mn[3], float mx[3], int* out) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&out[k], flt_ord(mn[k]));
            atomicMax(&out[3 + k], flt_ord(mx[k]));
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
    if ((reinterpret_cast<uintptr_t>(V) & 15u) == 0) {
        const float4* V4 = reinterpret_cast<const float4*>(V);
        const uint64_t n4 = nf / 4;
        for (uint64_t q = tid; q < n4; q += stride) {
            const float4 v = __ldg(&V4[q]);
            const int c = (int)(q % 3);
            fold_component(mn, mx, c, v.x);
            fold_component(mn, mx, c == 2 ? 0 : c + 1, v.y);
            fold_component(mn, mx, c == 0 ? 2 : c - 1, v.z);
            fold_component(mn, mx, c, v.w);
        }
        done = 4 * n4;
    }
    for (uint64_t f = done + tid; f < nf; f += stride) fold_component(mn, mx, (int)(f % 3), V[f]);
    block_minmax_atomic(mn, mx, bounds + 6);
    int mo = -1;
    if ((reinterpret_cast<uintptr_t>(t2o) & 15u) == 0) {
        const int4* T4 = reinterpret_cast<const int4*>(t2o);
        for (uint64_t q = tid; q < nF / 4; q += stride) {
            const int4 t = __ldg(&T4[q]);
            mo = max(max(mo, max(t.x, t.y)), max(t.z, t.w));
        }
        for (uint64_t t = 4 * (nF / 4) + tid; t < nF; t += stride) mo = max(mo, t2o[t]);
    } else {
        for (uint64_t t = tid; t < nF; t += stride) mo = max(mo, t2o[t]);
    }
    mo = __reduce_max_sync(0xffffffffu, mo);
    if ((threadIdx.x & 31) == 0 && mo >= 0) atomicMax(max_obj, mo);
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
__global__ void k_morton(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t nF,
                         const int* __restrict__ bounds, uint64_t* __restrict__ keys,
                         unsigned int* __restrict__ bad_index) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t < nF) {
        if (I[3 * t] >= nV || I[3 * t + 1] >= nV || I[3 * t + 2] >= nV) atomicOr(bad_index, 1u);
        float lo[3], hi[3];
        tri_box(V, nV, I, t, lo, hi);
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
    }
}

// Length of the common prefix of sorted keys i and i+1 (keys are distinct).
__device__ __forceinline__ int split_prefix(const uint64_t* __restrict__ keys, int i) {
    return __clzll((long long)(__ldg(&keys[i]) ^ __ldg(&keys[i + 1])));
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

// A subtree left open by the block phase of k_build_up: box, leaf range, node slot.
struct OpenTree {
    float lo[3], hi[3];
    int l, r, self;
};

// Bottom-up construction of the binary radix tree over the sorted keys, fused with
// the emission of the leaf-ordered triangles and the box refit (agglomerative LBVH,
// Apetrei 2014, "Fast and Simple Agglomerative LBVH Construction").  Thread k starts
// at leaf k with range [k, k].  A subtree [l, r] joins the neighbouring split whose
// keys share the longer prefix: split r (it is the left child) or split l-1 (the
// right child); a split with no neighbour on one side takes the other.  This yields
// the same tree as Karras' top-down construction.
//
// Merges inside a warp's 32 leaves run first, in lock-step rounds without memory
// fences: a subtree is owned by the lane of its leftmost leaf, so a left child finds
// its right sibling at lane r+1 and merges when that lane holds a complete subtree
// that chose the same split; the split prefixes come from the lanes by shuffle.  The
// rounds end when no merge happens.  The remaining subtrees meet their siblings across
// warps: at split p the child writes its box and entry into its half of node slot
// p+1, then exchanges its outer range bound in xchg[p] with acquire-release
// semantics; the first arrival stops, the second reads its sibling's half, merges and
// continues.  Every split therefore sees exactly one merge, in the warp or through
// xchg.  Subtrees of <= leaf_size triangles are entered as leaves (first triangle,
// count), larger ones by their slot (count 0); slot 0 receives the root.
__global__ void __launch_bounds__(kT) k_build_up(const float* __restrict__ V, uint64_t nV,
                                                 const uint32_t* __restrict__ I, const int32_t* __restrict__ t2o,
                                                 const uint64_t* __restrict__ keys, int n, int leaf_size,
                                                 float4* __restrict__ tris, BNode* __restrict__ nodes,
                                                 OpenTree* __restrict__ open, unsigned int* __restrict__ n_open) {
    __shared__ int s_absorbed[kT];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int base = k - lane;
    const bool valid = k < n;
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
    if (valid) {
        const uint32_t t = (uint32_t)(__ldg(&keys[k]) & 0xffffffffull);
        const uint64_t last = nV - 1;
        const uint64_t i0 = min((uint64_t)I[3 * (uint64_t)t], last),
                       i1 = min((uint64_t)I[3 * (uint64_t)t + 1], last),
                       i2 = min((uint64_t)I[3 * (uint64_t)t + 2], last);
        float a[3], b[3], c[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            a[q] = V[3 * i0 + q];
            b[q] = V[3 * i1 + q];
            c[q] = V[3 * i2 + q];
            lo[q] = fminf(fminf(a[q], b[q]), c[q]);
            hi[q] = fmaxf(fmaxf(a[q], b[q]), c[q]);
        }
        tris[3 * (uint64_t)k] = make_float4(a[0], a[1], a[2], __uint_as_float(t));
        tris[3 * (uint64_t)k + 1] = make_float4(b[0], b[1], b[2], __int_as_float(t2o[t]));
        tris[3 * (uint64_t)k + 2] = make_float4(c[0], c[1], c[2], 0.0f);
    }
    // Split prefixes: lane j holds split base+j; split base-1 is broadcast.
    const int d_own = (k < n - 1) ? split_prefix(keys, k) : -1;
    const int d_left = __shfl_sync(0xffffffffu, (lane == 0 && base > 0 && base - 1 < n - 1) ? split_prefix(keys, base - 1)
                                                                                          : -1, 0);
    int l = k, r = k, self = 0;
    bool active = valid;
    for (;;) {
        // Choose the parent split of the owned subtree (only meaningful when active).
        const bool root = active && l == 0 && r == n - 1;
        const int dr = __shfl_sync(0xffffffffu, d_own, min(max(r - base, 0), 31));
        const int dl_in = __shfl_sync(0xffffffffu, d_own, min(max(l - 1 - base, 0), 31));
        const int dl = (l - 1 == base - 1) ? d_left : dl_in;
        const bool left_child = (l == 0) ? true : (r == n - 1) ? false : dr > dl;
        // Sibling of a left child: the subtree owned by lane r+1-base.
        const int sl = min(max(r + 1 - base, 0), 31);
        const int o_active = __shfl_sync(0xffffffffu, (int)(active && !root), sl);
        const int o_l = __shfl_sync(0xffffffffu, l, sl);
        const int o_r = __shfl_sync(0xffffffffu, r, sl);
        const int o_left = __shfl_sync(0xffffffffu, (int)left_child, sl);
        const int o_self = __shfl_sync(0xffffffffu, self, sl);
        float olo[3], ohi[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            olo[q] = __shfl_sync(0xffffffffu, lo[q], sl);
            ohi[q] = __shfl_sync(0xffffffffu, hi[q], sl);
        }
        const bool merge = active && !root && left_child && r + 1 - base <= 31 && o_active && o_l == r + 1 && !o_left;
        s_absorbed[threadIdx.x] = 0;
        __syncwarp();
        if (merge) s_absorbed[threadIdx.x - lane + (r + 1 - base)] = 1;
        __syncwarp();
        const bool absorbed = s_absorbed[threadIdx.x] != 0;
        __syncwarp();
        if (merge) {
            const int p = r;
            const int size0 = r - l + 1, size1 = o_r - o_l + 1;
            store_node(nodes + (p + 1), lo, hi, size0 <= leaf_size ? l : self, size0 <= leaf_size ? size0 : 0, olo,
                       ohi, size1 <= leaf_size ? o_l : o_self, size1 <= leaf_size ? size1 : 0);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                lo[q] = fminf(lo[q], olo[q]);
                hi[q] = fmaxf(hi[q], ohi[q]);
            }
            r = o_r;
            self = p + 1;
            if (l == 0 && r == n - 1) {
                const BNode nd = nodes[self];
                nodes[0] = nd;
                active = false;
            }
        }
        if (absorbed) active = false;
        if (!__any_sync(0xffffffffu, merge)) break;
    }
    // Block rounds: the subtrees still open after the warp rounds meet siblings owned by
    // other warps of the block through shared memory, in lock-step rounds separated by
    // block barriers.  The owner of a subtree is still the thread of its leftmost leaf,
    // so l == k, r stays inside the block, and the sibling of a left child is owned by
    // thread r + 1 - bb.
    {
        __shared__ int s_d[kT + 1];  // split prefixes of splits bb-1 .. bb+kT-1
        __shared__ int s_r[kT], s_self[kT];
        __shared__ float s_box[6][kT];
        __shared__ unsigned char s_state[kT];  // bit 0: open subtree, bit 1: left child
        __shared__ unsigned char s_abs[kT];
        const int bb = blockIdx.x * blockDim.x;
        const int tid = threadIdx.x;
        s_d[tid + 1] = d_own;
        if (tid == 0) s_d[0] = (bb > 0 && bb - 1 < n - 1) ? split_prefix(keys, bb - 1) : -1;
        s_abs[tid] = 0;
        __syncthreads();
        for (int round = 0; round < kT; ++round) {
            bool left_child = false;
            if (active) {
                const int dr = s_d[r - bb + 1], dl = s_d[l - bb];
                left_child = (l == 0) ? true : (r == n - 1) ? false : dr > dl;
            }
            s_r[tid] = r;
            s_self[tid] = self;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                s_box[q][tid] = lo[q];
                s_box[3 + q][tid] = hi[q];
            }
            s_state[tid] = (unsigned char)((active ? 1 : 0) | (left_child ? 2 : 0));
            __syncthreads();
            bool merged = false;
            const int sib = r + 1 - bb;
            if (active && left_child && sib < kT && r + 1 < n && s_state[sib] == 1) {
                const int p = r;
                const int o_r = s_r[sib];
                const int size0 = r - l + 1, size1 = o_r - r;
                float olo[3], ohi[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    olo[q] = s_box[q][sib];
                    ohi[q] = s_box[3 + q][sib];
                }
                store_node(nodes + (p + 1), lo, hi, size0 <= leaf_size ? l : self, size0 <= leaf_size ? size0 : 0,
                           olo, ohi, size1 <= leaf_size ? r + 1 : s_self[sib], size1 <= leaf_size ? size1 : 0);
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    lo[q] = fminf(lo[q], olo[q]);
                    hi[q] = fmaxf(hi[q], ohi[q]);
                }
                r = o_r;
                self = p + 1;
                s_abs[sib] = 1;
                merged = true;
                if (l == 0 && r == n - 1) {
                    const BNode nd = nodes[self];
                    nodes[0] = nd;
                    active = false;
                }
            }
            __syncthreads();
            if (s_abs[tid]) {
                active = false;
                s_abs[tid] = 0;
            }
            if (!__syncthreads_or(merged)) break;
        }
    }
    // Subtrees still open go to the cross-block phase (k_build_cross), packed densely so
    // that its latency-bound walks do not hold this kernel's blocks.
    const unsigned m = __ballot_sync(0xffffffffu, active);
    if (!m) return;
    unsigned int slot = 0;
    if (lane == __ffs(m) - 1) slot = atomicAdd(n_open, (unsigned int)__popc(m));
    slot = __shfl_sync(0xffffffffu, slot, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1u));
    if (!active) return;
    OpenTree& o = open[slot];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        o.lo[q] = lo[q];
        o.hi[q] = hi[q];
    }
    o.l = l;
    o.r = r;
    o.self = self;
}

// Cross-block merges through the exchange array, one open subtree per thread.
__global__ void __launch_bounds__(kT) k_build_cross(const uint64_t* __restrict__ keys, int n, int leaf_size,
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
            const int size = r - l + 1;
            if (l == 0 && r == n - 1) {
                const float4* src = reinterpret_cast<const float4*>(nodes + self);
                float4* dst = reinterpret_cast<float4*>(nodes);
#pragma unroll
                for (int q = 0; q < 4; ++q) dst[q] = __ldcg(src + q);
                break;
            }
            const bool left_child =
                (l == 0) ? true : (r == n - 1) ? false : split_prefix(keys, r) > split_prefix(keys, l - 1);
            const int p = left_child ? r : l - 1;
            BNode* nd = nodes + (p + 1);
            store_half(nd, left_child ? 0 : 1, lo, hi, size <= leaf_size ? l : self, size <= leaf_size ? size : 0);
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

__global__ void k_emit_tris(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                            const int32_t* __restrict__ t2o, const uint64_t* __restrict__ order, int n,
                            float4* __restrict__ tris) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t t = (uint32_t)(order[k] & 0xffffffffull);
    const uint64_t last = nV - 1;
    const uint64_t i0 = min((uint64_t)I[3 * (uint64_t)t], last), i1 = min((uint64_t)I[3 * (uint64_t)t + 1], last),
                   i2 = min((uint64_t)I[3 * (uint64_t)t + 2], last);
    const float* a = V + 3 * (uint64_t)i0;
    const float* b = V + 3 * (uint64_t)i1;
    const float* c = V + 3 * (uint64_t)i2;
    tris[3 * (uint64_t)k] = make_float4(a[0], a[1], a[2], __uint_as_float(t));
    tris[3 * (uint64_t)k + 1] = make_float4(b[0], b[1], b[2], __int_as_float(t2o[t]));
    tris[3 * (uint64_t)k + 2] = make_float4(c[0], c[1], c[2], 0.0f);
}

// Root for n <= 1: child 0 is the single leaf (if any), child 1 an empty box.
__global__ void k_small_root(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, int n,
                             BNode* nodes) {
    const float inf = INFINITY;
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    if (n == 1) tri_box(V, nV, I, 0, lo, hi);
    BNode nd;
    nd.a = make_float4(lo[0], lo[1], lo[2], hi[0]);
    nd.b = make_float4(hi[1], hi[2], inf, inf);
    nd.c = make_float4(inf, -inf, -inf, -inf);
    nd.d = make_int4(0, n == 1 ? 1 : 0, 0, 0);
    // An empty child must never be entered: its count is 0 and its box is empty,
    // so the slab test rejects it before the index is used.
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
    if (bits & ST_TABLE_FULL) return RS_ERR_TABLE_FULL;
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
    if (h->nodes) cudaFree(h->nodes);
    if (h->tris) cudaFree(h->tris);
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
    if (leaf_size == 0) leaf_size = 4;
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
    int* bounds = nullptr;  // [6..11] vertex bounds (ordered ints), [12] bad-index flag, [13] max object
    uint64_t* keys = nullptr;
    int* xchg = nullptr;
    OpenTree* open = nullptr;
    unsigned int* n_open = nullptr;
    cudaError_t e = cudaSuccess;
    int* slot = nullptr;
    const int grid = 4 * sm_count();
    h->n_nodes = n >= 2 ? (uint64_t)n : 1;  // slot 0 = root, slot p+1 = split p
    h->n_tris = (uint64_t)n;
    const int ptok = prof_begin(P_BVH_BUILD, s);
    e = alloc(&h->nodes, h->n_nodes, s);
    if (e == cudaSuccess) e = alloc(&h->tris, 3 * (size_t)n, s);
    if (e == cudaSuccess) e = alloc(&bounds, 14, s);
    if (e != cudaSuccess) goto fail;
    launch(k_init_bounds, 1, 32, 0, s, bounds);
    cudaMemsetAsync(bounds + 12, 0, sizeof(int), s);
    cudaMemsetAsync(bounds + 13, 0xff, sizeof(int), s);
    if (nV || nF) launch(k_vertex_bounds, grid, kT, 0, s, d_vertices, nV, d_tri2obj, nF, bounds, bounds + 13);
    if (n <= 1) {
        launch(k_small_root, 1, 1, 0, s, d_vertices, nV, d_indices, n, h->nodes);
        if (n == 1) {
            e = alloc(&keys, 1, s);
            if (e == cudaSuccess) launch(k_morton, 1, 32, 0, s, d_vertices, nV, d_indices, nF, bounds, keys,
                                         reinterpret_cast<unsigned int*>(bounds + 12));
            if (e == cudaSuccess) launch(k_emit_tris, 1, 32, 0, s, d_vertices, nV, d_indices, d_tri2obj,
                                         (const uint64_t*)keys, 1, h->tris);
        }
    } else {
        const int nb = (n + kT - 1) / kT;
        e = alloc(&keys, n, s);
        if (e == cudaSuccess) e = alloc(&xchg, n - 1, s);
        if (e != cudaSuccess) goto fail;
        launch(k_morton, nb, kT, 0, s, d_vertices, nV, d_indices, nF, bounds, keys,
               reinterpret_cast<unsigned int*>(bounds + 12));
        e = radix_sort_u64(keys, nullptr, (size_t)n, 64, s, 32, reinterpret_cast<uint32_t*>(bounds + 12), 2u);
        if (e != cudaSuccess) goto fail;
        cudaMemsetAsync(xchg, 0xff, (size_t)(n - 1) * sizeof(int), s);
        // Open subtrees per block: at most two per level of the tree (64 key bits), so
        // n / 2 bounds them for blocks of 256 leaves.
        e = alloc(&open, (size_t)n / 2 + kT, s);
        if (e == cudaSuccess) e = alloc(&n_open, 1, s);
        if (e != cudaSuccess) goto fail;
        cudaMemsetAsync(n_open, 0, sizeof(unsigned int), s);
        launch(k_build_up, nb, kT, 0, s, d_vertices, nV, d_indices, d_tri2obj, (const uint64_t*)keys, n, leaf_size,
               h->tris, h->nodes, open, n_open);
        launch(k_build_cross, 4 * sm_count(), kT, 0, s, (const uint64_t*)keys, n, leaf_size, h->nodes, xchg,
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
    if (keys) cudaFreeAsync(keys, s);
    if (xchg) cudaFreeAsync(xchg, s);
    if (open) cudaFreeAsync(open, s);
    if (n_open) cudaFreeAsync(n_open, s);
    if (bounds) cudaFreeAsync(bounds, s);
    if (e != cudaSuccess) {
        if (h->nodes) cudaFreeAsync(h->nodes, s);
        if (h->tris) cudaFreeAsync(h->tris, s);
        h->nodes = nullptr;
        h->tris = nullptr;
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
