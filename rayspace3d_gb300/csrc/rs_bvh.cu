// rs_bvh.cu -- Morton-code LBVH builder.
//
// Replaces OptixAccelerationStructure::buildInternal
// (query/src/optix/OptixAccelerationStructure.cpp:22-68), which builds one
// triangle GAS over every triangle of a .pre set.  Steps:
//   1. per-triangle boxes, scene bounds of triangle centres and of all vertices;
//   2. keys = 32-bit Morton code of the centre (11/11/10 bits) << 32 | triangle id,
//      unique by construction;
//   3. stable radix sort of the 32 Morton bits only (4 passes; ids stay ascending
//      within equal codes);
//   4. Karras' binary radix tree over the sorted keys;
//   5. the triangles in leaf order (3 x float4 each);
//   6. bottom-up box refit that starts from leaf groups (subtrees of <= leaf_size
//      triangles, whose boxes are read straight from the leaf-ordered triangles),
//      with one acquire-release arrival counter per node;
//   7. emission of 64-byte nodes in which the leaf groups become leaves.
#include <cstdio>
#include <cstdlib>
#include <cstring>


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

__global__ void k_vertex_bounds(const float* __restrict__ V, uint64_t nV, int* bounds) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nV; i += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float v = V[3 * i + k];
            mn[k] = fminf(mn[k], v);
            mx[k] = fmaxf(mx[k], v);
        }
    }
    block_minmax_atomic(mn, mx, bounds + 6);
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

__global__ void k_centroid_bounds(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I,
                                  uint64_t nF, int* bounds, unsigned int* bad_index) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < nF; t += (uint64_t)gridDim.x * blockDim.x) {
        if (I[3 * t] >= nV || I[3 * t + 1] >= nV || I[3 * t + 2] >= nV) {
            atomicOr(bad_index, 1u);
            continue;
        }
        float lo[3], hi[3];
        tri_box(V, nV, I, t, lo, hi);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c = 0.5f * lo[k] + 0.5f * hi[k];
            mn[k] = fminf(mn[k], c);
            mx[k] = fmaxf(mx[k], c);
        }
    }
    block_minmax_atomic(mn, mx, bounds);
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void k_morton(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t nF,
                         const int* __restrict__ bounds, uint64_t* __restrict__ keys) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF) return;
    float lo[3], hi[3];
    tri_box(V, nV, I, t, lo, hi);
    uint32_t q[3];
    const float scale[3] = {2048.0f, 2048.0f, 1024.0f};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float cmin = ord_flt(bounds[k]), cmax = ord_flt(bounds[3 + k]);
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

__device__ __forceinline__ int delta(const uint64_t* __restrict__ keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll((long long)(a ^ b));
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d trees".
// Internal nodes 0..n-2, leaves n-1..2n-2.
__global__ void k_karras(const uint64_t* __restrict__ keys, int n, int* __restrict__ left, int* __restrict__ right,
                         int* __restrict__ parent, int2* __restrict__ range) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = (lo == gamma) ? (n - 1 + gamma) : gamma;
    const int rc = (hi == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    parent[lc] = i;
    parent[rc] = i;
    range[i] = make_int2(lo, hi);
}

// Bottom-up refit from the leaf groups.  One thread per internal node p whose range
// is larger than leaf_size (and the root): each child of p that spans <= leaf_size
// triangles is a leaf group whose box is the union of its triangles, contiguous in
// leaf order.  The thread stores that box and arrives at p; the second arrival at a
// node merges both children and moves up.  Each arrival publishes its box with a
// release fence before the counter increment; the second arrival's loads depend on
// the increment's result and bypass L1.
__device__ __forceinline__ void arrive(int node, float4 lo, float4 hi, int p, const int* __restrict__ left,
                                       const int* __restrict__ right, const int* __restrict__ parent,
                                       float4* __restrict__ blo, float4* __restrict__ bhi, int* __restrict__ flags) {
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&flags[p], 1) == 0) return;
        const int other = (__ldcg(&left[p]) == node) ? __ldcg(&right[p]) : __ldcg(&left[p]);
        const float4 ol = __ldcg(&blo[other]), oh = __ldcg(&bhi[other]);
        lo = make_float4(fminf(lo.x, ol.x), fminf(lo.y, ol.y), fminf(lo.z, ol.z), 0.f);
        hi = make_float4(fmaxf(hi.x, oh.x), fmaxf(hi.y, oh.y), fmaxf(hi.z, oh.z), 0.f);
        __stcg(&blo[p], lo);
        __stcg(&bhi[p], hi);
        node = p;
        p = __ldcg(&parent[p]);
    }
}

__global__ void k_refit(const float4* __restrict__ tris, int n, int leaf_size, const int* __restrict__ left,
                        const int* __restrict__ right, const int* __restrict__ parent, const int2* __restrict__ range,
                        float4* __restrict__ blo, float4* __restrict__ bhi, int* __restrict__ flags) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n - 1) return;
    const int2 rp = range[p];
    if (p != 0 && rp.y - rp.x + 1 <= leaf_size) return;  // inside a leaf group
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const int c = side == 0 ? left[p] : right[p];
        int first, size;
        if (c >= n - 1) {
            first = c - (n - 1);
            size = 1;
        } else {
            const int2 rc = range[c];
            first = rc.x;
            size = rc.y - rc.x + 1;
        }
        if (size > leaf_size) continue;
        float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
        for (int k = first; k < first + size; ++k) {
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                const float4 q = tris[3 * (size_t)k + v];
                lo = make_float4(fminf(lo.x, q.x), fminf(lo.y, q.y), fminf(lo.z, q.z), 0.f);
                hi = make_float4(fmaxf(hi.x, q.x), fmaxf(hi.y, q.y), fmaxf(hi.z, q.z), 0.f);
            }
        }
        __stcg(&blo[c], lo);
        __stcg(&bhi[c], hi);
        arrive(c, lo, hi, p, left, right, parent, blo, bhi, flags);
    }
}

__device__ __forceinline__ void child_entry(int c, int n, int leaf_size, const int2* __restrict__ range,
                                            int& idx, int& cnt) {
    if (c >= n - 1) {
        idx = c - (n - 1);
        cnt = 1;
        return;
    }
    const int2 r = range[c];
    const int size = r.y - r.x + 1;
    if (size <= leaf_size) {
        idx = r.x;
        cnt = size;
    } else {
        idx = c;
        cnt = 0;
    }
}

__global__ void k_emit_nodes(int n, int leaf_size, const int* __restrict__ left, const int* __restrict__ right,
                             const int2* __restrict__ range, const float4* __restrict__ blo,
                             const float4* __restrict__ bhi, BNode* __restrict__ nodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int l = left[i], r = right[i];
    int i0, c0, i1, c1;
    child_entry(l, n, leaf_size, range, i0, c0);
    child_entry(r, n, leaf_size, range, i1, c1);
    const float4 l0 = blo[l], h0 = bhi[l], l1 = blo[r], h1 = bhi[r];
    BNode nd;
    nd.a = make_float4(l0.x, l0.y, l0.z, h0.x);
    nd.b = make_float4(h0.y, h0.z, l1.x, l1.y);
    nd.c = make_float4(l1.z, h1.x, h1.y, h1.z);
    nd.d = make_int4(i0, c0, i1, c1);
    nodes[i] = nd;
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

extern "C" int rs_bvh_build(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                            const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, void* stream) {
    if (!out) return RS_ERR_INVALID;
    *out = nullptr;
    if ((nF && (!d_indices || !d_tri2obj || !d_vertices)) || (nV && !d_vertices)) return RS_ERR_INVALID;
    if (nF && nV == 0) return RS_ERR_INVALID;               // every index would be out of range
    if (nF >= (uint64_t)0x7fffffff) return RS_ERR_INVALID;  // node/leaf indices are int32
    if (leaf_size == 0) leaf_size = 4;
    if (leaf_size < 1 || leaf_size > 8) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    rs_bvh* h = new rs_bvh();
    h->V = d_vertices;
    h->nV = nV;
    h->I = d_indices;
    h->nF = nF;
    h->t2o = d_tri2obj;
    h->leaf_size = leaf_size;
    cudaGetDevice(&h->device);
    const int n = (int)nF;
    int* bounds = nullptr;  // 12 ordered-int bounds, then the bad-index flag
    uint64_t* keys = nullptr;
    int *left = nullptr, *right = nullptr, *parent = nullptr, *flags = nullptr;
    int2* range = nullptr;
    float4 *blo = nullptr, *bhi = nullptr;
    cudaError_t e = cudaSuccess;
    int hb[13];
    const int grid = 4 * sm_count();
    h->n_nodes = n >= 2 ? (uint64_t)(n - 1) : 1;
    h->n_tris = (uint64_t)n;
    prof_begin(P_BVH_BUILD, s);
    e = alloc(&h->nodes, h->n_nodes, s);
    if (e == cudaSuccess) e = alloc(&h->tris, 3 * (size_t)n, s);
    if (e == cudaSuccess) e = alloc(&bounds, 13, s);
    if (e != cudaSuccess) goto fail;
    launch(k_init_bounds, 1, 32, 0, s, bounds);
    cudaMemsetAsync(bounds + 12, 0, sizeof(int), s);
    if (nV) launch(k_vertex_bounds, grid, kT, 0, s, d_vertices, nV, bounds);
    if (nF) launch(k_centroid_bounds, grid, kT, 0, s, d_vertices, nV, d_indices, nF, bounds,
                   reinterpret_cast<unsigned int*>(bounds + 12));
    if (n <= 1) {
        launch(k_small_root, 1, 1, 0, s, d_vertices, nV, d_indices, n, h->nodes);
        if (n == 1) {
            e = alloc(&keys, 1, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(keys, 0, sizeof(uint64_t), s);
            if (e == cudaSuccess) launch(k_emit_tris, 1, 32, 0, s, d_vertices, nV, d_indices, d_tri2obj,
                                         (const uint64_t*)keys, 1, h->tris);
        }
    } else {
        const int nb = (n + kT - 1) / kT;
        const int nbi = (n - 1 + kT - 1) / kT;
        e = alloc(&keys, n, s);
        if (e == cudaSuccess) e = alloc(&left, n - 1, s);
        if (e == cudaSuccess) e = alloc(&right, n - 1, s);
        if (e == cudaSuccess) e = alloc(&parent, 2 * (size_t)n - 1, s);
        if (e == cudaSuccess) e = alloc(&flags, n - 1, s);
        if (e == cudaSuccess) e = alloc(&range, n - 1, s);
        if (e == cudaSuccess) e = alloc(&blo, 2 * (size_t)n - 1, s);
        if (e == cudaSuccess) e = alloc(&bhi, 2 * (size_t)n - 1, s);
        if (e != cudaSuccess) goto fail;
        launch(k_morton, nb, kT, 0, s, d_vertices, nV, d_indices, nF, bounds, keys);
        e = radix_sort_u64(keys, nullptr, (size_t)n, 64, s, 32);
        if (e != cudaSuccess) goto fail;
        cudaMemsetAsync(parent, 0xff, (2 * (size_t)n - 1) * sizeof(int), s);
        cudaMemsetAsync(flags, 0, (size_t)(n - 1) * sizeof(int), s);
        launch(k_karras, nbi, kT, 0, s, keys, n, left, right, parent, range);
        launch(k_emit_tris, nb, kT, 0, s, d_vertices, nV, d_indices, d_tri2obj, (const uint64_t*)keys, n, h->tris);
        launch(k_refit, nbi, kT, 0, s, (const float4*)h->tris, n, leaf_size, left, right, parent, range, blo, bhi,
               flags);
        launch(k_emit_nodes, nbi, kT, 0, s, n, leaf_size, left, right, range, blo, bhi, h->nodes);
    }
    prof_end(P_BVH_BUILD, s);
    e = cudaGetLastError();
    // One host round trip: vertex bounds for the filter box and the bad-index flag.
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    prof_collect();
fail:
    if (bounds) cudaFreeAsync(bounds, s);
    if (keys) cudaFreeAsync(keys, s);
    if (left) cudaFreeAsync(left, s);
    if (right) cudaFreeAsync(right, s);
    if (parent) cudaFreeAsync(parent, s);
    if (flags) cudaFreeAsync(flags, s);
    if (range) cudaFreeAsync(range, s);
    if (blo) cudaFreeAsync(blo, s);
    if (bhi) cudaFreeAsync(bhi, s);
    const bool bad = (e == cudaSuccess) && hb[12] != 0;
    if (e != cudaSuccess || bad) {
        if (h->nodes) cudaFreeAsync(h->nodes, s);
        if (h->tris) cudaFreeAsync(h->tris, s);
        cudaStreamSynchronize(s);
        delete h;
        return bad ? RS_ERR_INVALID : to_status(e);
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
    *out = h;
    return RS_OK;
}

extern "C" int rs_bvh_destroy(rs_bvh* bvh) {
    if (!bvh) return RS_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(bvh->device);
    if (bvh->nodes) cudaFree(bvh->nodes);
    if (bvh->tris) cudaFree(bvh->tris);
    for (auto& g : bvh->cgrid) {
        if (g.start) cudaFree(g.start);
        if (g.list) cudaFree(g.list);
    }
    cudaSetDevice(prev);
    delete bvh;
    return RS_OK;
}

extern "C" int rs_bvh_info(const rs_bvh* bvh, uint64_t* n_tri, uint64_t* n_nodes, uint64_t* bytes,
                           float* h_min3, float* h_max3) {
    if (!bvh) return RS_ERR_INVALID;
    if (n_tri) *n_tri = bvh->n_tris;
    if (n_nodes) *n_nodes = bvh->n_nodes;
    if (bytes) *bytes = bvh->n_nodes * sizeof(BNode) + bvh->n_tris * 3 * sizeof(float4);
    for (int k = 0; k < 3; ++k) {
        if (h_min3) h_min3[k] = bvh->vmin[k];
        if (h_max3) h_max3[k] = bvh->vmax[k];
    }
    return RS_OK;
}
