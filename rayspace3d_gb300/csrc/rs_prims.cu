// rs_prims.cu -- stable LSD radix sort, exclusive scans and ordered compaction.
//
// Replaces the thrust sort/unique/scan/reduce calls of the reference
// (query/src/cuda/mesh_query_deduplication.cu:56-90, scan_utils.cu:11-28) with
// the engine's own kernels.  Tiles are 4096 elements (256 threads x 16 items);
// the radix scatter ranks keys per warp with __match_any_sync so every pass is
// stable.
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr int kWarps = kThreads / 32;
constexpr int kWarpSpan = 32 * kItems;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(kThreads) k_radix_hist(const uint64_t* __restrict__ keys, size_t n, int shift,
                                                          uint32_t* __restrict__ hist, int num_tiles) {
    __shared__ uint32_t sh[kWarps][256];
    for (int i = threadIdx.x; i < kWarps * 256; i += kThreads) (&sh[0][0])[i] = 0;
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const size_t idx = base + (size_t)it * kThreads + threadIdx.x;
        if (idx < n) atomicAdd(&sh[w][(uint32_t)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    uint32_t s = 0;
#pragma unroll
    for (int ww = 0; ww < kWarps; ++ww) s += sh[ww][threadIdx.x];
    hist[(size_t)threadIdx.x * num_tiles + blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                             const uint32_t* __restrict__ vin,
                                                             uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                             size_t n, int shift, const uint32_t* __restrict__ offs,
                                                             int num_tiles) {
    __shared__ uint32_t cnt[kWarps][256];
    for (int i = threadIdx.x; i < kWarps * 256; i += kThreads) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t base = (size_t)blockIdx.x * kTile + (size_t)w * kWarpSpan;
    uint64_t k[kItems];
    uint32_t v[kItems];
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        k[r] = 0;
        v[r] = 0;
        if (idx < n) {
            k[r] = kin[idx];
            if (vin) v[r] = vin[idx];
        }
    }
    // Pass A: per-warp digit counts.
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        const bool valid = idx < n;
        const uint32_t dg = valid ? ((uint32_t)(k[r] >> shift) & 255u) : (256u + lane);
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        if (valid && lane == __ffs(peers) - 1) cnt[w][dg] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        uint32_t run = offs[(size_t)threadIdx.x * num_tiles + blockIdx.x];
#pragma unroll
        for (int ww = 0; ww < kWarps; ++ww) {
            const uint32_t c = cnt[ww][threadIdx.x];
            cnt[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
    // Pass B: stable ranks and scatter.
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        const bool valid = idx < n;
        const uint32_t dg = valid ? ((uint32_t)(k[r] >> shift) & 255u) : (256u + lane);
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        uint32_t pos = 0;
        if (valid) pos = cnt[w][dg] + __popc(peers & lt);
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) cnt[w][dg] += __popc(peers);
        __syncwarp();
        if (valid) {
            kout[pos] = k[r];
            if (vout) vout[pos] = v[r];
        }
    }
}

// ---------------------------------------------------------------------------
// Scan: per-tile reduce, single-block scan of the tile sums, per-tile scan.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_inclusive(T x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Exclusive scan of one value per thread across the block; returns the block total in `total`.
template <class T>
__device__ __forceinline__ T block_exclusive(T x, T& total) {
    __shared__ T wsum[33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    T inc = warp_inclusive(x);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = lane < nw ? wsum[lane] : T(0);
        T si = warp_inclusive(s);
        if (lane < nw) wsum[lane] = si - s;
        if (lane == nw - 1) wsum[32] = si;
    }
    __syncthreads();
    T res = inc - x + wsum[w];
    total = wsum[32];
    __syncthreads();
    return res;
}

template <class Tin, class Tacc>
__global__ void __launch_bounds__(kThreads) k_scan_reduce(const Tin* __restrict__ in, size_t n, Tacc* __restrict__ part) {
    const size_t base = (size_t)blockIdx.x * kTile;
    Tacc s = 0;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const size_t idx = base + (size_t)it * kThreads + threadIdx.x;
        if (idx < n) s += (Tacc)in[idx];
    }
    Tacc tot;
    block_exclusive<Tacc>(s, tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <class Tacc>
__global__ void __launch_bounds__(1024) k_scan_top(Tacc* __restrict__ part, size_t nb, Tacc* __restrict__ total) {
    Tacc carry = 0;
    for (size_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        const size_t i = b0 + threadIdx.x;
        Tacc x = i < nb ? part[i] : Tacc(0);
        Tacc tot;
        Tacc ex = block_exclusive<Tacc>(x, tot);
        if (i < nb) part[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <class Tin, class Tacc>
__global__ void __launch_bounds__(kThreads) k_scan_down(const Tin* in, Tacc* out, size_t n,  // may alias
                                                         const Tacc* __restrict__ part) {
    __shared__ Tacc tile[kTile];
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int j = it * kThreads + threadIdx.x;
        const size_t idx = base + j;
        tile[j] = idx < n ? (Tacc)in[idx] : Tacc(0);
    }
    __syncthreads();
    Tacc loc[kItems];
    Tacc s = 0;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        loc[it] = s;
        s += tile[threadIdx.x * kItems + it];
    }
    Tacc tot;
    const Tacc off = block_exclusive<Tacc>(s, tot) + part[blockIdx.x];
#pragma unroll
    for (int it = 0; it < kItems; ++it) tile[threadIdx.x * kItems + it] = off + loc[it];
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int j = it * kThreads + threadIdx.x;
        const size_t idx = base + j;
        if (idx < n) out[idx] = tile[j];
    }
}

template <class Tin, class Tacc>
cudaError_t scan_impl(const Tin* in, Tacc* out, size_t n, Tacc* total, cudaStream_t s) {
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(Tacc), s);
        return cudaSuccess;
    }
    const size_t nb = (n + kTile - 1) / kTile;
    Tacc* part = nullptr;
    cudaError_t e = dmalloc((void**)&part, nb * sizeof(Tacc), s);
    if (e != cudaSuccess) return e;
    launch(k_scan_reduce<Tin, Tacc>, (unsigned)nb, kThreads, 0, s, in, n, part);
    launch(k_scan_top<Tacc>, 1, 1024, 0, s, part, nb, total);
    launch(k_scan_down<Tin, Tacc>, (unsigned)nb, kThreads, 0, s, in, out, n, part);
    e = cudaGetLastError();
    cudaFreeAsync(part, s);
    return e;
}

// ---------------------------------------------------------------------------
// Ordered compaction of u64 values != skip (used for hash-table slots and
// for unique-after-sort).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_compact_count(const uint64_t* __restrict__ in, size_t n, uint64_t skip,
                                                             const uint64_t* __restrict__ prev_of, uint64_t* __restrict__ part) {
    const size_t base = (size_t)blockIdx.x * kTile;
    uint64_t c = 0;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const size_t idx = base + (size_t)it * kThreads + threadIdx.x;
        if (idx < n) {
            const uint64_t x = in[idx];
            const bool keep = prev_of ? (idx == 0 || x != prev_of[idx - 1]) : (x != skip);
            c += keep;
        }
    }
    uint64_t tot;
    block_exclusive<uint64_t>(c, tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kThreads) k_compact_write(const uint64_t* __restrict__ in, size_t n, uint64_t skip,
                                                             const uint64_t* __restrict__ prev_of,
                                                             const uint64_t* __restrict__ part, uint64_t* __restrict__ out) {
    __shared__ uint64_t tile[kTile];
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int j = it * kThreads + threadIdx.x;
        const size_t idx = base + j;
        tile[j] = idx < n ? in[idx] : skip;
    }
    __syncthreads();
    uint32_t flags = 0;
    uint64_t c = 0;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int j = threadIdx.x * kItems + it;
        const size_t idx = base + j;
        bool keep = false;
        if (idx < n) {
            const uint64_t x = tile[j];
            if (prev_of) {
                const uint64_t p = (j > 0) ? tile[j - 1] : (idx > 0 ? prev_of[idx - 1] : ~x);
                keep = (idx == 0) || x != p;
            } else {
                keep = x != skip;
            }
        }
        flags |= (uint32_t)keep << it;
        c += keep;
    }
    uint64_t tot;
    uint64_t pos = block_exclusive<uint64_t>(c, tot) + part[blockIdx.x];
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        if (flags & (1u << it)) out[pos++] = tile[threadIdx.x * kItems + it];
    }
}

// Single-block bitonic sort of up to kSmallSort keys in shared memory.
constexpr int kSmallSort = 4096;

__global__ void __launch_bounds__(1024) k_sort_small(uint64_t* __restrict__ keys, int n) {
    __shared__ uint64_t sh[kSmallSort];
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = threadIdx.x; i < m; i += blockDim.x) sh[i] = i < n ? keys[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = sh[i], b = sh[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        sh[i] = b;
                        sh[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = sh[i];
}

}  // namespace

cudaError_t sort_u64_any(uint64_t* keys, size_t n, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    if (n <= (size_t)kSmallSort) {
        launch(k_sort_small, 1, 1024, 0, s, keys, (int)n);
        return cudaGetLastError();
    }
    return radix_sort_u64(keys, nullptr, n, 64, s);
}

int sm_count() {
    static int cached = 0;
    if (!cached) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev);
        if (cached <= 0) cached = 1;
    }
    return cached;
}

cudaError_t radix_sort_u64(uint64_t* keys, uint32_t* vals, size_t n, int end_bit, cudaStream_t s, int begin_bit) {
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
    const int passes = (end_bit - begin_bit + 7) / 8;
    const size_t tiles = (n + kTile - 1) / kTile;
    uint64_t* k2 = nullptr;
    uint32_t* v2 = nullptr;
    uint32_t* hist = nullptr;
    cudaError_t e = dmalloc((void**)&k2, n * sizeof(uint64_t), s);
    if (e == cudaSuccess && vals) e = dmalloc((void**)&v2, n * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = dmalloc((void**)&hist, 256 * tiles * sizeof(uint32_t), s);
    if (e != cudaSuccess) {
        if (k2) cudaFreeAsync(k2, s);
        if (v2) cudaFreeAsync(v2, s);
        return e;
    }
    uint64_t* ka = keys;
    uint64_t* kb = k2;
    uint32_t* va = vals;
    uint32_t* vb = v2;
    for (int p = 0; p < passes && e == cudaSuccess; ++p) {
        const int shift = begin_bit + 8 * p;
        launch(k_radix_hist, (unsigned)tiles, kThreads, 0, s, ka, n, shift, hist, (int)tiles);
        e = scan_impl<uint32_t, uint32_t>(hist, hist, 256 * tiles, nullptr, s);
        if (e != cudaSuccess) break;
        launch(k_radix_scatter, (unsigned)tiles, kThreads, 0, s, ka, va, kb, vb, n, shift, hist, (int)tiles);
        e = cudaGetLastError();
        uint64_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    if (e == cudaSuccess && ka != keys) {
        e = cudaMemcpyAsync(keys, ka, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && vals) e = cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
    cudaFreeAsync(hist, s);
    cudaFreeAsync(k2, s);
    if (v2) cudaFreeAsync(v2, s);
    return e;
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* total, cudaStream_t s) {
    return scan_impl<uint32_t, uint32_t>(in, out, n, total, s);
}

cudaError_t exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, size_t n, int64_t* total, cudaStream_t s) {
    return scan_impl<int32_t, long long>(in, reinterpret_cast<long long*>(out), n,
                                         reinterpret_cast<long long*>(total), s);
}

static cudaError_t compact_impl(const uint64_t* in, size_t n, uint64_t skip, const uint64_t* prev_of,
                                uint64_t* out, uint64_t* count, cudaStream_t s) {
    if (n == 0) return count ? cudaMemsetAsync(count, 0, sizeof(uint64_t), s) : cudaSuccess;
    const size_t nb = (n + kTile - 1) / kTile;
    uint64_t* part = nullptr;
    cudaError_t e = dmalloc((void**)&part, nb * sizeof(uint64_t), s);
    if (e != cudaSuccess) return e;
    launch(k_compact_count, (unsigned)nb, kThreads, 0, s, in, n, skip, prev_of, part);
    launch(k_scan_top<unsigned long long>, 1, 1024, 0, s, reinterpret_cast<unsigned long long*>(part), nb,
                                                      reinterpret_cast<unsigned long long*>(count));
    launch(k_compact_write, (unsigned)nb, kThreads, 0, s, in, n, skip, prev_of, part, out);
    e = cudaGetLastError();
    cudaFreeAsync(part, s);
    return e;
}

cudaError_t compact_u64(const uint64_t* in, size_t n, uint64_t skip, uint64_t* out, uint64_t* count,
                        cudaStream_t s) {
    return compact_impl(in, n, skip, nullptr, out, count, s);
}

cudaError_t unique_sorted_u64(uint64_t* keys, size_t n, uint64_t* count, cudaStream_t s) {
    if (n == 0) return count ? cudaMemsetAsync(count, 0, sizeof(uint64_t), s) : cudaSuccess;
    uint64_t* tmp = nullptr;
    cudaError_t e = dmalloc((void**)&tmp, n * sizeof(uint64_t), s);
    if (e != cudaSuccess) return e;
    e = compact_impl(keys, n, 0, keys, tmp, count, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(keys, tmp, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
    cudaFreeAsync(tmp, s);
    return e;
}

}  // namespace rs
