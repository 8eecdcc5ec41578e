// rs_prims.cu -- stable LSD radix sort, exclusive scans and ordered compaction.
//
// Replaces the thrust sort/unique/scan/reduce calls of the reference
// (query/src/cuda/mesh_query_deduplication.cu:56-90, scan_utils.cu:11-28) with
// the engine's own kernels.  Scan and compaction tiles are 4096 elements (256 threads
// x 16 items); the radix sort is a onesweep LSD sort whose passes rank keys per warp
// with __match_any_sync, so every pass is stable.
#include "rs_prims.cuh"

#include <algorithm>
#include <mutex>

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

// ---------------------------------------------------------------------------
// Onesweep LSD radix sort: one histogram kernel for every digit of the sort, then
// one kernel per 8-bit digit.  A block takes the next tile (ids in start order),
// counts its digits per warp, publishes the tile's per-digit counts, learns the counts
// of all earlier tiles by decoupled look-back (each status word carries a count and a
// flag: aggregate of that tile alone, or inclusive prefix through it), ranks its keys
// stably into shared memory by digit and writes them out in digit runs.  A block only
// ever waits on tiles that started before it, and every wait is bounded: past the
// limit the block records the failure in the error word and stops waiting.
// ---------------------------------------------------------------------------
constexpr int kOsItems = 12;
constexpr int kOsTile = kThreads * kOsItems;  // 3072 keys
constexpr int kOsWarpSpan = 32 * kOsItems;
constexpr int kMaxPasses = 8;
constexpr unsigned long long kFlagAgg = 1ull << 62, kFlagPre = 2ull << 62, kCountMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kLookAhead = 8;

__device__ __forceinline__ uint32_t os_digit(uint64_t k, int shift, int end_bit) {
    const int w = min(8, end_bit - shift);
    return (uint32_t)(k >> shift) & ((1u << w) - 1u);
}

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Counts of every digit of every pass (hist[p * 256 + d]).
__global__ void __launch_bounds__(kThreads) k_os_hist(const uint64_t* __restrict__ keys, size_t n, int begin_bit,
                                                       int end_bit, int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kMaxPasses * 256];
    for (int i = threadIdx.x; i < passes * 256; i += kThreads) sh[i] = 0;
    __syncthreads();
    const size_t stride = (size_t)gridDim.x * kThreads;
    for (size_t i0 = blockIdx.x * (size_t)kThreads + threadIdx.x; i0 < n; i0 += 4 * stride) {
        uint64_t k[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) k[u] = i0 + u * stride < n ? keys[i0 + u * stride] : 0ull;
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i0 + u * stride < n)
                for (int p = 0; p < passes; ++p)
                    atomicAdd(&sh[p * 256 + os_digit(k[u], begin_bit + 8 * p, end_bit)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += kThreads)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// In place: each pass's 256 counts become exclusive digit offsets (one warp per pass).
__global__ void __launch_bounds__(256) k_os_offsets(uint32_t* __restrict__ hist, int passes) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int p = w; p < passes; p += 8) {
        uint32_t* h = hist + p * 256;
        uint32_t c[8], sum = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            c[j] = h[lane * 8 + j];
            sum += c[j];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        uint32_t run = x - sum;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            h[lane * 8 + j] = run;
            run += c[j];
        }
    }
}

template <bool VALS>
__global__ void __launch_bounds__(kThreads, 4) k_os_pass(const uint64_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                                       uint32_t* __restrict__ vout, size_t n, int shift, int end_bit,
                                                       const uint32_t* __restrict__ digit_base,
                                                       unsigned long long* __restrict__ status,
                                                       unsigned int* __restrict__ tile_ctr,
                                                       uint32_t* __restrict__ err, uint32_t err_bit) {
    __shared__ uint64_t s_keys[kOsTile];
    __shared__ uint32_t s_vals[kOsTile];
    __shared__ uint32_t s_cnt[kWarps][256];
    __shared__ uint32_t s_dstart[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_wsum[kWarps];
    __shared__ unsigned int s_tile;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < kWarps * 256; i += kThreads) (&s_cnt[0][0])[i] = 0;
    __syncthreads();
    const unsigned int tile = s_tile;
    const size_t base = (size_t)tile * kOsTile + (size_t)w * kOsWarpSpan;
    uint64_t k[kOsItems];
    uint32_t v[kOsItems];
    unsigned peers[kOsItems];  // lanes of the warp holding the same digit in item r
#pragma unroll
    for (int r = 0; r < kOsItems; ++r) {
        const size_t idx = base + (size_t)r * 32 + lane;
        const bool valid = idx < n;
        k[r] = valid ? kin[idx] : 0ull;
        if (VALS) v[r] = valid ? vin[idx] : 0u;
    }
    // Per-warp digit counts (an invalid key gets a digit of its own: 256 + lane).
#pragma unroll
    for (int r = 0; r < kOsItems; ++r) {
        const bool valid = base + (size_t)r * 32 + lane < n;
        const uint32_t dg = valid ? os_digit(k[r], shift, end_bit) : (256u + lane);
        peers[r] = __match_any_sync(0xffffffffu, dg);
        if (valid && lane == __ffs(peers[r]) - 1) s_cnt[w][dg] += __popc(peers[r]);
        __syncwarp();
    }
    __syncthreads();
    // Thread d: the tile's count of digit d, per-warp offsets within the digit, publication.
    const int d = tid;
    uint32_t tc = 0;
#pragma unroll
    for (int ww = 0; ww < kWarps; ++ww) {
        const uint32_t c = s_cnt[ww][d];
        s_cnt[ww][d] = tc;
        tc += c;
    }
    unsigned long long* mine = status + (size_t)tile * 256 + d;
    st_relaxed(mine, (tile == 0 ? kFlagPre : kFlagAgg) | tc);
    // Tile-local start of each digit's run: exclusive scan of tc over the digits.
    {
        uint32_t x = tc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wsum[w] = x;
        __syncthreads();
        uint32_t before = 0;
#pragma unroll
        for (int ww = 0; ww < kWarps; ++ww)
            if (ww < w) before += s_wsum[ww];
        s_dstart[d] = before + x - tc;
    }
    // Decoupled look-back over the earlier tiles, kLookAhead status words in flight at a
    // time: aggregates are summed until an inclusive prefix is met; a word not yet
    // published stops the batch, and the walk resumes from it.
    unsigned long long prefix = 0;
    if (tile > 0) {
        long long j = (long long)tile - 1;
        uint32_t spins = 0;
        bool found = false;
        while (!found) {
            unsigned long long sv[kLookAhead];
#pragma unroll
            for (int q = 0; q < kLookAhead; ++q)
                sv[q] = (j - q >= 0) ? ld_relaxed(status + (size_t)(j - q) * 256 + d) : 0ull;
            int used = 0;
#pragma unroll
            for (int q = 0; q < kLookAhead; ++q) {
                if (found || used != q || j - q < 0) continue;
                const unsigned long long f = sv[q] & ~kCountMask;
                if (f == 0ull) continue;
                prefix += sv[q] & kCountMask;
                ++used;
                if (f == kFlagPre) found = true;
            }
            if (found) break;
            if (used == 0 && ++spins > kSpinLimit) {
                atomicOr(err, err_bit);
                break;
            }
            j -= used;
        }
        st_relaxed(mine, kFlagPre | (prefix + tc));
    }
    s_gbase[d] = digit_base[d] + (uint32_t)prefix;
    __syncthreads();
    // Stable ranks into shared memory, digit-major.
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kOsItems; ++r) {
        const bool valid = base + (size_t)r * 32 + lane < n;
        const uint32_t dg = os_digit(k[r], shift, end_bit);
        uint32_t pos = 0;
        if (valid) pos = s_dstart[dg] + s_cnt[w][dg] + __popc(peers[r] & lt);
        __syncwarp();
        if (valid && lane == __ffs(peers[r]) - 1) s_cnt[w][dg] += __popc(peers[r]);
        __syncwarp();
        if (valid) {
            s_keys[pos] = k[r];
            if (VALS) s_vals[pos] = v[r];
        }
    }
    __syncthreads();
    // Digit runs out to their global positions.
    const size_t t0 = (size_t)tile * kOsTile;
    const uint32_t tn = (uint32_t)min((size_t)kOsTile, n - t0);
    for (uint32_t i = tid; i < tn; i += kThreads) {
        const uint64_t kk = s_keys[i];
        const uint32_t dd = os_digit(kk, shift, end_bit);
        const size_t pos = (size_t)s_gbase[dd] + (i - s_dstart[dd]);
        kout[pos] = kk;
        if (VALS) vout[pos] = s_vals[i];
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

__global__ void __launch_bounds__(1024) k_sort_small(uint64_t* __restrict__ keys, int n, int swap_out) {
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
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t k = sh[i];
        keys[i] = swap_out ? (k << 32) | (k >> 32) : k;
    }
}

// The keys of a hash table (slots not equal to `empty`) appended to out in any order,
// halves swapped when swap; positions from a zeroed counter, those at or past n dropped.
__global__ void k_table_gather(const uint64_t* __restrict__ slots, uint64_t capacity, uint64_t empty, int swap,
                               uint64_t* __restrict__ out, uint64_t n, unsigned long long* __restrict__ counter) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < capacity; base += stride) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t k = i < capacity ? slots[i] : empty;
        const bool keep = k != empty;
        const unsigned int m = __ballot_sync(0xffffffffu, keep);
        if (!m) continue;
        const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
        unsigned long long pos = 0;
        if (lane == leader) pos = atomicAdd(counter, (unsigned long long)__popc(m));
        pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(m & ((1u << lane) - 1u));
        if (keep && pos < n) out[pos] = swap ? (k << 32) | (k >> 32) : k;
    }
}

}  // namespace

cudaError_t table_keys_sorted_small(const uint64_t* slots, uint64_t capacity, uint64_t empty, int swap, uint64_t* out,
                                    uint64_t n, unsigned long long* counter, cudaStream_t s) {
    if (n > (uint64_t)kSmallSort) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || n == 0) return e;
    const uint64_t blocks = std::min<uint64_t>((capacity + 255) / 256, 4ull * sm_count());
    launch(k_table_gather, (unsigned)std::max<uint64_t>(blocks, 1), 256, 0, s, slots, capacity, empty, swap, out, n,
           counter);
    launch(k_sort_small, 1, 1024, 0, s, out, (int)n, swap);
    return cudaGetLastError();
}

cudaError_t sort_u64_any(uint64_t* keys, size_t n, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    if (n <= (size_t)kSmallSort) {
        launch(k_sort_small, 1, 1024, 0, s, keys, (int)n, 0);
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

uint32_t* sort_error_word() {
    static uint32_t* words[64] = {};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!words[dev]) {
        uint32_t* p = nullptr;
        if (cudaMalloc((void**)&p, sizeof(uint32_t)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(uint32_t)) != cudaSuccess) return nullptr;
        words[dev] = p;
    }
    return words[dev];
}

namespace {
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
}  // namespace

size_t radix_sort_scratch_bytes(size_t n, int end_bit, int begin_bit, bool vals) {
    if (n <= 1 || end_bit <= begin_bit) return 0;
    const int passes = (end_bit - begin_bit + 7) / 8;
    const size_t tiles = (n + kOsTile - 1) / kOsTile;
    return align256(n * sizeof(uint64_t)) + (vals ? align256(n * sizeof(uint32_t)) : 0) +
           align256((size_t)passes * 256 * sizeof(uint32_t) + passes * sizeof(unsigned int)) +
           (size_t)passes * tiles * 256 * sizeof(unsigned long long);
}

uint32_t* radix_sort_hist(void* scratch, size_t n, bool vals) {
    char* base = static_cast<char*>(scratch) + align256(n * sizeof(uint64_t)) + (vals ? align256(n * sizeof(uint32_t)) : 0);
    return reinterpret_cast<uint32_t*>(base);
}

// The sort over caller scratch: [k2 | v2 | hist, ctr | status]; the last two regions are
// zeroed with one memset (without the histogram when the caller has filled it).
cudaError_t radix_sort_u64_in(uint64_t* keys, uint32_t* vals, size_t n, int end_bit, cudaStream_t s, int begin_bit,
                              uint32_t* err, uint32_t err_bit, void* scratch, bool hist_ready) {
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
    if (n > 0xffffffffull || end_bit > 64 || begin_bit < 0 || !scratch) return cudaErrorInvalidValue;
    if (!err) {
        err = sort_error_word();
        err_bit = 1;
        if (!err) return cudaErrorMemoryAllocation;
    }
    const int passes = (end_bit - begin_bit + 7) / 8;
    const size_t tiles = (n + kOsTile - 1) / kOsTile;
    char* base = static_cast<char*>(scratch);
    uint64_t* k2 = reinterpret_cast<uint64_t*>(base);
    base += align256(n * sizeof(uint64_t));
    uint32_t* v2 = nullptr;
    if (vals) {
        v2 = reinterpret_cast<uint32_t*>(base);
        base += align256(n * sizeof(uint32_t));
    }
    char* zero = base;
    uint32_t* hist = reinterpret_cast<uint32_t*>(base);
    unsigned int* ctr = reinterpret_cast<unsigned int*>(base + (size_t)passes * 256 * sizeof(uint32_t));
    base += align256((size_t)passes * 256 * sizeof(uint32_t) + passes * sizeof(unsigned int));
    unsigned long long* status = reinterpret_cast<unsigned long long*>(base);
    const size_t status_bytes = (size_t)passes * tiles * 256 * sizeof(unsigned long long);
    char* zero_from = hist_ready ? reinterpret_cast<char*>(ctr) : zero;
    cudaError_t e = cudaMemsetAsync(zero_from, 0, (size_t)(base - zero_from) + status_bytes, s);
    if (e == cudaSuccess) {
        if (!hist_ready) {
            const unsigned hb = (unsigned)std::min<size_t>(tiles, 4 * (size_t)sm_count());
            launch(k_os_hist, hb, kThreads, 0, s, (const uint64_t*)keys, n, begin_bit, end_bit, passes, hist);
        }
        launch(k_os_offsets, 1, 256, 0, s, hist, passes);
        e = cudaGetLastError();
    }
    uint64_t* ka = keys;
    uint64_t* kb = k2;
    uint32_t* va = vals;
    uint32_t* vb = v2;
    for (int p = 0; p < passes && e == cudaSuccess; ++p) {
        auto kern = vals ? k_os_pass<true> : k_os_pass<false>;
        launch(kern, (unsigned)tiles, kThreads, 0, s, (const uint64_t*)ka, (const uint32_t*)va, kb, vb, n,
               begin_bit + 8 * p, end_bit, (const uint32_t*)(hist + p * 256), status + (size_t)p * tiles * 256,
               ctr + p, err, err_bit);
        e = cudaGetLastError();
        uint64_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    if (e == cudaSuccess && ka != keys) {
        e = cudaMemcpyAsync(keys, ka, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && vals) e = cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
    return e;
}

cudaError_t radix_sort_u64(uint64_t* keys, uint32_t* vals, size_t n, int end_bit, cudaStream_t s, int begin_bit,
                           uint32_t* err, uint32_t err_bit) {
    const size_t bytes = radix_sort_scratch_bytes(n, end_bit, begin_bit, vals != nullptr);
    if (bytes == 0) return cudaSuccess;
    if (n > 0xffffffffull || end_bit > 64 || begin_bit < 0) return cudaErrorInvalidValue;
    void* scratch = nullptr;
    cudaError_t e = dmalloc(&scratch, bytes, s);
    if (e != cudaSuccess) return e;
    e = radix_sort_u64_in(keys, vals, n, end_bit, s, begin_bit, err, err_bit, scratch, false);
    cudaFreeAsync(scratch, s);
    return e;
}

cudaError_t sort_error_read(uint32_t* h_word, cudaStream_t s) {
    uint32_t* w = sort_error_word();
    if (!w) return cudaErrorMemoryAllocation;
    return cudaMemcpyAsync(h_word, w, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
}

cudaError_t sort_error_clear(cudaStream_t s) {
    uint32_t* w = sort_error_word();
    if (!w) return cudaErrorMemoryAllocation;
    return cudaMemsetAsync(w, 0, sizeof(uint32_t), s);
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
