// rs_mlp.cu -- learned selectivity estimator: a 32768 -> 512 -> 512 -> 1 MLP over pooled
// grid statistics, trained and evaluated with hand-written BF16 tensor-core GEMMs.
//
// The reference sizes its pair table from the grid estimator alone
// (query/src/cuda/estimated_overlap.cu:8-41, raytracer_overlap_estimated_main.cpp:252-325).
// This estimator reads the same two grids: each 128^3 GridCell grid is pooled to 16^3
// blocks x 4 channels (log1p of the CenterCount and TouchCount sums, log1p of the
// TouchCount-weighted AvgSizeMean, the TouchCount-weighted VolRatio), the two sides are
// concatenated (32768 features), and the network predicts log1p(pairs).  The reference
// GridCell carries CenterCount where a triangle count might be wanted; the features use
// the four fields the .pre file has.
//
// GEMMs: BF16 operands, FP32 accumulation.  Products whose operands are both K-major (the
// forward pass: features x W1^T, hidden x W2^T) run on tcgen05 with TMA-fed shared memory
// and tensor-memory accumulators (rs_umma.cu); the backward products, whose operands are
// stored M- or N-contiguous, run on mma.sync tiles (128x128x64, ldmatrix, cp.async stages).
// rs_mlp_set_gemm(1) sends every product to mma.sync (the tests compare the two paths).
// Weights keep an FP32 master copy (Adam) and a BF16 copy that the GEMMs read.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
// The tcgen05 GEMM (rs_umma.cu).
bool umma_gemm_fits(const void* A, int lda, const void* B, int ldb, int M, int N, int K);
cudaError_t umma_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int M,
                      int N, int K, cudaStream_t s);
cudaError_t umma_error_take(unsigned int* h_word, cudaStream_t s);

namespace {

// 0: K-major x K-major products on tcgen05 where the shapes allow, the rest on mma.sync;
// 1: every product on mma.sync (rs_mlp_set_gemm).
int g_gemm_mode = 0;

constexpr int kIn = 32768;
constexpr int kHid = 512;
constexpr int kSide = 16;                 // pooled blocks per axis
constexpr int kFeatSide = 4 * 16 * 16 * 16;  // features per grid

// ---------------------------------------------------------------------------------
// Tensor-core GEMM: C[m][n] (+)= sum_k A(m,k) B(n,k), BF16 in, FP32 out.
// A_KM: A(m,k) = A[m*lda + k] (else A[k*lda + m]); B_KM: B(n,k) = B[n*ldb + k]
// (else B[k*ldb + n]).  ATOMIC: C += with atomicAdd (split-K), else C = .
// ---------------------------------------------------------------------------------
constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Loads a BMN x BK tile of an operand into s[BMN][BK+PAD] (row = m or n, k contiguous).
template <bool KM>
__device__ __forceinline__ void load_tile(__nv_bfloat16 (*s)[BK + PAD], const __nv_bfloat16* __restrict__ g,
                                          int ld, int row0, int rows, int k0, int K) {
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    if (KM) {
        // 64 rows x 32 k: 256 vectors of 8 elements, two per thread.
        for (int v = threadIdx.x; v < BM * BK / 8; v += blockDim.x) {
            const int r = v / (BK / 8), kk = (v % (BK / 8)) * 8;
            const int gr = row0 + r, gk = k0 + kk;
            __nv_bfloat16 tmp[8];
            if (gr < rows && gk + 8 <= K && ((((uintptr_t)(g + (size_t)gr * ld + gk)) & 15) == 0)) {
                *reinterpret_cast<uint4*>(tmp) = *reinterpret_cast<const uint4*>(g + (size_t)gr * ld + gk);
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) tmp[e] = (gr < rows && gk + e < K) ? g[(size_t)gr * ld + gk + e] : zero;
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) s[r][kk + e] = tmp[e];
        }
    } else {
        // Element (row, k) at g[k*ld + row]: read along rows, store transposed.
        for (int v = threadIdx.x; v < BM * BK; v += blockDim.x) {
            const int kk = v / BM, r = v % BM;
            const int gr = row0 + r, gk = k0 + kk;
            s[r][kk] = (gr < rows && gk < K) ? g[(size_t)gk * ld + gr] : zero;
        }
    }
}

template <bool A_KM, bool B_KM, bool ATOMIC>
__global__ void __launch_bounds__(128) k_gemm(const __nv_bfloat16* __restrict__ A, int lda,
                                              const __nv_bfloat16* __restrict__ B, int ldb, float* __restrict__ C,
                                              int ldc, int M, int N, int K, int k_per_split) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int kb = blockIdx.z * k_per_split, ke = min(K, kb + k_per_split);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;
    for (int k0 = kb; k0 < ke; k0 += BK) {
        load_tile<A_KM>(As, A, lda, m0, M, k0, ke);
        load_tile<B_KM>(Bs, B, ldb, n0, N, k0, ke);
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + 16 * i + g;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * t + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + 8 * j + g;
                bf[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t]);
                bf[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = m0 + wm + 16 * i + g + (e >= 2 ? 8 : 0);
                const int c = n0 + wn + 8 * j + 2 * t + (e & 1);
                if (r < M && c < N) {
                    if (ATOMIC) atomicAdd(&C[(size_t)r * ldc + c], acc[i][j][e]);
                    else C[(size_t)r * ldc + c] = acc[i][j][e];
                }
            }
}

// ---------------------------------------------------------------------------------
// Pipelined tensor-core GEMM for 16-byte-aligned operands: 128 x 128 x 64 CTA tiles, 8
// warps of 64 x 32, three cp.async stages, fragments by ldmatrix (.trans for an operand
// stored m- or n-contiguous), mma.sync m16n8k16 BF16 with FP32 accumulation.  A K-major
// operand tile is kept as [row][k] (144-byte rows), an MN-major one as [k][row] (272-byte
// rows); both paddings make the eight 16-byte rows of each ldmatrix fall in distinct banks.
// SLAB (split K): split z writes its partial product to the z-th M x N slab of C.
// ---------------------------------------------------------------------------------
constexpr int TBM = 128, TBN = 128, TBK = 64, TST = 3, TTH = 256;
constexpr int KM_LD = TBK + 8;    // bf16 per row of a K-major tile
constexpr int MN_LD = TBM + 8;    // bf16 per row of an MN-major tile
constexpr int TILE_ELEMS = TBM * KM_LD > TBK * MN_LD ? TBM * KM_LD : TBK * MN_LD;
constexpr size_t kGemm2Smem = (size_t)2 * TST * TILE_ELEMS * sizeof(__nv_bfloat16);

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const int bytes = valid ? 16 : 0;  // 0: the 16 bytes are zero-filled, nothing is read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <bool TRANS>
__device__ __forceinline__ void ldsm_x4(uint32_t* r, const void* smem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if (TRANS)
        asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(sa));
    else
        asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(sa));
}

// One operand tile (128 rows x 64 k) of stage memory `t`: 1024 16-byte chunks, four per
// thread.
template <bool KM>
__device__ __forceinline__ void load_tile2(__nv_bfloat16* t, const __nv_bfloat16* __restrict__ g, int ld, int row0,
                                           int rows, int k0, int kend) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = threadIdx.x + q * TTH;
        if (KM) {  // element (row, k) at g[row*ld + k]; chunk = 8 consecutive k
            const int r = c >> 3, kk = (c & 7) * 8;
            const bool ok = row0 + r < rows && k0 + kk < kend;
            const __nv_bfloat16* src = ok ? g + (size_t)(row0 + r) * ld + (k0 + kk) : g;
            cp_async16(t + r * KM_LD + kk, src, ok);
        } else {   // element (row, k) at g[k*ld + row]; chunk = 8 consecutive rows
            const int kk = c >> 4, r = (c & 15) * 8;
            const bool ok = row0 + r < rows && k0 + kk < kend;
            const __nv_bfloat16* src = ok ? g + (size_t)(k0 + kk) * ld + (row0 + r) : g;
            cp_async16(t + kk * MN_LD + r, src, ok);
        }
    }
}

template <bool A_KM, bool B_KM, bool SLAB>
__global__ void __launch_bounds__(TTH) k_gemm2(const __nv_bfloat16* __restrict__ A, int lda,
                                               const __nv_bfloat16* __restrict__ B, int ldb, float* __restrict__ C,
                                               int ldc, int M, int N, int K, int k_per_split) {
    extern __shared__ __align__(16) __nv_bfloat16 smem[];
    __nv_bfloat16* As = smem;                       // TST stages
    __nv_bfloat16* Bs = smem + TST * TILE_ELEMS;    // TST stages
    const int m0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;
    const int kb = blockIdx.z * k_per_split, ke = min(K, kb + k_per_split);
    const int nk = (ke - kb + TBK - 1) / TBK;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;
    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;
    // Prologue: the first TST - 1 stages.
#pragma unroll
    for (int st = 0; st < TST - 1; ++st) {
        if (st < nk) {
            load_tile2<A_KM>(As + st * TILE_ELEMS, A, lda, m0, M, kb + st * TBK, ke);
            load_tile2<B_KM>(Bs + st * TILE_ELEMS, B, ldb, n0, N, kb + st * TBK, ke);
        }
        cp_async_commit();
    }
    // Lane addresses inside a 16 x 16 fragment block (see the fragment layouts of
    // mma.m16n8k16): A K-major (row, k), A MN-major (k, row), B K-major, B MN-major.
    const int a_r = A_KM ? (lane & 15) : (((lane >> 3) & 1) * 8);
    const int a_k = A_KM ? ((lane >> 4) * 8) : ((lane & 7) + ((lane >> 4) << 3));
    const int b_r = B_KM ? ((lane & 7) + ((lane >> 4) << 3)) : ((lane >> 4) * 8);
    const int b_k = B_KM ? (((lane >> 3) & 1) * 8) : (lane & 15);
    for (int it = 0; it < nk; ++it) {
        cp_async_wait<TST - 2>();
        __syncthreads();
        {   // refill the stage consumed TST - 1 iterations ago
            const int nxt = it + TST - 1;
            if (nxt < nk) {
                load_tile2<A_KM>(As + (nxt % TST) * TILE_ELEMS, A, lda, m0, M, kb + nxt * TBK, ke);
                load_tile2<B_KM>(Bs + (nxt % TST) * TILE_ELEMS, B, ldb, n0, N, kb + nxt * TBK, ke);
            }
            cp_async_commit();
        }
        const __nv_bfloat16* at = As + (it % TST) * TILE_ELEMS;
        const __nv_bfloat16* bt = Bs + (it % TST) * TILE_ELEMS;
#pragma unroll
        for (int ks = 0; ks < TBK; ks += 16) {
            uint32_t af[4][4], bfr[2][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = wm + 16 * i + a_r, k = ks + a_k;
                ldsm_x4<!A_KM>(af[i], A_KM ? at + r * KM_LD + k : at + k * MN_LD + r);
            }
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int r = wn + 16 * j + b_r, k = ks + b_k;
                ldsm_x4<!B_KM>(bfr[j], B_KM ? bt + r * KM_LD + k : bt + k * MN_LD + r);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t bb[2] = {bfr[j >> 1][(j & 1) * 2], bfr[j >> 1][(j & 1) * 2 + 1]};
                    mma_bf16(acc[i][j], af[i], bb);
                }
        }
    }
    cp_async_wait<0>();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = m0 + wm + 16 * i + g + (e >= 2 ? 8 : 0);
                const int c = n0 + wn + 8 * j + 2 * t + (e & 1);
                // PARTIAL (split K): each split writes its own M x N slab of C.
                if (r < M && c < N) C[(SLAB ? (size_t)blockIdx.z * M * ldc : 0) + (size_t)r * ldc + c] = acc[i][j][e];
            }
}

// Sum of the split-K slabs: C[r][c] = sum_z W[z][r][c] (W rows of ldw).
__global__ void k_splitk_sum(const float* __restrict__ W, int split, int M, int N, int ldw, float* __restrict__ C,
                             int ldc) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)M * N) return;
    const int r = (int)(i / N), c = (int)(i % N);
    float sum = 0.0f;
    for (int z = 0; z < split; ++z) sum += W[((size_t)z * M + r) * ldw + c];
    C[(size_t)r * ldc + c] = sum;
}

// The pipelined kernel needs 16-byte chunks along each operand's contiguous dimension.
template <bool KM>
bool chunkable(const __nv_bfloat16* p, int ld, int rows, int K) {
    if ((reinterpret_cast<uintptr_t>(p) & 15) || (ld % 8)) return false;
    return KM ? (K % 8 == 0) : (rows % 8 == 0);
}

template <bool A_KM, bool B_KM>
void gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int M, int N, int K,
          cudaStream_t s) {
    if (A_KM && B_KM && g_gemm_mode == 0 && umma_gemm_fits(A, lda, B, ldb, M, N, K) &&
        umma_gemm(A, lda, B, ldb, C, ldc, M, N, K, s) == cudaSuccess)
        return;
    if (chunkable<A_KM>(A, lda, M, K) && chunkable<B_KM>(B, ldb, N, K)) {
        static bool attr_set[64] = {};  // the kernels' shared-memory opt-in, once per device
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev >= 0 && dev < 64 && !attr_set[dev]) {
            cudaFuncSetAttribute(k_gemm2<A_KM, B_KM, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kGemm2Smem);
            cudaFuncSetAttribute(k_gemm2<A_KM, B_KM, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kGemm2Smem);
            attr_set[dev] = true;
        }
        const int tiles2 = ((M + TBM - 1) / TBM) * ((N + TBN - 1) / TBN);
        int split2 = 1;
        const int target2 = 2 * sm_count();
        while (tiles2 * split2 < target2 && K / (split2 * 2) >= 4 * TBK) split2 *= 2;
        int kps2 = (K + split2 - 1) / split2;
        kps2 = (kps2 + TBK - 1) / TBK * TBK;
        split2 = (K + kps2 - 1) / kps2;
        const dim3 grid2((N + TBN - 1) / TBN, (M + TBM - 1) / TBM, split2);
        float* ws = nullptr;
        const int ptok = prof_begin(P_GEMM, s);
        if (split2 > 1 && dmalloc((void**)&ws, (size_t)split2 * M * N * sizeof(float), s) == cudaSuccess) {
            // Split K: each split writes its own slab of the workspace, then one pass sums them
            // (in split order, so the result does not depend on scheduling).
            launch(k_gemm2<A_KM, B_KM, true>, grid2, TTH, kGemm2Smem, s, A, lda, B, ldb, ws, N, M, N, K, kps2);
            launch(k_splitk_sum, (unsigned)(((uint64_t)M * N + 255) / 256), 256, 0, s, (const float*)ws, split2, M, N,
                   N, C, ldc);
            cudaFreeAsync(ws, s);
        } else if (split2 > 1) {
            launch(k_gemm2<A_KM, B_KM, false>, dim3(grid2.x, grid2.y, 1), TTH, kGemm2Smem, s, A, lda, B, ldb, C, ldc,
                   M, N, K, K);
        } else {
            launch(k_gemm2<A_KM, B_KM, false>, grid2, TTH, kGemm2Smem, s, A, lda, B, ldb, C, ldc, M, N, K, kps2);
        }
        prof_end(P_GEMM, s, ptok);
        return;
    }
    const int tiles = ((M + BM - 1) / BM) * ((N + BN - 1) / BN);
    int split = 1;
    const int target = 2 * sm_count();
    while (tiles * split < target && K / (split * 2) >= 4 * BK) split *= 2;
    int kps = (K + split - 1) / split;
    kps = (kps + BK - 1) / BK * BK;
    split = (K + kps - 1) / kps;
    const dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, split);
    if (split > 1) {
        if (ldc == N) cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), s);
        else
            for (int r = 0; r < M; ++r) cudaMemsetAsync(C + (size_t)r * ldc, 0, N * sizeof(float), s);
        launch(k_gemm<A_KM, B_KM, true>, grid, 128, 0, s, A, lda, B, ldb, C, ldc, M, N, K, kps);
    } else {
        launch(k_gemm<A_KM, B_KM, false>, grid, 128, 0, s, A, lda, B, ldb, C, ldc, M, N, K, kps);
    }
}

// ---------------------------------------------------------------------------------
// Elementwise and reduction kernels.
// ---------------------------------------------------------------------------------
// Four elements per thread: one 16-byte load and one 8-byte store when both arrays are
// aligned for them, element by element otherwise (and for the tail).
__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, uint64_t n) {
    const uint64_t i = 4 * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
    if (i >= n) return;
    const bool vec = ((reinterpret_cast<uintptr_t>(x) & 15) == 0) && ((reinterpret_cast<uintptr_t>(y) & 7) == 0);
    if (vec && i + 4 <= n) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(x + i));
        const __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
        uint2 w;
        w.x = *reinterpret_cast<const uint32_t*>(&lo);
        w.y = *reinterpret_cast<const uint32_t*>(&hi);
        *reinterpret_cast<uint2*>(y + i) = w;
    } else {
        for (uint64_t k = i; k < n && k < i + 4; ++k) y[k] = __float2bfloat16_rn(x[k]);
    }
}

// h = relu(h + bias) in place (rows x cols), with a BF16 copy.
__global__ void k_bias_relu(float* __restrict__ h, const float* __restrict__ bias, __nv_bfloat16* __restrict__ hb,
                            int rows, int cols) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)rows * cols) return;
    const float v = fmaxf(h[i] + bias[i % cols], 0.0f);
    h[i] = v;
    hb[i] = __float2bfloat16_rn(v);
}

// y[b] = dot(h2[b], w3) + b3 with the BF16-rounded operands the GEMMs would use.
__global__ void k_head(const __nv_bfloat16* __restrict__ h2, const float* __restrict__ w3, const float* __restrict__ b3,
                       float* __restrict__ y, int B) {
    const int b = blockIdx.x;
    float acc = 0.0f;
    for (int i = threadIdx.x; i < kHid; i += blockDim.x)
        acc += __bfloat162float(h2[(size_t)b * kHid + i]) * __bfloat162float(__float2bfloat16_rn(w3[i]));
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0 && b < B) y[b] = red[0] + b3[0];
}

// Loss and output gradient: dy = 2 (y - t) / B; loss = mean (y - t)^2.
__global__ void k_loss(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                       float* __restrict__ loss, int B) {
    __shared__ float red[256];
    float acc = 0.0f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) {
        const float d = y[b] - t[b];
        dy[b] = 2.0f * d / (float)B;
        acc += d * d;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)B;
}

// dW3[i] = sum_b dy[b] h2[b][i]; db3 = sum_b dy[b]; dh2[b][i] = dy[b] w3[i] [h2 > 0].
__global__ void k_head_back(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ h2,
                            const float* __restrict__ h2f, const float* __restrict__ w3, float* __restrict__ gw3,
                            float* __restrict__ gb3, float* __restrict__ dh2, __nv_bfloat16* __restrict__ dh2b,
                            int B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kHid) {
        float acc = 0.0f;
        const float w = __bfloat162float(__float2bfloat16_rn(w3[i]));
        for (int b = 0; b < B; ++b) {
            acc += dy[b] * __bfloat162float(h2[(size_t)b * kHid + i]);
            const float d = h2f[(size_t)b * kHid + i] > 0.0f ? dy[b] * w : 0.0f;
            dh2[(size_t)b * kHid + i] = d;
            dh2b[(size_t)b * kHid + i] = __float2bfloat16_rn(d);
        }
        gw3[i] = acc;
    }
    if (i == 0) {
        float acc = 0.0f;
        for (int b = 0; b < B; ++b) acc += dy[b];
        gb3[0] = acc;
    }
}

// Column sums: g[c] = sum_r x[r][c].
__global__ void k_colsum(const float* __restrict__ x, float* __restrict__ g, int rows, int cols) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float acc = 0.0f;
    for (int r = 0; r < rows; ++r) acc += x[(size_t)r * cols + c];
    g[c] = acc;
}

// d[r][c] *= [h[r][c] > 0], with a BF16 copy.
__global__ void k_relu_back(float* __restrict__ d, const float* __restrict__ h, __nv_bfloat16* __restrict__ db,
                            uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = h[i] > 0.0f ? d[i] : 0.0f;
    d[i] = v;
    db[i] = __float2bfloat16_rn(v);
}

// Adam (Kingma & Ba 2015) over all parameters, refreshing the BF16 copies of W1, W2.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, uint64_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ w1h, uint64_t n_w1, __nv_bfloat16* __restrict__ w2h,
                       uint64_t w2_off, uint64_t n_w2, float wd, uint64_t w3_off, uint64_t n_w3) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    // Decoupled weight decay (Loshchilov & Hutter 2019) on the weight matrices only.
    const bool weight = i < n_w1 || (i >= w2_off && i < w2_off + n_w2) || (i >= w3_off && i < w3_off + n_w3);
    const float p0 = weight ? p[i] * (1.0f - lr * wd) : p[i];
    const float pi = p0 - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (i < n_w1) w1h[i] = __float2bfloat16_rn(pi);
    else if (i >= w2_off && i < w2_off + n_w2) w2h[i - w2_off] = __float2bfloat16_rn(pi);
}

// Deterministic uniform(-bound, bound) initialisation from a counter hash (splitmix64).
__global__ void k_init(float* __restrict__ p, uint64_t n, float bound, uint64_t seed) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t z = seed + (i + 1) * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    const float u = (float)((z >> 40) & 0xffffff) / 16777216.0f;  // [0,1)
    p[i] = (2.0f * u - 1.0f) * bound;
}

// Pooled features of one grid into f[4][16][16][16].
__global__ void k_pool(const uint4* __restrict__ cells, int R, float* __restrict__ f) {
    const int blk = blockIdx.x * blockDim.x + threadIdx.x;
    if (blk >= kSide * kSide * kSide) return;
    const int bx = blk % kSide, by = (blk / kSide) % kSide, bz = blk / (kSide * kSide);
    const int x0 = (bx * R + kSide - 1) / kSide, x1 = ((bx + 1) * R + kSide - 1) / kSide;
    const int y0 = (by * R + kSide - 1) / kSide, y1 = ((by + 1) * R + kSide - 1) / kSide;
    const int z0 = (bz * R + kSide - 1) / kSide, z1 = ((bz + 1) * R + kSide - 1) / kSide;
    double cc = 0.0, tc = 0.0, sa = 0.0, sr = 0.0;
    for (int z = z0; z < z1; ++z)
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) {
                const uint4 c = cells[((size_t)z * R + y) * R + x];
                cc += (double)c.x;
                tc += (double)c.y;
                sa += (double)c.y * (double)__uint_as_float(c.z);
                sr += (double)c.y * (double)__uint_as_float(c.w);
            }
    const int n3 = kSide * kSide * kSide;
    f[blk] = (float)log1p(cc);
    f[n3 + blk] = (float)log1p(tc);
    f[2 * n3 + blk] = tc > 0.0 ? (float)log1p(sa / tc) : 0.0f;
    f[3 * n3 + blk] = tc > 0.0 ? (float)(sr / tc) : 0.0f;
}

}  // namespace
}  // namespace rs

using namespace rs;

struct rs_mlp {
    // Parameters, gradients and Adam moments, each one contiguous FP32 array:
    // W1 [512][32768], b1 [512], W2 [512][512], b2 [512], W3 [512], b3 [1].
    float* p = nullptr;
    float* g = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    uint64_t n = 0;
    __nv_bfloat16* w1h = nullptr;
    __nv_bfloat16* w2h = nullptr;
    int step = 0;
    // Activations of the last forward pass (batch capacity cap).
    int cap = 0;
    __nv_bfloat16 *xh = nullptr, *h1h = nullptr, *h2h = nullptr, *d2h = nullptr, *d1h = nullptr;
    float *h1 = nullptr, *h2 = nullptr, *y = nullptr, *dy = nullptr, *d2 = nullptr, *d1 = nullptr, *loss = nullptr;
    float* feat = nullptr;  // one feature vector for rs_estimate_mlp
    int device = 0;
    // Decoupled weight decay of W1, W2, W3 (rs_mlp_set_weight_decay).
    float weight_decay = 0.0f;
    // Grid-estimator prior (rs_mlp_set_prior): the network's output is a correction added
    // to log1p of the grid estimate of the same two grids, in rs_estimate_mlp.
    int prior = 0;
    float prior_cell_volume = 0.0f, prior_eps = 0.001f, prior_gamma = 0.8f;
    int prior_alpha = 1;
};

namespace {

constexpr uint64_t oW1 = 0, oB1 = (uint64_t)kIn * kHid, oW2 = oB1 + kHid, oB2 = oW2 + (uint64_t)kHid * kHid,
                   oW3 = oB2 + kHid, oB3 = oW3 + kHid, kParams = oB3 + 1;

void free_acts(rs_mlp* h) {
    for (void* q : {(void*)h->xh, (void*)h->h1h, (void*)h->h2h, (void*)h->d2h, (void*)h->d1h, (void*)h->h1,
                    (void*)h->h2, (void*)h->y, (void*)h->dy, (void*)h->d2, (void*)h->d1})
        if (q) cudaFree(q);
    h->xh = h->h1h = h->h2h = h->d2h = h->d1h = nullptr;
    h->h1 = h->h2 = h->y = h->dy = h->d2 = h->d1 = nullptr;
    h->cap = 0;
}

cudaError_t ensure_acts(rs_mlp* h, int B) {
    if (B <= h->cap) return cudaSuccess;
    free_acts(h);
    const size_t b = (size_t)B;
    cudaError_t e = cudaMalloc((void**)&h->xh, b * kIn * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->h1h, b * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->h2h, b * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d2h, b * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d1h, b * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->h1, b * kHid * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->h2, b * kHid * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->y, b * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->dy, b * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d2, b * kHid * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d1, b * kHid * 4);
    if (e != cudaSuccess) {
        free_acts(h);
        return e;
    }
    h->cap = B;
    return cudaSuccess;
}

unsigned blocks(uint64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Forward pass on B feature rows (FP32, row-major [B][32768]); outputs in h->y.
cudaError_t forward(rs_mlp* h, const float* X, int B, cudaStream_t s) {
    cudaError_t e = ensure_acts(h, B);
    if (e != cudaSuccess) return e;
    launch(k_to_bf16, blocks(((uint64_t)B * kIn + 3) / 4), 256, 0, s, X, h->xh, (uint64_t)B * kIn);
    gemm<true, true>(h->xh, kIn, h->w1h, kIn, h->h1, kHid, B, kHid, kIn, s);
    launch(k_bias_relu, blocks((uint64_t)B * kHid), 256, 0, s, h->h1, (const float*)(h->p + oB1), h->h1h, B, kHid);
    gemm<true, true>(h->h1h, kHid, h->w2h, kHid, h->h2, kHid, B, kHid, kHid, s);
    launch(k_bias_relu, blocks((uint64_t)B * kHid), 256, 0, s, h->h2, (const float*)(h->p + oB2), h->h2h, B, kHid);
    launch(k_head, B, 256, 0, s, (const __nv_bfloat16*)h->h2h, (const float*)(h->p + oW3), (const float*)(h->p + oB3),
           h->y, B);
    return cudaGetLastError();
}

// Backward pass after forward(): gradients into h->g, loss into h->loss[0].
cudaError_t backward(rs_mlp* h, const float* target, int B, cudaStream_t s) {
    launch(k_loss, 1, 256, 0, s, (const float*)h->y, target, h->dy, h->loss, B);
    launch(k_head_back, blocks(kHid), 256, 0, s, (const float*)h->dy, (const __nv_bfloat16*)h->h2h,
           (const float*)h->h2, (const float*)(h->p + oW3), h->g + oW3, h->g + oB3, h->d2, h->d2h, B);
    // dW2[o][i] = sum_b d2[b][o] h1[b][i];  db2 = column sums of d2.
    gemm<false, false>(h->d2h, kHid, h->h1h, kHid, h->g + oW2, kHid, kHid, kHid, B, s);
    launch(k_colsum, blocks(kHid), 256, 0, s, (const float*)h->d2, h->g + oB2, B, kHid);
    // d1[b][i] = sum_o d2[b][o] W2[o][i], masked by relu'.
    gemm<true, false>(h->d2h, kHid, h->w2h, kHid, h->d1, kHid, B, kHid, kHid, s);
    launch(k_relu_back, blocks((uint64_t)B * kHid), 256, 0, s, h->d1, (const float*)h->h1, h->d1h,
           (uint64_t)B * kHid);
    // dW1[o][j] = sum_b d1[b][o] x[b][j];  db1 = column sums of d1.
    gemm<false, false>(h->d1h, kHid, h->xh, kIn, h->g + oW1, kIn, kHid, kIn, B, s);
    launch(k_colsum, blocks(kHid), 256, 0, s, (const float*)h->d1, h->g + oB1, B, kHid);
    return cudaGetLastError();
}

}  // namespace

extern "C" int rs_mlp_create(uint64_t seed, rs_mlp** out) {
    if (!out) return RS_ERR_INVALID;
    rs_mlp* h = new rs_mlp();
    cudaGetDevice(&h->device);
    h->n = kParams;
    cudaError_t e = cudaMalloc((void**)&h->p, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->g, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->m, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->v, kParams * 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->w1h, (size_t)kIn * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->w2h, (size_t)kHid * kHid * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->loss, 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->feat, 2 * kFeatSide * 4);
    if (e == cudaSuccess) e = cudaMemset(h->p, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(h->m, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(h->v, 0, kParams * 4);
    if (e == cudaSuccess) e = cudaMemset(h->g, 0, kParams * 4);
    if (e != cudaSuccess) {
        rs_mlp* tmp = h;
        for (void* q : {(void*)tmp->p, (void*)tmp->g, (void*)tmp->m, (void*)tmp->v, (void*)tmp->w1h, (void*)tmp->w2h,
                        (void*)tmp->loss, (void*)tmp->feat})
            if (q) cudaFree(q);
        delete tmp;
        return to_status(e);
    }
    // Uniform(+-1/sqrt(fan_in)) weights and biases (PyTorch's Linear default range).
    const float s1 = 1.0f / std::sqrt((float)kIn), s2 = 1.0f / std::sqrt((float)kHid);
    launch(k_init, blocks(oB1), 256, 0, nullptr, h->p + oW1, oB1, s1, seed * 4 + 1);
    launch(k_init, blocks(kHid), 256, 0, nullptr, h->p + oB1, (uint64_t)kHid, s1, seed * 4 + 2);
    launch(k_init, blocks((uint64_t)kHid * kHid + kHid), 256, 0, nullptr, h->p + oW2, (uint64_t)kHid * kHid + kHid, s2,
           seed * 4 + 3);
    launch(k_init, blocks(kHid + 1), 256, 0, nullptr, h->p + oW3, (uint64_t)kHid + 1, s2, seed * 4 + 4);
    launch(k_to_bf16, blocks((oB1 + 3) / 4), 256, 0, nullptr, (const float*)(h->p + oW1), h->w1h, oB1);
    launch(k_to_bf16, blocks(((uint64_t)kHid * kHid + 3) / 4), 256, 0, nullptr, (const float*)(h->p + oW2), h->w2h,
           (uint64_t)kHid * kHid);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return to_status(e);
    *out = h;
    return RS_OK;
}

extern "C" int rs_mlp_destroy(rs_mlp* h) {
    if (!h) return RS_OK;
    free_acts(h);
    for (void* q : {(void*)h->p, (void*)h->g, (void*)h->m, (void*)h->v, (void*)h->w1h, (void*)h->w2h, (void*)h->loss,
                    (void*)h->feat})
        if (q) cudaFree(q);
    delete h;
    return RS_OK;
}

extern "C" uint64_t rs_mlp_num_params(void) { return kParams; }

extern "C" int rs_mlp_get_params(const rs_mlp* h, float* h_params, float* h_grads) {
    if (!h) return RS_ERR_INVALID;
    cudaError_t e = cudaSuccess;
    if (h_params) e = cudaMemcpy(h_params, h->p, kParams * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h_grads) e = cudaMemcpy(h_grads, h->g, kParams * 4, cudaMemcpyDeviceToHost);
    return to_status(e);
}

extern "C" int rs_mlp_set_params(rs_mlp* h, const float* h_params) {
    if (!h || !h_params) return RS_ERR_INVALID;
    cudaError_t e = cudaMemcpy(h->p, h_params, kParams * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return to_status(e);
    launch(k_to_bf16, blocks((oB1 + 3) / 4), 256, 0, nullptr, (const float*)(h->p + oW1), h->w1h, oB1);
    launch(k_to_bf16, blocks(((uint64_t)kHid * kHid + 3) / 4), 256, 0, nullptr, (const float*)(h->p + oW2), h->w2h,
           (uint64_t)kHid * kHid);
    return to_status(cudaDeviceSynchronize());
}

extern "C" int rs_mlp_features(const void* d_cellsA, const void* d_cellsB, int resolution, float* d_out, void* stream) {
    if (!d_cellsA || !d_cellsB || !d_out || resolution < 1) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = kSide * kSide * kSide;
    launch(k_pool, blocks(nb, 128), 128, 0, s, (const uint4*)d_cellsA, resolution, d_out);
    launch(k_pool, blocks(nb, 128), 128, 0, s, (const uint4*)d_cellsB, resolution, d_out + kFeatSide);
    return to_status(cudaGetLastError());
}

// Status of a finished call: a CUDA error, or RS_ERR_ITER_LIMIT when a tcgen05 GEMM wait ran
// out (its products are then incomplete).
static int mlp_status(cudaError_t e, cudaStream_t s) {
    if (e != cudaSuccess) return to_status(e);
    if (g_gemm_mode != 0) return RS_OK;
    unsigned int w = 0;
    e = umma_error_take(&w, s);
    if (e != cudaSuccess) return to_status(e);
    return w ? RS_ERR_ITER_LIMIT : RS_OK;
}

extern "C" int rs_mlp_set_gemm(int mode) {
    if (mode != 0 && mode != 1) return RS_ERR_INVALID;
    g_gemm_mode = mode;
    return RS_OK;
}

extern "C" int rs_mlp_gemm(const void* d_A, int lda, const void* d_B, int ldb, float* d_C, int ldc, int M, int N,
                           int K, int mode, void* stream) {
    if (!d_A || !d_B || !d_C || M <= 0 || N <= 0 || K <= 0 || (mode != 0 && mode != 1)) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const __nv_bfloat16* A = static_cast<const __nv_bfloat16*>(d_A);
    const __nv_bfloat16* B = static_cast<const __nv_bfloat16*>(d_B);
    cudaError_t e;
    if (mode == 0) {
        if (!umma_gemm_fits(A, lda, B, ldb, M, N, K)) return RS_ERR_INVALID;
        e = umma_gemm(A, lda, B, ldb, d_C, ldc, M, N, K, s);
    } else {
        const int saved = g_gemm_mode;
        g_gemm_mode = 1;
        gemm<true, true>(A, lda, B, ldb, d_C, ldc, M, N, K, s);
        g_gemm_mode = saved;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return to_status(e);
    if (mode == 0) {
        unsigned int w = 0;
        e = umma_error_take(&w, s);
        if (e != cudaSuccess) return to_status(e);
        if (w) return RS_ERR_ITER_LIMIT;
    }
    return RS_OK;
}

extern "C" int rs_mlp_forward(rs_mlp* h, const float* d_X, int B, float* d_y, void* stream) {
    if (!h || !d_X || B <= 0) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = forward(h, d_X, B, s);
    if (e == cudaSuccess && d_y) e = cudaMemcpyAsync(d_y, h->y, B * 4, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return mlp_status(e, s);
}

extern "C" int rs_mlp_gradients(rs_mlp* h, const float* d_X, const float* d_target, int B, float* h_loss,
                                void* stream) {
    if (!h || !d_X || !d_target || B <= 0) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = forward(h, d_X, B, s);
    if (e == cudaSuccess) e = backward(h, d_target, B, s);
    if (e == cudaSuccess && h_loss) e = cudaMemcpyAsync(h_loss, h->loss, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return mlp_status(e, s);
}

extern "C" int rs_mlp_train_step(rs_mlp* h, const float* d_X, const float* d_target, int B, float lr, float* h_loss,
                                 void* stream) {
    if (!h || !d_X || !d_target || B <= 0) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = forward(h, d_X, B, s);
    if (e == cudaSuccess) e = backward(h, d_target, B, s);
    if (e != cudaSuccess) return to_status(e);
    ++h->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)h->step), c2 = 1.0f - std::pow(b2, (float)h->step);
    launch(k_adam, blocks(kParams), 256, 0, s, h->p, (const float*)h->g, h->m, h->v, kParams, lr, b1, b2, 1e-8f, c1,
           c2, h->w1h, oB1, h->w2h, oW2, (uint64_t)kHid * kHid, h->weight_decay, oW3, (uint64_t)kHid);
    e = cudaGetLastError();
    if (e == cudaSuccess && h_loss) e = cudaMemcpyAsync(h_loss, h->loss, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return mlp_status(e, s);
}

extern "C" int rs_estimate_mlp(rs_mlp* h, const void* d_cellsA, const void* d_cellsB, int resolution,
                               int64_t* h_estimate, double* h_log1p, void* stream) {
    if (!h || !h_estimate) return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    int st = rs_mlp_features(d_cellsA, d_cellsB, resolution, h->feat, stream);
    if (st != RS_OK) return st;
    cudaError_t e = forward(h, h->feat, 1, s);
    float y = 0.0f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&y, h->y, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = mlp_status(e, s);
    if (st != RS_OK) return st;
    double base = 0.0;
    if (h->prior) {
        // The grid estimator's count on the same grids (rs_estimate_grid and
        // rs_estimate_pairs_from_raw), the prior the network corrects.
        double raw = 0.0;
        float means[4];
        const uint64_t ncells = (uint64_t)resolution * resolution * resolution;
        st = rs_estimate_grid(d_cellsA, d_cellsB, ncells, h->prior_cell_volume, h->prior_eps, h->prior_gamma, &raw,
                              means, stream);
        if (st != RS_OK) return st;
        const int64_t g = rs_estimate_pairs_from_raw(raw, means, h->prior_cell_volume, h->prior_alpha);
        base = std::log1p((double)std::max<int64_t>(g, 0));
    }
    const double v = std::expm1((double)y + base);
    *h_estimate = v > 0.0 ? (int64_t)std::llround(v) : 0;
    if (h_log1p) *h_log1p = (double)y + base;
    return RS_OK;
}

extern "C" int rs_mlp_set_weight_decay(rs_mlp* h, float weight_decay) {
    if (!h || !(weight_decay >= 0.0f)) return RS_ERR_INVALID;
    h->weight_decay = weight_decay;
    return RS_OK;
}

extern "C" int rs_mlp_set_prior(rs_mlp* h, int on, float cell_volume, float epsilon, float gamma,
                                int alpha_correction) {
    if (!h || (on && !(cell_volume > 0.0f))) return RS_ERR_INVALID;
    h->prior = on != 0;
    h->prior_cell_volume = cell_volume;
    h->prior_eps = epsilon;
    h->prior_gamma = gamma;
    h->prior_alpha = alpha_correction != 0;
    return RS_OK;
}
