// rs_umma.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05) for the learned
// estimator: C[m][n] = sum_k A[m][k] B[n][k], both operands K-major (row-major with k
// contiguous), FP32 accumulation in tensor memory.
//
// One CTA computes a 128 x 256 tile of C over a range of 64-wide k-blocks.  Warp 0's
// elected thread streams the operand tiles into a 4-stage shared-memory ring with TMA
// (cp.async.bulk.tensor, 128-byte swizzle, one 64-element row of 128 bytes per tile row);
// warp 1's elected thread issues tcgen05.mma (M 128, N 256, K 16) from shared-memory
// descriptors into a 256-column FP32 accumulator in tensor memory, and each commit
// returns its stage to the producer; at the end all four warps read the accumulator back
// with tcgen05.ld (warp w owns rows 32w..32w+31) and store it.  Splits of K write their own
// slab of a workspace, summed in split order by the caller (deterministic results).
//
// Every wait is bounded: a wait that runs out records an error bit, the CTA skips its
// remaining work, waits (bounded) for the copies and products it issued, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int UM = 128, UN = 256, UK = 64;  // CTA tile and k-block
constexpr int kStages = 4;
constexpr int kATile = UM * UK * 2;  // 16 KB
constexpr int kBTile = UN * UK * 2;  // 32 KB
constexpr int kStageBytes = kATile + kBTile;
constexpr size_t kUmmaSmem = (size_t)kStages * kStageBytes + 1024;  // + alignment slack
constexpr int kTmemCols = 256;
constexpr uint32_t kSpin = 1u << 20;  // polls of one wait before it gives up

// Instruction descriptor of tcgen05.mma kind::f16: D F32 (bits 4-5 = 1), A BF16 (bits 7-9 =
// 1), B BF16 (bits 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at 24.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(UN >> 3) << 17) |
                            ((uint32_t)(UM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Waits (bounded) for the completion of the phase of `bar` with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < kSpin; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile stored as rows of 64 BF16 (128
// bytes) with the 128-byte swizzle: start address >> 4 (bits 0-13), leading byte offset 16 >> 4
// (unused by swizzled K-major layouts), stride byte offset 1024 >> 4 (8 rows of 128 bytes, bits
// 32-45), descriptor version 1 (bit 46), swizzle mode 2 = 128 bytes (bits 61-63).  The tile base
// is 1024-byte aligned, so the base offset (bits 49-51) is 0.
__device__ __forceinline__ uint64_t tile_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive accumulator columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// C (or split z's slab of the workspace) tile (blockIdx.y, blockIdx.x) over k-blocks
// [z * kps, min(total, (z + 1) * kps)).  Rows m >= M are not stored.  err: device word, bit 0
// set when a wait ran out.
__global__ void __launch_bounds__(128, 1) k_umma_gemm(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, float* __restrict__ C,
                                                      int ldc, size_t slab, int M, int kps, int total,
                                                      unsigned int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * UN, m0 = blockIdx.y * UM;
    const int kb0 = blockIdx.z * kps, kb1 = min(total, kb0 + kps);
    const int nkb = kb1 - kb0;
    float* Cz = C + (size_t)blockIdx.z * slab;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = s_tmem;

    // The producer and issuer roles belong to whole warps: lane 0 works, lanes 1-31 wait at
    // the warp's reconvergence point instead of polling `done` in a branch that would share
    // the warp's issue slots with lane 0's loop.
    int issued_tma = 0;  // k-blocks whose copies the producer issued
    if (warp == 0 && nkb > 0) {
        if (lane == 0) {
            // Producer: stage s = i % kStages, round r = i / kStages; a round r >= 1 waits for the
            // products of round r - 1 to release the stage.
            for (int i = 0; i < nkb; ++i) {
                const int s = i % kStages, r = i / kStages;
                if (r > 0 && !mbar_wait(&empty[s], (uint32_t)((r - 1) & 1))) {
                    atomicOr(err, 1u);
                    atomicExch(&s_abort, 1);
                    break;
                }
                if (*(volatile int*)&s_abort) break;
                uint8_t* a = smem + (size_t)s * kStageBytes;
                mbar_expect_tx(&full[s], kStageBytes);
                tma_load_2d(a, &tmA, &full[s], (kb0 + i) * UK, m0);
                tma_load_2d(a + kATile, &tmB, &full[s], (kb0 + i) * UK, n0);
                issued_tma = i + 1;
            }
        }
        __syncwarp();
    } else if (warp == 1 && nkb > 0) {
        if (lane == 0) {
            // Issuer: four K=16 products per k-block; the commit frees the stage once they finish.
            for (int i = 0; i < nkb; ++i) {
                const int s = i % kStages, r = i / kStages;
                if (!mbar_wait(&full[s], (uint32_t)(r & 1))) {
                    atomicOr(err, 1u);
                    atomicExch(&s_abort, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a = smem_u32(smem + (size_t)s * kStageBytes);
                const uint64_t da = tile_desc(a), db = tile_desc(a + kATile);
#pragma unroll
                for (int j = 0; j < UK / 16; ++j)  // 16 BF16 = 32 bytes = 2 in the address field
                    umma_bf16(taddr, da + 2 * j, db + 2 * j, (i > 0 || j > 0) ? 1u : 0u);
                umma_commit(&empty[s]);
            }
            umma_commit(&done);  // arrives when every product issued above has finished
        }
        __syncwarp();
    }
    // Every thread waits for the last products (the issuer commits `done` even after an
    // abort, covering whatever it issued).
    const bool ok = nkb > 0 ? mbar_wait(&done, 0) : true;
    if (!ok) {
        atomicOr(err, 1u);
        atomicExch(&s_abort, 1);
    }
    __syncthreads();
    if (s_abort && warp == 0 && lane == 0) {
        // After an abort, copies may still be in flight into the ring: wait (bounded) for the
        // last kStages k-blocks the producer issued before leaving the shared memory.
        for (int i = max(0, issued_tma - kStages); i < issued_tma; ++i)
            mbar_wait(&full[i % kStages], (uint32_t)((i / kStages) & 1));
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_abort && nkb > 0) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c = 0; c < UN / 32; ++c) {
            float v[32];
            tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
            if (row < M) {
                float4* dst = reinterpret_cast<float4*>(Cz + (size_t)row * ldc + n0 + c * 32);
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
    }
}

// Sum of split-K slabs in split order: C[r][c] = sum_z W[z][r][c].
__global__ void k_umma_sum(const float* __restrict__ W, int split, int M, int N, float* __restrict__ C, int ldc) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)M * N) return;
    const int r = (int)(i / N), c = (int)(i % N);
    float acc = 0.0f;
    for (int z = 0; z < split; ++z) acc += W[(size_t)z * M * N + i];
    C[(size_t)r * ldc + c] = acc;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tensor map of a row-major BF16 matrix [rows][ld] whose first K columns are read, in boxes
// of 64 columns x box_rows rows with the 128-byte swizzle; rows past the end read as zero.
bool make_map(CUtensorMap* map, const __nv_bfloat16* p, int rows, int K, int ld, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)UK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(p), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

unsigned int* umma_err_word() {
    static unsigned int* w[64] = {};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!w[dev] && cudaMalloc((void**)&w[dev], sizeof(unsigned int)) == cudaSuccess)
        cudaMemset(w[dev], 0, sizeof(unsigned int));
    return w[dev];
}

}  // namespace

// Shapes the tcgen05 path takes: K a multiple of 64, N a multiple of 256, 16-byte aligned
// operands with row strides of whole 16-byte units.
bool umma_gemm_fits(const void* A, int lda, const void* B, int ldb, int M, int N, int K) {
    return M > 0 && N % UN == 0 && K % UK == 0 && K > 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
           (reinterpret_cast<uintptr_t>(B) & 15) == 0 && lda % 8 == 0 && ldb % 8 == 0;
}

// C[M][N] (row stride ldc) = A[M][K] B[N][K]^T on tcgen05, split over K to fill the GPU.
cudaError_t umma_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* C, int ldc, int M,
                      int N, int K, cudaStream_t s) {
    static bool attr[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUmmaSmem);
        if (e != cudaSuccess) return e;
        attr[dev] = true;
    }
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda, UM) || !make_map(&mb, B, N, K, ldb, UN)) return cudaErrorInvalidValue;
    unsigned int* err = umma_err_word();
    if (!err) return cudaErrorMemoryAllocation;
    const int tiles = (N / UN) * ((M + UM - 1) / UM);
    const int total = K / UK;
    // One CTA per SM (the 4-stage ring fills the shared memory).  The split of K is the one
    // with the least estimated time: waves x k-blocks per CTA at about 0.34 us per k-block
    // (a second, partial wave costs as much as a full one), plus, for a split, writing and
    // reading its FP32 slabs (8 bytes per element and split at about 6,800 bytes per ns); at
    // least 4 k-blocks per CTA, the smaller split on ties.
    const int sms = sm_count();
    int split = 1;
    double best = -1.0;
    for (int sp = 1; sp <= std::max(1, total / 4); ++sp) {
        const double waves = (double)(((long long)tiles * sp + sms - 1) / sms);
        const double cost = waves * (double)((total + sp - 1) / sp) * 340.0 +
                            (sp > 1 ? (double)sp * M * N * 8.0 / 6800.0 : 0.0);
        if (best < 0.0 || cost < best) {
            best = cost;
            split = sp;
        }
    }
    int kps = (total + split - 1) / split;
    split = (total + kps - 1) / kps;
    const dim3 grid(N / UN, (M + UM - 1) / UM, split);
    const int ptok = prof_begin(P_GEMM, s);
    cudaError_t e = cudaSuccess;
    if (split == 1) {
        launch(k_umma_gemm, grid, 128, kUmmaSmem, s, ma, mb, C, ldc, (size_t)0, M, kps, total, err);
    } else {
        float* ws = nullptr;
        e = dmalloc((void**)&ws, (size_t)split * M * N * sizeof(float), s);
        if (e == cudaSuccess) {
            launch(k_umma_gemm, grid, 128, kUmmaSmem, s, ma, mb, ws, N, (size_t)M * N, M, kps, total, err);
            launch(k_umma_sum, (unsigned)(((uint64_t)M * N + 255) / 256), 256, 0, s, (const float*)ws, split, M, N, C,
                   ldc);
            cudaFreeAsync(ws, s);
        }
    }
    prof_end(P_GEMM, s, ptok);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

// Reads and clears the tcgen05 path's error word (nonzero: a wait ran out).
cudaError_t umma_error_take(unsigned int* h_word, cudaStream_t s) {
    unsigned int* err = umma_err_word();
    if (!err) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMemcpyAsync(h_word, err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && *h_word) e = cudaMemsetAsync(err, 0, sizeof(unsigned int), s);
    return e;
}

}  // namespace rs
