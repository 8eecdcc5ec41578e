// rs_est.cu -- grid selectivity estimator.
//
// Replaces estimateSelectivityKernel + thrust::reduce<float>
// (query/src/cuda/estimated_overlap.cu:8-77, estimated_intersection.cu:8-79) and the
// host loops calculateGlobalAvgSize / calculateGlobalAvgVolRatio
// (query/src/applications/raytracer_overlap_estimated_main.cpp:129-158).  One pass
// over both grids computes the per-cell float estimate exactly as the reference
// kernel does and, in the same read, the TouchCount-weighted means; all sums are
// FP64 in a fixed tree order, so the result does not depend on scheduling.
#include <cmath>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kT = 256;
constexpr int kBlocks = 1216;  // fixed, so the summation order is the same on every GPU
constexpr int kSums = 7;      // raw, sizeA*touch, ratioA*touch, touchA, sizeB*touch, ratioB*touch, touchB

struct Cell {
    uint32_t center, touch;
    float avg, ratio;
};

__device__ __forceinline__ float cell_estimate(const Cell& A, const Cell& B, float cell_volume, float eps, float gamma) {
    if (A.touch == 0 || B.touch == 0) return 0.0f;
    const float cs = __fadd_rn(__fadd_rn(A.avg, B.avg), eps);
    const float mv = __fmul_rn(__fmul_rn(cs, cs), cs);
    float prob = __fdiv_rn(mv, cell_volume);
    const float ratio = __fsqrt_rn(__fmul_rn(A.ratio, B.ratio));
    const float corr = powf(ratio, gamma);
    prob = __fmul_rn(prob, corr);
    prob = fminf(prob, 1.0f);
    return __fmul_rn(__fmul_rn((float)A.touch, (float)B.touch), prob);
}

__global__ void __launch_bounds__(kT) k_estimate(const uint4* __restrict__ A, const uint4* __restrict__ B, uint64_t n,
                                                 float cell_volume, float eps, float gamma, double* __restrict__ part) {
    double acc[kSums] = {0, 0, 0, 0, 0, 0, 0};
    for (uint64_t i = blockIdx.x * (uint64_t)kT + threadIdx.x; i < n; i += (uint64_t)kBlocks * kT) {
        const uint4 ra = __ldg(&A[i]), rb = __ldg(&B[i]);
        Cell a{ra.x, ra.y, __uint_as_float(ra.z), __uint_as_float(ra.w)};
        Cell b{rb.x, rb.y, __uint_as_float(rb.z), __uint_as_float(rb.w)};
        acc[0] += (double)cell_estimate(a, b, cell_volume, eps, gamma);
        if (a.touch) {
            acc[1] += (double)a.avg * (double)a.touch;
            acc[2] += (double)a.ratio * (double)a.touch;
            acc[3] += (double)a.touch;
        }
        if (b.touch) {
            acc[4] += (double)b.avg * (double)b.touch;
            acc[5] += (double)b.ratio * (double)b.touch;
            acc[6] += (double)b.touch;
        }
    }
    __shared__ double sh[kSums][kT];
#pragma unroll
    for (int k = 0; k < kSums; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = kT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < kSums; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < kSums) part[blockIdx.x * kSums + threadIdx.x] = sh[threadIdx.x][0];
}

// Per-cell estimates only (rs_estimate_grid_cells): the values estimateSelectivityKernel
// writes to its result buffer (estimated_overlap.cu:8-41).
__global__ void __launch_bounds__(kT) k_estimate_cells(const uint4* __restrict__ A, const uint4* __restrict__ B,
                                                       uint64_t n, float cell_volume, float eps, float gamma,
                                                       float* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)kT + threadIdx.x;
    if (i >= n) return;
    const uint4 ra = __ldg(&A[i]), rb = __ldg(&B[i]);
    const Cell a{ra.x, ra.y, __uint_as_float(ra.z), __uint_as_float(ra.w)};
    const Cell b{rb.x, rb.y, __uint_as_float(rb.z), __uint_as_float(rb.w)};
    out[i] = cell_estimate(a, b, cell_volume, eps, gamma);
}

// Fixed-order reduction of the per-block partials: thread t sums blocks t, t+256, ...
// in order, then a fixed shared-memory tree combines the 256 thread sums.
__global__ void __launch_bounds__(256) k_estimate_final(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[kSums][256];
    double acc[kSums] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < kBlocks; b += 256) {
#pragma unroll
        for (int k = 0; k < kSums; ++k) acc[k] += part[b * kSums + k];
    }
#pragma unroll
    for (int k = 0; k < kSums; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < kSums; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < kSums) out[threadIdx.x] = sh[threadIdx.x][0];
}

}  // namespace

// Shared by rs_estimate_grid and the reference-compatible wrappers.
int estimate_device(const void* d_a, const void* d_b, uint64_t n, float cell_volume, float eps, float gamma,
                    double out[kSums], cudaStream_t s) {
    double* part = nullptr;
    cudaError_t e = dmalloc((void**)&part, (kBlocks * kSums + kSums) * sizeof(double), s);
    if (e != cudaSuccess) return to_status(e);
    const int ptok = prof_begin(P_ESTIMATE, s);
    launch(k_estimate, kBlocks, kT, 0, s, reinterpret_cast<const uint4*>(d_a), reinterpret_cast<const uint4*>(d_b), n,
                                      cell_volume, eps, gamma, part);
    launch(k_estimate_final, 1, 256, 0, s, part, part + kBlocks * kSums);
    prof_end(P_ESTIMATE, s, ptok);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, part + kBlocks * kSums, kSums * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(part, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    prof_collect();
    if (e == cudaSuccess) e = e2;
    return to_status(e);
}

}  // namespace rs

using namespace rs;

extern "C" int rs_estimate_grid(const void* d_cellsA, const void* d_cellsB, uint64_t ncells, float cell_volume,
                                float epsilon, float gamma, double* h_raw, float* h_means4, void* stream) {
    if (!h_raw || (ncells && (!d_cellsA || !d_cellsB))) return RS_ERR_INVALID;
    double sums[7] = {0, 0, 0, 0, 0, 0, 0};
    if (ncells) {
        int st = estimate_device(d_cellsA, d_cellsB, ncells, cell_volume, epsilon, gamma, sums, (cudaStream_t)stream);
        if (st != RS_OK) return st;
    }
    *h_raw = sums[0];
    if (h_means4) {
        // calculateGlobalAvgSize / calculateGlobalAvgVolRatio: size 0 and ratio 1 without touches.
        h_means4[0] = sums[3] > 0 ? (float)(sums[1] / sums[3]) : 0.0f;
        h_means4[1] = sums[3] > 0 ? (float)(sums[2] / sums[3]) : 1.0f;
        h_means4[2] = sums[6] > 0 ? (float)(sums[4] / sums[6]) : 0.0f;
        h_means4[3] = sums[6] > 0 ? (float)(sums[5] / sums[6]) : 1.0f;
    }
    return RS_OK;
}

extern "C" int rs_estimate_grid_cells(const void* d_cellsA, const void* d_cellsB, uint64_t ncells, float cell_volume,
                                      float epsilon, float gamma, float* d_values, void* stream) {
    if (ncells && (!d_cellsA || !d_cellsB || !d_values)) return RS_ERR_INVALID;
    if (ncells == 0) return RS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    launch(k_estimate_cells, (unsigned)((ncells + kT - 1) / kT), kT, 0, s, reinterpret_cast<const uint4*>(d_cellsA),
           reinterpret_cast<const uint4*>(d_cellsB), ncells, cell_volume, epsilon, gamma, d_values);
    cudaError_t e = cudaGetLastError();
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    return to_status(e);
}

extern "C" int64_t rs_estimate_pairs_from_raw(double raw, const float* m, float cell_volume, int alpha_correction) {
    // raytracer_overlap_estimated_main.cpp:275-291
    float alpha = 1.0f;
    if (alpha_correction && m) {
        const float e1 = m[0] * std::cbrt(m[1]);
        const float e2 = m[2] * std::cbrt(m[3]);
        const float cs = e1 + e2;
        const float mv = cs * cs * cs;
        if (cell_volume < 1e-9f) cell_volume = 1e-9f;
        alpha = mv / cell_volume;
        if (alpha < 1.0f) alpha = 1.0f;
    }
    return (int64_t)((float)raw / alpha);
}
