// rs_grid.cu -- per-cell grid statistics on the GPU (generateGridStats,
// preprocess/src/preprocess_dataset.cpp:37-181), for datasets built in device memory
// (the learned estimator's training data).
//
// Per object: its box over the valid triangles, its signed volume relative to the box
// centre (float terms summed in FP64), ratio = |volume|/6 / box volume clamped to
// [.., 1], mean extent; then CenterCount of the anchor cell and TouchCount /
// AvgSizeMean / VolRatio sums over the touched cells, normalised per cell.  Every
// quantity uses the reference's float formulas; the float sums per cell are taken with
// atomics in arrival order (the reference sums in std::unordered_map order), so
// AvgSizeMean and VolRatio can differ from the reference's in the last bits.
#include <cstring>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
namespace {

constexpr int kGT = 256;

__device__ __forceinline__ int g_f2ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float g_ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct ObjStats {
    int box[6];     // ordered-int min xyz, max xyz
    double volume;  // signed volume sum
};

__global__ void k_gs_init(ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_obj) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        o[i].box[c] = g_f2ord(1e30f);
        o[i].box[3 + c] = g_f2ord(-1e30f);
    }
    o[i].volume = 0.0;
}

__device__ __forceinline__ bool tri_valid(const uint32_t* __restrict__ I, uint64_t nV, uint64_t t) {
    return I[3 * t] < nV && I[3 * t + 1] < nV && I[3 * t + 2] < nV;
}

// Pass 1 (preprocess_dataset.cpp:69-86): object boxes.
__global__ void k_gs_boxes(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t nF,
                           const int32_t* __restrict__ T, ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF || !tri_valid(I, nV, t)) return;
    const int32_t obj = T[t];
    if (obj < 0 || (uint64_t)obj >= n_obj) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a = V[3 * (uint64_t)I[3 * t] + c], b = V[3 * (uint64_t)I[3 * t + 1] + c],
                    d = V[3 * (uint64_t)I[3 * t + 2] + c];
        atomicMin(&o[obj].box[c], g_f2ord(fminf(fminf(a, b), d)));
        atomicMax(&o[obj].box[3 + c], g_f2ord(fmaxf(fmaxf(a, b), d)));
    }
}

// Pass 2 (:88-114): signed volume about the box centre, float terms, FP64 sum.
__global__ void k_gs_volume(const float* __restrict__ V, uint64_t nV, const uint32_t* __restrict__ I, uint64_t nF,
                            const int32_t* __restrict__ T, ObjStats* __restrict__ o, uint64_t n_obj) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nF || !tri_valid(I, nV, t)) return;
    const int32_t obj = T[t];
    if (obj < 0 || (uint64_t)obj >= n_obj) return;
    float c[3], p[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        c[k] = __fmul_rn(__fadd_rn(g_ord2f(o[obj].box[k]), g_ord2f(o[obj].box[3 + k])), 0.5f);
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int k = 0; k < 3; ++k) p[v][k] = __fsub_rn(V[3 * (uint64_t)I[3 * t + v] + k], c[k]);
    const float cx = __fsub_rn(__fmul_rn(p[0][1], p[1][2]), __fmul_rn(p[0][2], p[1][1]));
    const float cy = __fsub_rn(__fmul_rn(p[0][2], p[1][0]), __fmul_rn(p[0][0], p[1][2]));
    const float cz = __fsub_rn(__fmul_rn(p[0][0], p[1][1]), __fmul_rn(p[0][1], p[1][0]));
    const float term = __fadd_rn(__fadd_rn(__fmul_rn(cx, p[2][0]), __fmul_rn(cy, p[2][1])), __fmul_rn(cz, p[2][2]));
    atomicAdd(&o[obj].volume, (double)term);
}

struct GridFrame {
    float mn[3], cs[3];
    int res;
};

// Pass 3 (:116-168): per object, anchor cell and touched cells.  A grid-stride loop
// over the touched cells of one object runs in one thread.
__global__ void k_gs_cells(const ObjStats* __restrict__ o, uint64_t n_obj, GridFrame f, uint32_t* __restrict__ cells) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_obj) return;
    float mnb[3], mxb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mnb[k] = g_ord2f(o[i].box[k]);
        mxb[k] = g_ord2f(o[i].box[3 + k]);
    }
    if (!(mnb[0] <= mxb[0])) return;  // no valid triangle: the reference has no entry for it
    const float meshVol = __fdiv_rn(fabsf((float)o[i].volume), 6.0f);
    const float w = __fsub_rn(mxb[0], mnb[0]), h = __fsub_rn(mxb[1], mnb[1]), d = __fsub_rn(mxb[2], mnb[2]);
    float aabb = __fmul_rn(__fmul_rn(w, h), d);
    if (aabb < 1e-9f) aabb = 1e-9f;
    float ratio = __fdiv_rn(meshVol, aabb);
    if (ratio > 1.0f) ratio = 1.0f;
    const float avg = __fdiv_rn(__fadd_rn(__fadd_rn(w, h), d), 3.0f);
    const int R = f.res;
    int a[3], lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ctr = __fmul_rn(__fadd_rn(mnb[k], mxb[k]), 0.5f);
        a[k] = (int)__fdiv_rn(__fsub_rn(ctr, f.mn[k]), f.cs[k]);
        lo[k] = max(0, (int)__fdiv_rn(__fsub_rn(mnb[k], f.mn[k]), f.cs[k]));
        hi[k] = min(R - 1, (int)__fdiv_rn(__fsub_rn(__fsub_rn(mxb[k], f.mn[k]), 1e-5f), f.cs[k]));
    }
    if (a[0] >= 0 && a[0] < R && a[1] >= 0 && a[1] < R && a[2] >= 0 && a[2] < R)
        atomicAdd(&cells[4 * ((uint64_t)(a[2] * R + a[1]) * R + a[0])], 1u);
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                uint32_t* c = cells + 4 * ((uint64_t)(z * R + y) * R + x);
                atomicAdd(c + 1, 1u);
                atomicAdd(reinterpret_cast<float*>(c + 2), avg);
                atomicAdd(reinterpret_cast<float*>(c + 3), ratio);
            }
}

// Pass 4 (:170-177): means.
__global__ void k_gs_normalise(uint32_t* __restrict__ cells, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t tc = cells[4 * i + 1];
    if (!tc) return;
    float* f = reinterpret_cast<float*>(cells + 4 * i);
    f[2] = __fdiv_rn(f[2], (float)tc);
    f[3] = __fdiv_rn(f[3], (float)tc);
}

__global__ void k_gs_vbounds(const float* __restrict__ V, uint64_t nV, int* __restrict__ b) {
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nV; i += (uint64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], V[3 * i + k]);
            mx[k] = fmaxf(mx[k], V[3 * i + k]);
        }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        atomicMin(&b[k], g_f2ord(mn[k]));
        atomicMax(&b[3 + k], g_f2ord(mx[k]));
    }
}

}  // namespace
}  // namespace rs

using namespace rs;

extern "C" int rs_grid_stats(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                             const int32_t* d_tri2obj, uint64_t n_obj, int resolution, float world_size,
                             void* d_cells, float* h_bounds6, void* stream) {
    if (resolution <= 0 || resolution > 1024 || !d_cells || (nF && (!d_indices || !d_tri2obj)) ||
        (nV && !d_vertices))
        return RS_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t ncell = (uint64_t)resolution * resolution * resolution;
    // Frame: [0, world]^3, or the bounds of all vertices (:40-60).
    float mn[3], mx[3];
    if (world_size > 0.0f) {
        for (int k = 0; k < 3; ++k) {
            mn[k] = 0.0f;
            mx[k] = world_size;
        }
    } else {
        int* b = nullptr;
        cudaError_t e = dmalloc((void**)&b, 6 * sizeof(int), s);
        if (e != cudaSuccess) return to_status(e);
        const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
        int hb[6];
        e = cudaMemcpyAsync(b, init, sizeof(init), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && nV) launch(k_gs_vbounds, 2 * sm_count(), kGT, 0, s, d_vertices, nV, b);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hb, b, sizeof(hb), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFreeAsync(b, s);
        if (e != cudaSuccess) return to_status(e);
        for (int k = 0; k < 3; ++k) {
            auto dec = [](int i) {
                int v = i >= 0 ? i : i ^ 0x7fffffff;
                float f;
                std::memcpy(&f, &v, 4);
                return f;
            };
            // The reference starts its min/max at +-1e30 (an empty set keeps them).
            mn[k] = nV ? dec(hb[k]) : 1e30f;
            mx[k] = nV ? dec(hb[3 + k]) : -1e30f;
        }
    }
    GridFrame f;
    f.res = resolution;
    for (int k = 0; k < 3; ++k) {
        f.mn[k] = mn[k];
        f.cs[k] = (mx[k] - mn[k]) / (float)resolution;
        if (h_bounds6) {
            h_bounds6[k] = mn[k];
            h_bounds6[3 + k] = mx[k];
        }
    }
    cudaError_t e = cudaMemsetAsync(d_cells, 0, ncell * 16, s);
    ObjStats* o = nullptr;
    if (e == cudaSuccess && n_obj) e = dmalloc((void**)&o, n_obj * sizeof(ObjStats), s);
    if (e != cudaSuccess) return to_status(e);
    if (n_obj) {
        const unsigned go = (unsigned)((n_obj + kGT - 1) / kGT), gt = (unsigned)((nF + kGT - 1) / kGT);
        launch(k_gs_init, go, kGT, 0, s, o, n_obj);
        if (nF) {
            launch(k_gs_boxes, gt, kGT, 0, s, d_vertices, nV, d_indices, nF, d_tri2obj, o, n_obj);
            launch(k_gs_volume, gt, kGT, 0, s, d_vertices, nV, d_indices, nF, d_tri2obj, o, n_obj);
        }
        launch(k_gs_cells, go, kGT, 0, s, (const ObjStats*)o, n_obj, f, (uint32_t*)d_cells);
        launch(k_gs_normalise, (unsigned)((ncell + kGT - 1) / kGT), kGT, 0, s, (uint32_t*)d_cells, ncell);
        cudaFreeAsync(o, s);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return to_status(e);
}
