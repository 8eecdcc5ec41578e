// rs_compat.cu -- the reference's extern "C" helpers, same names and signatures.
//
// query/src/cuda/scan_utils.h:7-9, mesh_query_deduplication.h:6-18,
// result_compaction.h:5-22, estimated_overlap.h:6-13 / estimated_intersection.h.
// Like the reference they run on the legacy default stream and return after the
// work finished.  Outputs that the reference leaves in atomic order (hash-slot and
// hit compaction) come out here in index order, one valid instance of it.
#include <cstdio>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {
int estimate_device(const void* d_a, const void* d_b, uint64_t n, float cell_volume, float eps, float gamma,
                    double out[7], cudaStream_t s);
namespace {

__global__ void k_swap_halves_c(uint64_t* __restrict__ k, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) k[i] = (k[i] << 32) | (k[i] >> 32);
}

__global__ void k_ray_flags(const int2* __restrict__ r, uint64_t n, uint32_t* __restrict__ f) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) f[i] = r[i].y != -1;
}

__global__ void k_ray_scatter(const int2* __restrict__ r, uint64_t n, const uint32_t* __restrict__ pos,
                              int2* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n && r[i].y != -1) out[pos[i]] = r[i];
}

}  // namespace
}  // namespace rs

using namespace rs;

extern "C" long long exclusive_scan_gpu(const int* d_input, long long* d_output, int num_elements) {
    if (num_elements <= 0) return 0;
    int64_t* total = nullptr;
    if (dmalloc((void**)&total, sizeof(int64_t), 0) != cudaSuccess) return 0;
    int64_t h = 0;
    if (exclusive_scan_i32_to_i64(d_input, reinterpret_cast<int64_t*>(d_output), (size_t)num_elements, total, 0) ==
        cudaSuccess)
        cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, 0);
    cudaFreeAsync(total, 0);
    cudaStreamSynchronize(0);
    return (long long)h;
}

extern "C" long long merge_and_deduplicate_pairs_gpu(const void* d_results1, long long num_results1,
                                                     const void* d_results2, long long num_results2,
                                                     void* d_merged_output) {
    const long long total = num_results1 + num_results2;
    if (total <= 0) return 0;
    // mesh_query_deduplication.cu:105-116: inputs that are NULL are already in place.
    if (d_results1 && num_results1 > 0)
        cudaMemcpyAsync(d_merged_output, d_results1, (size_t)num_results1 * 8, cudaMemcpyDeviceToDevice, 0);
    if (d_results2 && num_results2 > 0)
        cudaMemcpyAsync((char*)d_merged_output + (size_t)num_results1 * 8, d_results2, (size_t)num_results2 * 8,
                        cudaMemcpyDeviceToDevice, 0);
    uint64_t* keys = reinterpret_cast<uint64_t*>(d_merged_output);
    uint64_t* cnt = nullptr;
    uint64_t h = 0;
    if (sort_u64_any(keys, (size_t)total, 0) != cudaSuccess) return 0;
    if (dmalloc((void**)&cnt, sizeof(uint64_t), 0) != cudaSuccess) return 0;
    if (unique_sorted_u64(keys, (size_t)total, cnt, 0) == cudaSuccess)
        cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, 0);
    uint32_t sort_err = 0;
    sort_error_read(&sort_err, 0);
    cudaFreeAsync(cnt, 0);
    cudaStreamSynchronize(0);
    if (sort_err) {  // a failed sort: report no result, as on an allocation failure
        sort_error_clear(0);
        return 0;
    }
    return (long long)h;
}

extern "C" int compact_hash_table_pairs(const unsigned long long* d_hash_table, unsigned long long table_size,
                                        void* d_output, int max_output_size) {
    if (table_size == 0 || max_output_size <= 0) return 0;
    uint64_t* tmp = nullptr;
    uint64_t* cnt = nullptr;
    uint64_t h = 0;
    if (dmalloc((void**)&tmp, table_size * sizeof(uint64_t), 0) != cudaSuccess) return 0;
    if (dmalloc((void**)&cnt, sizeof(uint64_t), 0) == cudaSuccess &&
        compact_u64(reinterpret_cast<const uint64_t*>(d_hash_table), table_size, kEmptyKey, tmp, cnt, 0) ==
            cudaSuccess) {
        cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, 0);
        cudaStreamSynchronize(0);
        const uint64_t m = h < (uint64_t)max_output_size ? h : (uint64_t)max_output_size;
        // key = id1<<32 | id2 becomes MeshQueryResult{id1, id2}, i.e. the swapped u64.
        if (m) {
            launch(k_swap_halves_c, (unsigned)((m + 255) / 256), 256, 0, 0, tmp, m);
            cudaMemcpyAsync(d_output, tmp, m * sizeof(uint64_t), cudaMemcpyDeviceToDevice, 0);
        }
    }
    if (cnt) cudaFreeAsync(cnt, 0);
    cudaFreeAsync(tmp, 0);
    cudaStreamSynchronize(0);
    return (int)(h < (uint64_t)max_output_size ? h : (uint64_t)max_output_size);
}

extern "C" int count_hits_gpu(const void* d_results, int num_results) {
    if (num_results <= 0 || !d_results) return 0;
    uint32_t* f = nullptr;
    uint32_t* tot = nullptr;
    uint32_t h = 0;
    const uint64_t n = (uint64_t)num_results;
    if (dmalloc((void**)&f, n * sizeof(uint32_t), 0) != cudaSuccess) return 0;
    if (dmalloc((void**)&tot, sizeof(uint32_t), 0) == cudaSuccess) {
        launch(k_ray_flags, (unsigned)((n + 255) / 256), 256, 0, 0, reinterpret_cast<const int2*>(d_results), n, f);
        if (exclusive_scan_u32(f, f, n, tot, 0) == cudaSuccess)
            cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, 0);
        cudaFreeAsync(tot, 0);
    }
    cudaFreeAsync(f, 0);
    cudaStreamSynchronize(0);
    return (int)h;
}

extern "C" void compact_hits_gpu(const void* d_input, void* d_output, int num_results, int* h_num_hits) {
    if (h_num_hits) *h_num_hits = 0;
    if (num_results <= 0 || !d_input) return;
    uint32_t* f = nullptr;
    uint32_t* tot = nullptr;
    uint32_t h = 0;
    const uint64_t n = (uint64_t)num_results;
    if (dmalloc((void**)&f, n * sizeof(uint32_t), 0) != cudaSuccess) return;
    if (dmalloc((void**)&tot, sizeof(uint32_t), 0) == cudaSuccess) {
        const unsigned grid = (unsigned)((n + 255) / 256);
        launch(k_ray_flags, grid, 256, 0, 0, reinterpret_cast<const int2*>(d_input), n, f);
        if (exclusive_scan_u32(f, f, n, tot, 0) == cudaSuccess) {
            launch(k_ray_scatter, grid, 256, 0, 0, reinterpret_cast<const int2*>(d_input), n, f,
                                               reinterpret_cast<int2*>(d_output));
            cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, 0);
        }
        cudaFreeAsync(tot, 0);
    }
    cudaFreeAsync(f, 0);
    cudaStreamSynchronize(0);
    if (h_num_hits) *h_num_hits = (int)h;
}

static float estimate_host_grids(const void* hA, const void* hB, int numCells, float cellVolume, float eps,
                                 float gamma) {
    if (numCells <= 0) return 0.0f;
    const size_t bytes = (size_t)numCells * 16;
    void* dA = nullptr;
    void* dB = nullptr;
    if (cudaMalloc(&dA, bytes) != cudaSuccess) return -1.0f;
    if (cudaMalloc(&dB, bytes) != cudaSuccess) {
        cudaFree(dA);
        return -1.0f;
    }
    cudaMemcpy(dA, hA, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, hB, bytes, cudaMemcpyHostToDevice);
    double sums[7];
    const int st = estimate_device(dA, dB, (uint64_t)numCells, cellVolume, eps, gamma, sums, 0);
    cudaFree(dA);
    cudaFree(dB);
    return st == RS_OK ? (float)sums[0] : -1.0f;
}

extern "C" float rs_estimate_overlap_selectivity(const void* h_gridA, const void* h_gridB, int numCells,
                                                 float cellVolume, float epsilon, float gamma) {
    return estimate_host_grids(h_gridA, h_gridB, numCells, cellVolume, epsilon, gamma);
}

extern "C" float rs_estimate_intersection_selectivity(const void* h_gridA, const void* h_gridB, int numCells,
                                                      float cellVolume, float epsilon, float gamma) {
    return estimate_host_grids(h_gridA, h_gridB, numCells, cellVolume, epsilon, gamma);
}

// The reference's own declarations (estimated_overlap.h:6-13, estimated_intersection.h:6-13)
// have C++ linkage and take the GridCell of common/include/GridCell.h:5-10; this struct has
// that name and layout, so these definitions carry the symbols the reference's mains link to.
struct GridCell {
    uint32_t CenterCount;
    uint32_t TouchCount;
    float AvgSizeMean;
    float VolRatio;
};
static_assert(sizeof(GridCell) == 16, "GridCell is 16 bytes");

float estimateOverlapSelectivity(const GridCell* h_gridA, const GridCell* h_gridB, int numCells, float cellVolume,
                                 float epsilon, float gamma) {
    return estimate_host_grids(h_gridA, h_gridB, numCells, cellVolume, epsilon, gamma);
}

float estimateIntersectionSelectivity(const GridCell* h_gridA, const GridCell* h_gridB, int numCells,
                                      float cellVolume, float epsilon, float gamma) {
    return estimate_host_grids(h_gridA, h_gridB, numCells, cellVolume, epsilon, gamma);
}
