// rs_launch.cuh -- counted kernel launches and opt-in per-kernel CUDA-event timing.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <utility>

namespace rs {

extern std::atomic<uint64_t> g_launches;

// Stream-ordered device allocation from a library-owned pool that keeps freed
// memory for reuse (the default pool hands it back to the driver at every sync).
cudaError_t dmalloc(void** p, size_t bytes, cudaStream_t s);
template <class T>
inline cudaError_t dmalloc(T** p, size_t bytes, cudaStream_t s) {
    return dmalloc(reinterpret_cast<void**>(p), bytes, s);
}

// Pool allocations of one call, released (stream-ordered) when the scope ends.
struct Scratch {
    cudaStream_t s;
    void* p[16] = {};
    int n = 0;
    template <class T>
    cudaError_t get(T** out, size_t bytes) {
        if (n == 16) return cudaErrorMemoryAllocation;
        cudaError_t e = dmalloc((void**)out, bytes ? bytes : 16, s);
        if (e == cudaSuccess) p[n++] = *out;
        return e;
    }
    ~Scratch() {
        for (int i = 0; i < n; ++i) cudaFreeAsync(p[i], s);
    }
};

// Number of bits needed to write v (0 for 0).
inline int bits_for(unsigned long long v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b;
}

// Every kernel of the engine is launched through this wrapper so the number of
// launches is observable (rs_launch_count).
template <class... KArgs, class... Args>
inline void launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
    kernel<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

// Kernels whose device time the profiler accumulates (rs_profile_read ids).
enum ProfId { P_EDGE_JOIN = 0, P_CONTAINMENT = 1, P_PIM = 2, P_BVH_BUILD = 3, P_FINALIZE = 4, P_ESTIMATE = 5,
              P_BUILD_UP = 6, P_GEMM = 7, P_COUNT = 8 };

// Records an event pair around one launch when profiling is on; prof_collect()
// (called after the stream has been synchronised) accumulates the elapsed time.
int prof_begin(int id, cudaStream_t s);          // returns a token for prof_end
// Pinned host slots of 16 ints (nullptr when pinned memory is unavailable).
int* pinned_slot_acquire();
void pinned_slot_release(int* p);
void prof_end(int id, cudaStream_t s, int token);
void prof_collect();

}  // namespace rs
