// Host-memory stand-ins for the two CUDA runtime calls the reference's PinnedAllocator
// makes (common/include/PinnedMemory.h:20-40), so the reference's host code runs on a
// machine without a GPU.  Part of the oracle's reference build only.
#include <cstdlib>
#include <cuda_runtime_api.h>

extern "C" cudaError_t cudaMallocHost(void** ptr, size_t size) {
    *ptr = std::malloc(size ? size : 1);
    return *ptr ? cudaSuccess : cudaErrorMemoryAllocation;
}
extern "C" cudaError_t cudaFreeHost(void* ptr) {
    std::free(ptr);
    return cudaSuccess;
}
extern "C" const char* cudaGetErrorString(cudaError_t) { return "host shim"; }
