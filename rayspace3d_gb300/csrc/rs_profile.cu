// rs_profile.cu -- launch counter and the opt-in per-kernel event profiler.
#include <mutex>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {

std::atomic<uint64_t> g_launches{0};

cudaError_t dmalloc(void** p, size_t bytes, cudaStream_t s) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> g(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            e = cudaMemPoolCreate(&pools[dev], &props);
            if (e != cudaSuccess) return e;
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

namespace {
struct Slot {
    cudaEvent_t a = nullptr, b = nullptr;
    bool pending = false;
    double total_ms = 0.0;
    uint64_t launches = 0;
};
std::mutex g_mu;
bool g_on = false;
Slot g_slots[P_COUNT];
}  // namespace

void prof_begin(int id, cudaStream_t s) {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_on) return;
    Slot& sl = g_slots[id];
    if (!sl.a) {
        cudaEventCreate(&sl.a);
        cudaEventCreate(&sl.b);
    }
    cudaEventRecord(sl.a, s);
}

void prof_end(int id, cudaStream_t s) {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_on || !g_slots[id].a) return;
    cudaEventRecord(g_slots[id].b, s);
    g_slots[id].pending = true;
}

void prof_collect() {
    std::lock_guard<std::mutex> g(g_mu);
    for (Slot& sl : g_slots) {
        if (!sl.pending) continue;
        float ms = 0.0f;
        if (cudaEventSynchronize(sl.b) == cudaSuccess && cudaEventElapsedTime(&ms, sl.a, sl.b) == cudaSuccess) {
            sl.total_ms += ms;
            sl.launches += 1;
        }
        sl.pending = false;
    }
}

}  // namespace rs

extern "C" uint64_t rs_launch_count(void) { return rs::g_launches.load(); }

extern "C" int rs_profile_enable(int on) {
    std::lock_guard<std::mutex> g(rs::g_mu);
    rs::g_on = on != 0;
    return RS_OK;
}

extern "C" int rs_profile_reset(void) {
    std::lock_guard<std::mutex> g(rs::g_mu);
    for (auto& sl : rs::g_slots) {
        sl.total_ms = 0.0;
        sl.launches = 0;
        sl.pending = false;
    }
    return RS_OK;
}

extern "C" int rs_profile_read(int kernel, double* total_ms, uint64_t* launches) {
    if (kernel < 0 || kernel >= rs::P_COUNT) return RS_ERR_INVALID;
    rs::prof_collect();
    std::lock_guard<std::mutex> g(rs::g_mu);
    if (total_ms) *total_ms = rs::g_slots[kernel].total_ms;
    if (launches) *launches = rs::g_slots[kernel].launches;
    return RS_OK;
}
