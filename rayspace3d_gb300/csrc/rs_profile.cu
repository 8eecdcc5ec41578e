// rs_profile.cu -- launch counter and the opt-in per-kernel event profiler.
#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "rs_engine.h"
#include "rs_prims.cuh"

namespace rs {

std::atomic<uint64_t> g_launches{0};

// Device allocations requested through dmalloc since the library was loaded
// (rs_alloc_count).
static std::atomic<uint64_t> g_alloc_count{0};

cudaError_t dmalloc(void** p, size_t bytes, cudaStream_t s) {
    g_alloc_count.fetch_add(1, std::memory_order_relaxed);
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
            // A block freed on one stream is reused on another only through an event
            // dependency the caller made: with opportunistic reuse on, an allocation on the
            // second of two concurrently building streams took 115-140 us of host time
            // (measured on GB300), against 1-2 us without it.
            int off = 0;
            cudaMemPoolSetAttribute(pools[dev], cudaMemPoolReuseAllowOpportunistic, &off);
            cudaMemPoolSetAttribute(pools[dev], cudaMemPoolReuseAllowInternalDependencies, &off);
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// Small pinned host slots (16 ints) that asynchronous builds copy their result words
// into, so reading them needs only the build's event.  Slots come from 256-slot pinned
// blocks allocated on demand and are recycled.
namespace {
std::mutex g_slot_mu;
std::vector<int*> g_free_slots;
}  // namespace

int* pinned_slot_acquire() {
    std::lock_guard<std::mutex> g(g_slot_mu);
    if (g_free_slots.empty()) {
        int* block = nullptr;
        if (cudaMallocHost((void**)&block, 256 * 16 * sizeof(int)) != cudaSuccess) return nullptr;
        for (int i = 255; i >= 0; --i) g_free_slots.push_back(block + 16 * i);
    }
    int* p = g_free_slots.back();
    g_free_slots.pop_back();
    return p;
}

void pinned_slot_release(int* p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(g_slot_mu);
    g_free_slots.push_back(p);
}

namespace {
// One event pair per profiled launch between collections; launches on several
// streams may be open at once (each begin returns its own token).
struct Slot {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    std::vector<char> done;  // 0 open, 1 ended, 2 collected
    size_t used = 0;
    double total_ms = 0.0;
    uint64_t launches = 0;
};
std::mutex g_mu;
bool g_on = false;
Slot g_slots[P_COUNT];
}  // namespace

int prof_begin(int id, cudaStream_t s) {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_on) return -1;
    Slot& sl = g_slots[id];
    if (sl.used == sl.ev.size()) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (cudaEventCreate(&a) != cudaSuccess) return -1;
        if (cudaEventCreate(&b) != cudaSuccess) {
            cudaEventDestroy(a);
            return -1;
        }
        sl.ev.push_back({a, b});
        sl.done.push_back(0);
    }
    const int tok = (int)sl.used++;
    sl.done[tok] = 0;
    cudaEventRecord(sl.ev[tok].first, s);
    return tok;
}

void prof_end(int id, cudaStream_t s, int tok) {
    std::lock_guard<std::mutex> g(g_mu);
    Slot& sl = g_slots[id];
    if (tok < 0 || (size_t)tok >= sl.used) return;
    cudaEventRecord(sl.ev[tok].second, s);
    sl.done[tok] = 1;
}

void prof_collect() {
    std::lock_guard<std::mutex> g(g_mu);
    for (Slot& sl : g_slots) {
        bool all = true;
        for (size_t i = 0; i < sl.used; ++i) {
            if (sl.done[i] == 0) all = false;  // still open on some stream
            if (sl.done[i] != 1) continue;
            float ms = 0.0f;
            if (cudaEventSynchronize(sl.ev[i].second) == cudaSuccess &&
                cudaEventElapsedTime(&ms, sl.ev[i].first, sl.ev[i].second) == cudaSuccess) {
                sl.total_ms += ms;
                sl.launches += 1;
            }
            sl.done[i] = 2;
        }
        if (all) sl.used = 0;
    }
}

}  // namespace rs

extern "C" uint64_t rs_launch_count(void) { return rs::g_launches.load(); }

extern "C" uint64_t rs_alloc_count(void) { return rs::g_alloc_count.load(); }

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
        sl.used = 0;
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

extern "C" int rs_recheck_enable(int on) {
    int e = rs::recheck_pim(on ? 1 : 0, nullptr);
    if (e == 0) e = rs::recheck_join(on ? 1 : 0, nullptr);
    if (e == 0) e = rs::recheck_batch(on ? 1 : 0, nullptr);
    return rs::to_status((cudaError_t)e);
}

extern "C" int rs_recheck_reset(void) {
    int e = rs::recheck_pim(2, nullptr);
    if (e == 0) e = rs::recheck_join(2, nullptr);
    if (e == 0) e = rs::recheck_batch(2, nullptr);
    return rs::to_status((cudaError_t)e);
}

extern "C" int rs_recheck_read(uint64_t* exact_signs, uint64_t* triangle_tests) {
    unsigned long long v[2] = {0, 0};
    int e = rs::recheck_pim(3, v);
    if (e == 0) e = rs::recheck_join(3, v);
    if (e == 0) e = rs::recheck_batch(3, v);
    if (e != 0) return rs::to_status((cudaError_t)e);
    if (exact_signs) *exact_signs = v[0];
    if (triangle_tests) *triangle_tests = v[1];
    return RS_OK;
}
