// rs_engine.h -- engine-internal host structures behind the opaque C-ABI handles.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rayspace3d.h"
#include "rs_device.cuh"

// Column grid for rays along +e_axis: a uniform grid over the two other axes whose
// cells list (in leaf order) every triangle whose projected box touches the cell.
struct rs_column_grid {
    int built = 0;
    float u0 = 0, v0 = 0, su = 0, sv = 0;  // cell(x) = clamp(floor((x - u0) * su), 0, gu - 1)
    float u1 = 0, v1 = 0;                  // projected bounds of all triangles
    int gu = 1, gv = 1;
    uint32_t* start = nullptr;             // gu*gv + 1 offsets into list
    uint32_t* list = nullptr;              // leaf-order triangle indices
    uint64_t nlist = 0;
};

struct rs_bvh {
    // Caller-owned device inputs; they must outlive the handle.
    const float* V = nullptr;
    uint64_t nV = 0;
    const uint32_t* I = nullptr;
    uint64_t nF = 0;
    const int32_t* t2o = nullptr;
    // Engine-owned device arrays.
    rs::BNode* nodes = nullptr;
    uint64_t n_nodes = 0;
    float4* tris = nullptr;
    uint64_t n_tris = 0;
    int leaf_size = 2;
    rs_column_grid cgrid[3];
    // Bounds of all vertices (the reference's BoundingBox::computeFromGeometry).
    float vmin[3] = {0, 0, 0};
    float vmax[3] = {0, 0, 0};
    // Largest object id + 1 over the triangles (0 when there are none).
    uint64_t n_obj = 0;
    // Object boxes (ordered-int min xyz, max xyz per object) from the build's Morton
    // pass, for the objects below obox_cap; valid when n_obj <= obox_cap.
    int* obox = nullptr;
    uint64_t obox_cap = 0;
    // One device allocation holds nodes, tris and obox.
    void* mem = nullptr;
    int device = 0;
    // Completion of the build, and its device result words until bvh_ready() has read
    // them (asynchronous builds); the fields above that come from them (vmin, vmax,
    // n_obj) are valid only after bvh_ready().
    cudaEvent_t done = nullptr;
    int* pending = nullptr;
    int build_status = RS_OK;
};

struct rs_pairset {
    unsigned long long* slots = nullptr;
    unsigned long long capacity = 0;
    int pow2 = 1;
    unsigned int max_probes = 4096;
    // Device scratch: [0] status bits (u32 in the low word), [1] distinct-key count,
    // [2] slot accesses, [3] contended probes, [4..8] query counters (see rs_pairset_counters),
    // [10] finalize gather counter, [11] overflow-table key count; the overflow table follows
    // (kOverSlots slots, one allocation with the words), empty between joins.
    unsigned long long* meta = nullptr;
    unsigned long long* over = nullptr;
    bool over_dirty = false;  // a launch may have left keys in the overflow table
    // Incremented whenever the slots are reallocated (growth): a captured batch that holds
    // the old slot pointer recaptures.
    uint64_t generation = 0;
    int track = 0;  // count slot accesses and contention
    int device = 0;
    // Edge-ray hit rule (rs_pairset_set_edge_rule): the reference's kMaxIterations and
    // advance step of the overlap loop.
    int edge_max_hits = 100;
    int edge_next_float = 0;
    // meta[1] as last read by the host with status ok, while no launch has been given the
    // table since (table_view() resets it); -1 when unknown.
    long long known_count = -1;
};

namespace rs {
constexpr int kMetaWords = 16;
constexpr int kGatherWord = 10;  // meta word used as the finalize gather counter
constexpr int kOverWord = 11;    // meta word counting the overflow table's keys
constexpr uint64_t kOverSlots = 1ull << 20;
// Waits for the stream and turns the table's status bits into an rs_status.  A table that
// spilled (and lost no key) is first regrown from its slots and its overflow table, without
// rerunning the launches that filled it; the overflow table is left empty.
int table_status(rs_pairset* ps, cudaStream_t s, cudaError_t e);
// Queues the regrowth of a spilled table holding `count` keys in its slots and `over` in
// its overflow table: new slots with room for all of them, both tables' keys reinserted,
// the overflow table cleared.
cudaError_t table_regrow(rs_pairset* ps, uint64_t count, uint64_t over, cudaStream_t s);
// Queues the clearing of the overflow table (and its count) when a launch may have used it.
cudaError_t over_clear(rs_pairset* ps, cudaStream_t s);
// Upper bound on the node visits of one traversal of a valid tree.
inline uint32_t max_steps(const rs_bvh* b) { return (uint32_t)(2 * b->n_nodes + 8); }
int to_status(cudaError_t e);
// Asynchronous builds: bvh_ready() waits for the build and reads its host-side results
// (returns the build status); bvh_use() orders stream s after the build.
int bvh_ready(const rs_bvh* h);
int bvh_use(const rs_bvh* h, cudaStream_t s);
// Builds the column grid of +e_axis rays for the handle if it does not exist yet.
int ensure_grid(const rs_bvh* h, int axis, cudaStream_t s);
// Broad-phase flags for one edge direction: cand[o] != 0 for source objects o that may
// have a partner; no culling when cand is null.  With partner lists (part != null):
// cand[o] = the number of partner objects of the other set (0..kPartners) listed in
// part[o * kPartners ...], or kCandAll when they were not all collected; pbox holds the
// other set's object boxes (ordered-int min xyz, max xyz), n_pbox of them.  entry
// (nullable, with part): per source object whose flag is set, the node of the other set's
// BVH under which lie all triangles its edges' rays can hit; they start there.
constexpr int kPartners = 8;
constexpr uint8_t kCandAll = 255;
struct EdgeCull {
    const uint8_t* cand = nullptr;
    uint64_t n_obj = 0;
    const int32_t* part = nullptr;
    const int* pbox = nullptr;
    uint64_t n_pbox = 0;
    const uint32_t* entry = nullptr;
    // Slab index of the source payload (rs_edge_index; nullable) and the source objects' own
    // boxes (as pbox): with both, only the payload's slabs that can hold an edge of an object
    // with a partner are checked for live edges.
    const long long* xindex = nullptr;
    const int* sbox = nullptr;
};

// Recheck statistics of the translation units that run hit tests (see rs_device.cuh).
int recheck_pim(int op, unsigned long long* out);
int recheck_join(int op, unsigned long long* out);
int recheck_batch(int op, unsigned long long* out);
int status_from_bits(uint32_t bits);
}  // namespace rs
