/*
 * oracle.h -- CPU oracle for the RaySpace3D query path (TEST INFRASTRUCTURE).
 *
 * This library is the checker, never the product: only tests/, the smoke()
 * entry of __graft_entry__.py and the cpu_baseline / reference leg of bench.py
 * may load it.  The GPU engine (librs) never links or calls it.
 *
 * It restates, on the CPU, the reference query semantics:
 *   - point-in-mesh parity along a ray (query/src/cuda/raytracing.cu:9-78)
 *   - filter-refine with the 12-triangle bounding box mesh
 *     (query/src/raytracing/FilterRefine.cpp:81-122, geometry/BoundingBox.cpp:12-50)
 *   - edge-ray overlap (query/src/cuda/mesh_overlap_edges.cu:106-216)
 *   - any-hit containment fallback (query/src/cuda/mesh_intersection_anyhit.cu:46-240)
 *   - sorted unique pair keys (query/src/cuda/mesh_query_deduplication.cu:56-120)
 *   - the grid selectivity estimator (query/src/cuda/estimated_overlap.cu:8-41,
 *     query/src/applications/raytracer_overlap_estimated_main.cpp:129-158,252-325)
 *   - the preprocessing payloads: unique edges (preprocess/src/EdgePreprocessor.cpp:41-119)
 *     and grid statistics (preprocess/src/preprocess_dataset.cpp:37-179)
 * under the engine's exact hit contract (exact-sign orientation predicates with
 * a symbolic-perturbation tie-break, float hit distance by a fixed operation
 * sequence clamped to the triangle's slab interval).  Its exact arithmetic is a
 * big-integer evaluation, independent of the GPU's FP64 expansion arithmetic.
 *
 * Parity against OptiX itself is unpinned: the reference ships no tests or
 * golden vectors for this path and its ray/triangle test is closed.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Point-in-mesh parity.  out_obj[i] = object of the first counted hit when the
 * number of counted crossings is odd, else -1.  use_bvh=0 tests every triangle. */
int orc_pim(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
            const float* pts, uint64_t n, float dx, float dy, float dz,
            int32_t* out_obj, int nthreads, int use_bvh);

/* Filter-refine: parity against the bounding-box mesh first, then against the mesh. */
int orc_pim_filtered(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                     const float* pts, uint64_t n, float dx, float dy, float dz,
                     int32_t* out_obj, int nthreads, int use_bvh);

/* Edge-ray overlap of one direction: the edges of the source set against the
 * triangles of the target set, each edge's crossings taken by the reference's edge loop
 * (at most max_hits, <= 0 meaning 100; t_min stepped by 1e-6, or to the next float when
 * next_float).  Returns sorted unique keys (id1<<32 | id2) in a malloc'd buffer (*keys,
 * *nkeys); free with orc_free.  swap=1 emits (target,source). */
int orc_edge_join(const float* starts, const float* ends, const int32_t* offsets, const int32_t* counts,
                  const int32_t* sources, uint64_t nE,
                  const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                  int swap, uint64_t** keys, uint64_t* nkeys, int nthreads, int use_bvh, int max_hits,
                  int next_float);

/* Every crossing of the segment start -> end with t in [1e-6, len + 1e-6] (all triangles
 * tested, unsorted): up to cap (t, triangle) pairs; *n receives the total. */
int orc_segment_hits(const float* start, const float* end, const float* V, uint64_t nV, const uint32_t* I,
                     uint64_t nF, const int32_t* tri2obj, float* out_t, uint64_t* out_tri, uint64_t cap,
                     uint64_t* n);

/* Containment fallback of one direction: one +Z ray per source object from the
 * first vertex of its lowest-index triangle, parity per target object. */
int orc_containment(const float* srcV, uint64_t srcNV, const uint32_t* srcI, uint64_t srcNF, const int32_t* srcT2O,
                    const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                    int swap, uint64_t** keys, uint64_t* nkeys, int nthreads, int use_bvh);

/* Containment (swap=0) with the per-source diagnostics of the tracked variant
 * (query/src/utilities/PairHitTracking.h:31-150): out_candidates[o] = distinct target
 * objects crossed (capacity >= number of source objects, else returns 1); the odd-parity
 * (source<<32 | target) keys, sorted, with the number of the target's triangles crossed. */
int orc_containment_diag(const float* srcV, uint64_t srcNV, const uint32_t* srcI, uint64_t srcNF,
                         const int32_t* srcT2O, const float* V, uint64_t nV, const uint32_t* I, uint64_t nF,
                         const int32_t* tri2obj, uint32_t* out_candidates, uint64_t capacity,
                         uint64_t** odd_keys, uint32_t** odd_hits, uint64_t* n_odd, int nthreads);

/* Grid estimator raw sum (float per-cell values summed in double, index order). */
double orc_estimate_raw(const void* cellsA, const void* cellsB, uint64_t ncells,
                        float cellVolume, float epsilon, float gamma);

/* Full estimate as the reference host computes it (alpha correction optional). */
int64_t orc_estimate_pairs(const void* cellsA, const void* cellsB, uint64_t ncells,
                           const float minA[3], const float maxA[3], const uint32_t resA[3],
                           float epsilon, float gamma, int alpha_correction, double* raw_out);

/* Exact sign of det[d, a-o, b-o] and of the tie-break determinants; exposed for tests. */
int orc_orient(const float d[3], const float o[3], const float a[3], const float b[3]);
int orc_perturbed_sign(const float d[3], const float o[3], const float a[3], const float b[3]);

/* The 12-triangle bounding-box mesh of all vertices (BoundingBox.cpp:4-50):
 * out_v float[24] (8 vertices), out_i uint32[36] (12 triangles). */
void orc_box_mesh(const float* V, uint64_t nV, float* out_v, uint32_t* out_i);

/* Unique-edge payload (EdgePreprocessor.cpp:41-119): an ordered map from the quantised
 * endpoint pair to the first occurrence's endpoints and the distinct source objects in
 * first-seen order.  Arrays are malloc'd (free with orc_free); *nE, *nS their lengths. */
int orc_extract_edges(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* T,
                      float** starts, float** ends, int32_t** offsets, int32_t** counts, int32_t** sources,
                      uint64_t* nE, uint64_t* nS);

/* Grid statistics (preprocess_dataset.cpp:37-179) into res^3 16-byte cells; bounds6
 * receives the frame (min xyz, max xyz). */
void orc_grid_stats(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* T, int res,
                    float world_size, void* cells, float* bounds6);

void orc_free(void* p);

#ifdef __cplusplus
}
#endif
