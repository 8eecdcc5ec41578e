/*
 * rayspace3d.h -- C ABI of the GB300 engine for the RaySpace3D query path (librs.so).
 *
 * Conventions (all entry points):
 *   - plain pointers and sizes; device pointers are prefixed d_, host pointers h_;
 *   - the caller owns every input and output buffer; engine objects are opaque
 *     handles released with the matching _destroy call;
 *   - work is issued on `stream` (a cudaStream_t passed as void*, NULL = legacy
 *     default stream) and the call returns after that stream has finished it,
 *     like the reference launchers, which synchronise after every launch
 *     (query/src/raytracing/RayLauncher.cpp:44-58, MeshOverlapEdgesLauncher.cpp:162-168);
 *   - every call returns an rs_status and never exits the process.
 *
 * Section 2 keeps the reference's own extern "C" helper signatures so the
 * reference host code links against this library unchanged.
 */
#ifndef RAYSPACE3D_H
#define RAYSPACE3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rs_status {
    RS_OK = 0,
    RS_ERR_CUDA = 1,            /* a CUDA runtime call failed */
    RS_ERR_INVALID = 2,         /* bad argument (null pointer, index out of range, size) */
    RS_ERR_TABLE_FULL = 3,      /* pair table could not place a key (caller may grow and retry) */
    RS_ERR_OUTPUT_OVERFLOW = 4, /* caller's output buffer is smaller than the result */
    RS_ERR_ITER_LIMIT = 5,      /* an iteration budget ran out; result not valid */
    RS_ERR_FORMAT = 6,          /* malformed input file */
    RS_ERR_OOM = 7,             /* device allocation failed */
    RS_ERR_TARGET_OVERFLOW = 8, /* reserved: containment handles any number of distinct targets */
    RS_ERR_TOO_LARGE = 9        /* input larger than a fixed-capacity entry point accepts */
} rs_status;

typedef struct rs_bvh rs_bvh;         /* triangle BVH of one geometry set, device resident */
typedef struct rs_pairset rs_pairset; /* open-addressing table of (id1<<32 | id2) pair keys */

/* ========================================================================== */
/* 1. Engine entry points                                                      */
/* ========================================================================== */

/* Library version string (diagnostics). */
const char* rs_version(void);

/* Build a BVH over all triangles of one set.
 * Replaces OptixAccelerationStructure::buildInternal (query/src/optix/OptixAccelerationStructure.cpp:22-68),
 * fed by GeometryUploader::upload (query/src/geometry/GeometryUploader.cpp:12-34).
 * d_vertices: float32[nV*3]; d_indices: uint32[nF*3]; d_tri2obj: int32[nF].  The three
 * arrays stay owned by the caller and must outlive the handle.  leaf_size in [1,16]
 * (0 = default 2): subtrees of at most leaf_size triangles become leaves.  Fails with
 * RS_ERR_INVALID if an index is >= nV. */
int rs_bvh_build(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                 const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, void* stream);
int rs_bvh_destroy(rs_bvh* bvh);

/* Asynchronous build (no counterpart in the reference): queues the same build on `stream`
 * and returns at once.  Queries on any stream are ordered after the build automatically;
 * rs_bvh_wait blocks until it is done and returns its status (RS_ERR_INVALID for
 * out-of-range vertex indices, which rs_bvh_build reports directly).  Two builds on two
 * streams run concurrently. */
int rs_bvh_build_async(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                       const int32_t* d_tri2obj, int leaf_size, rs_bvh** out, void* stream);
int rs_bvh_wait(const rs_bvh* bvh);
/* Number of triangles, nodes, engine-owned device bytes, and the bounds of all vertices. */
int rs_bvh_info(const rs_bvh* bvh, uint64_t* n_tri, uint64_t* n_nodes, uint64_t* bytes,
                float* h_min3, float* h_max3);

/* Point-in-mesh parity (replaces __raygen__rg, query/src/cuda/raytracing.cu:9-78, launched by
 * RayLauncher::launch, query/src/raytracing/RayLauncher.cpp:44-58).  One ray per point along
 * (dx,dy,dz) (the reference uses +Z); hits are ordered by distance and counted with the
 * reference's advance rule t_min = t + 1e-6; as in the reference's 10000-iteration loop, a
 * hit at a t where t + 1e-6 rounds to t (t >= 32) makes the count 10000, and no count
 * exceeds 10000.  d_obj[i] = object of the first counted hit
 * when the count is odd, else -1 (RayResult.polygon_index); d_inside[i] = count & 1.
 * Either output may be NULL.  d_points: float32[n*3]. */
int rs_pim(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
           int32_t* d_obj, uint8_t* d_inside, void* stream);

/* Filter-refine (replaces FilterRefinePipeline::execute, query/src/raytracing/FilterRefine.cpp:81-122):
 * parity against the 12-triangle box of all vertices (geometry/BoundingBox.cpp:12-50), then
 * parity against the mesh for the points the box test keeps, in one fused launch. */
int rs_pim_filtered(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
                    int32_t* d_obj, uint8_t* d_inside, void* stream);

/* Point-in-mesh without any device allocation (no counterpart in the reference).
 * For callers that cannot allocate device memory while they query: services whose own
 * allocator has reserved the whole GPU (a memory pool sized to the device leaves nothing
 * for cudaMalloc or a second pool), and hosts with a fixed device-memory budget checked
 * per request.  Same results as rs_pim / rs_pim_filtered (filtered != 0).  Per-call
 * scratch comes from a fixed 4 MiB array inside the library that every GPU which loads
 * it holds until the process exits; n above 1,048,576 points returns RS_ERR_TOO_LARGE.
 * The first call on a device looks the array up (cudaGetSymbolAddress); make that first
 * call before any stream capture.  The call waits for `stream` and returns once the
 * results are written.  All calls share the one array, so calls whose work overlaps on
 * the GPU (other streams or threads) race: serialise them.  It uses an axis-aligned
 * column grid only if an earlier rs_pim built it, never building one. */
int rs_pim_noalloc(const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy, float dz,
                   int32_t* d_obj, uint8_t* d_inside, int filtered, void* stream);

/* Ordered compaction of point results (replaces ResultProcessor::compactAndDownload,
 * query/src/raytracing/ResultProcessor.cpp:8-35): writes the ids of points with
 * d_obj[i] != -1, ascending, to d_point_ids and their objects to d_point_obj; *h_count
 * receives the number of hits.  RS_ERR_OUTPUT_OVERFLOW if it exceeds `capacity`. */
int rs_compact_hits(const int32_t* d_obj, uint64_t n, int32_t* d_point_ids, int32_t* d_point_obj,
                    uint64_t capacity, uint64_t* h_count, void* stream);

/* Pair tables (the hash tables of query/src/cuda/mesh_overlap_edges.cu:62-104 and
 * mesh_intersection.cu:108-132).  pow2 != 0: capacity is rounded up to a power of two and
 * slots are hash & (capacity-1); pow2 == 0: slot = hash % capacity (the intersection
 * variant).  A key that finds no slot raises RS_ERR_TABLE_FULL instead of being dropped. */
int rs_pairset_create(uint64_t capacity, int pow2, rs_pairset** out, void* stream);
int rs_pairset_clear(rs_pairset* ps, void* stream);
int rs_pairset_destroy(rs_pairset* ps);
/* Capacity in slots and number of distinct keys inserted so far. */
int rs_pairset_info(const rs_pairset* ps, uint64_t* capacity, uint64_t* count, void* stream);

/* Edge-ray overlap of one direction (replaces __raygen__mesh_overlap_edges,
 * query/src/cuda/mesh_overlap_edges.cu:183-216, and __raygen__mesh_overlap,
 * mesh_intersection.cu:288-334).  Each unique source edge is traced as the segment
 * t in [1e-6, |e-s| + 1e-6] along normalize(e-s) against `target`; the target object o of
 * every crossing the table's hit rule takes (rs_pairset_set_edge_rule) and every source
 * object k of the edge insert (k,o), or (o,k) when swap != 0.
 * Edge arrays are the .pre v2 edge payload on the device (float32[nE*3] starts/ends,
 * int32 offsets/counts[nE], int32 sources[]). */
int rs_edge_join(const rs_bvh* target, const float* d_starts, const float* d_ends,
                 const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources,
                 uint64_t nE, int swap, rs_pairset* ps, void* stream);

/* Containment fallback of one direction (replaces __raygen__mesh_containment_anyhit and
 * __anyhit__ah_containment, query/src/cuda/mesh_intersection_anyhit.cu:46-240): for every
 * source object, one +Z ray from the first vertex of its lowest-index triangle
 * (raytracer_intersection_estimated_main.cpp:539-552), t in [1e-4, 1e10]; a target object
 * crossed an odd number of times inserts (source,target), or (target,source) when swap. */
int rs_containment(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                   const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj,
                   int swap, rs_pairset* ps, void* stream);

/* Containment with the per-source diagnostics of raytracer_intersection_estimated
 * (query/src/utilities/PairHitTracking.h:31-150, ContainmentTracking.h:22-120): for every
 * source object o < capacity, d_candidate_counts[o] = number of distinct target objects the
 * ray crossed, and d_target_ids/d_target_hits[o*max_targets + j] = the odd-parity targets
 * (traversal order within passes of 32 ids) and how many of their triangles the ray crossed;
 * -1/0 where unused.
 * RS_ERR_OUTPUT_OVERFLOW if the source set has more than `capacity` objects. */
int rs_containment_tracked(const rs_bvh* target, const float* d_src_vertices, uint64_t src_nV,
                           const uint32_t* d_src_indices, uint64_t src_nF, const int32_t* d_src_tri2obj,
                           int swap, rs_pairset* ps, int max_targets, int32_t* d_target_ids,
                           uint32_t* d_target_hits, uint32_t* d_candidate_counts, uint64_t capacity, void* stream);

/* Query counters of a table (mesh_overlap_edges.cu:83-96 hash contention tracking and the
 * profiling counters of mesh_intersection.h:7-22), collected while tracking is on:
 * [0] slot accesses, [1] contended probes, [2] edge rays traced, [3] edge-ray hits taken
 * (overlap_hits_total), [4] containment rays, [5] containment crossings, [6] distinct
 * containment targets, [7] 0.  Counters reset with rs_pairset_clear. */
int rs_pairset_set_tracking(rs_pairset* ps, int on);
int rs_pairset_counters(const rs_pairset* ps, uint64_t* h_out8, void* stream);

/* Hit rule of the edge rays inserting into this table (the iteration cap and t_min step of
 * the reference's edge loops).  Each edge's crossings are taken in (distance, triangle id)
 * order as repeated closest-hit traces would return them: the first at t >= 1e-6, each next
 * at t >= the previous t + 1e-6 (t + 2e-4 when that float sum does not exceed t), at most
 * max_hits of them (max_hits <= 0 means 100); crossings skipped by the step, or beyond the
 * cap, add no pair.  Default (100, 0): trace_edge_multi_hits_edges of raytracer_mesh_overlap
 * and the estimated joins (query/src/cuda/mesh_overlap_edges.cu:106-178), with max_hits =
 * --overlap-max-iterations for raytracer_intersection_estimated (mesh_intersection.cu:16-91).
 * next_float != 0: the next t_min is the next float after t, the rule of raytracer_containment's
 * edge check (mesh_containment.cu:99-170, used there with max_hits = 256). */
int rs_pairset_set_edge_rule(rs_pairset* ps, int max_hits, int next_float);

/* Sorted unique keys of a table (replaces compact_hash_table_pairs + the sort/unique of
 * merge_and_deduplicate_pairs_gpu, query/src/cuda/mesh_query_deduplication.cu:56-144).
 * order 0: ascending (id1,id2); order 1: ascending (id2,id1), the order of
 * raytracer_mesh_overlap's output, whose dedup sorts MeshQueryResult{id1,id2} reinterpreted
 * as a little-endian u64.  d_keys receives up to `capacity` keys (id1<<32 | id2) and
 * *h_count the total; RS_ERR_OUTPUT_OVERFLOW if it exceeds capacity.  The function returns
 * after d_keys is written, unless `order` carries RS_FINALIZE_NO_WAIT: then, for up to 4096
 * keys that fit, it returns once the work is queued on `stream` (read d_keys in stream
 * order).  The count comes from the table's last status read (the one every join entry
 * point makes) when no launch has used the table since, else from a read of its own. */
#define RS_FINALIZE_NO_WAIT 0x100
int rs_pairset_finalize(rs_pairset* ps, int order, uint64_t* d_keys, uint64_t capacity,
                        uint64_t* h_count, void* stream);

/* Grid selectivity estimator (replaces estimateSelectivityKernel + thrust::reduce,
 * query/src/cuda/estimated_overlap.cu:8-77 and estimated_intersection.cu:8-79, plus the host
 * means calculateGlobalAvgSize / calculateGlobalAvgVolRatio,
 * raytracer_overlap_estimated_main.cpp:129-158).  d_cells*: GridCell{u32 CenterCount,
 * u32 TouchCount, f32 AvgSizeMean, f32 VolRatio}[ncells] on the device.  Writes the raw
 * sum (per-cell float values summed in double, fixed order) and, when h_means is non-NULL,
 * {avgSizeA, avgVolRatioA, avgSizeB, avgVolRatioB} as the reference host code computes them. */
int rs_estimate_grid(const void* d_cellsA, const void* d_cellsB, uint64_t ncells, float cell_volume,
                     float epsilon, float gamma, double* h_raw, float* h_means4, void* stream);

/* The per-cell estimates that rs_estimate_grid sums (estimateSelectivityKernel's result
 * buffer, query/src/cuda/estimated_overlap.cu:8-41): d_values[i] =
 * TA*TB*min(1, (SA+SB+eps)^3/cellVolume * sqrt(RA*RB)^gamma), 0 where either TouchCount is 0,
 * in the reference kernel's float operation order.  d_values: float32[ncells] on the device. */
int rs_estimate_grid_cells(const void* d_cellsA, const void* d_cellsB, uint64_t ncells, float cell_volume,
                           float epsilon, float gamma, float* d_values, void* stream);

/* Estimated pairs from the raw sum, as raytracer_overlap_estimated_main.cpp:275-291 does:
 * alpha = max(1, ((sA*cbrt(rA)) + (sB*cbrt(rB)))^3 / cellVolume), est = (int64)((float)raw/alpha);
 * alpha_correction == 0 uses alpha = 1 (raytracer_overlap_direct_estimation --no-alpha-correction). */
int64_t rs_estimate_pairs_from_raw(double raw, const float* h_means4, float cell_volume, int alpha_correction);

/* Hash table sizing rules of the reference:
 *   pow2 variant (raytracer_overlap_estimated_main.cpp:316-325): nextPow2(clamp(est/0.5, 1024, 2^30)),
 *     16777216 when est <= 0;
 *   odd variant (raytracer_intersection_estimated_main.cpp:466-477): clamp(est/loadFactor, 1024, 2^30)
 *     made odd, 16777216 when est <= 0. */
uint64_t rs_hash_size_pow2(int64_t estimated_pairs);
uint64_t rs_hash_size_odd(int64_t estimated_pairs, float load_factor);

/* The address through which the engine's kernels read the buffer at p (no counterpart in
 * the reference): device or managed memory as it is; pinned or registered host memory
 * through its mapped device address, read in place over the host link (only what a kernel
 * loads crosses it).  RS_ERR_INVALID for pageable host memory, which no kernel may read.
 * rs_overlap_join and rs_overlap_join_after resolve every edge-payload pointer this way, so
 * a payload may stay in pinned host memory: the join then reads only the endpoints of the
 * edges its broad phase keeps (all of them when every object has a partner). */
int rs_kernel_pointer(const void* p, const void** out);

/* Full joins with automatic table growth on RS_ERR_TABLE_FULL.  The table `ps` is cleared
 * first.  overlap: A-edges into B and B-edges into A (swapped).  intersection: overlap plus
 * containment in both directions.  direction: 0 both, 1 mesh1->mesh2 only, 2 mesh2->mesh1 only
 * (--query-direction). */
int rs_overlap_join(const rs_bvh* A, const float* d_startsA, const float* d_endsA, const int32_t* d_offsetsA,
                    const int32_t* d_countsA, const int32_t* d_sourcesA, uint64_t nEA,
                    const rs_bvh* B, const float* d_startsB, const float* d_endsB, const int32_t* d_offsetsB,
                    const int32_t* d_countsB, const int32_t* d_sourcesB, uint64_t nEB,
                    int direction, int with_containment, rs_pairset* ps, void* stream);

/* Slab index of an edge payload (no counterpart in the reference), built once per dataset:
 * d_index receives 3 + ceil(nE / 256) int64 -- [0] 1 when the payload is in the
 * reference's order (EdgePreprocessor's std::map over quantised endpoint pairs, so sorted by
 * the quantised x of each edge's lower endpoint, llround(x * 1e5)) and no source id is
 * negative, else 0; [1] the largest source id; [2] nE; [3 + b] the key of edge 256 * b.
 * *h_ordered (nullable) receives [0].  Pointers may be device or pinned host memory. */
int rs_edge_index(const float* d_starts, const float* d_ends, const int32_t* d_sources, uint64_t nE, uint64_t nS,
                  int64_t* d_index, int* h_ordered, void* stream);

/* rs_overlap_join_after with each payload's slab index (rs_edge_index; either nullable):
 * the live-edge check then reads only the slabs of 256 edges that can hold an edge of an
 * object the broad phase gave a partner -- an index whose [0] is 0, whose [2] is not the
 * payload's edge count, or whose largest source id is not an object of its set, makes the
 * check read every edge, as without one.  With
 * the payloads in pinned host memory a sparse join reads a few of their slabs over the host
 * link instead of all of them.  Same pair set as rs_overlap_join. */
int rs_overlap_join_indexed(const rs_bvh* A, const float* d_startsA, const float* d_endsA,
                            const int32_t* d_offsetsA, const int32_t* d_countsA, const int32_t* d_sourcesA,
                            uint64_t nEA, const int64_t* d_indexA, const rs_bvh* B, const float* d_startsB,
                            const float* d_endsB, const int32_t* d_offsetsB, const int32_t* d_countsB,
                            const int32_t* d_sourcesB, uint64_t nEB, const int64_t* d_indexB, int direction,
                            int with_containment, rs_pairset* ps, void* edges_a_ready, void* edges_b_ready,
                            void* stream);

/* rs_overlap_join whose edge payloads may still be in flight (no counterpart in the
 * reference): the broad phase runs at once, each direction's edge rays wait on the stream
 * for the caller's event (cudaEvent_t; nullable) marking its source payload as written --
 * edges_a_ready for the A->B rays, edges_b_ready for B->A.  A host that copies the payloads
 * in hides the broad phase, and the first direction, behind the copies. */
int rs_overlap_join_after(const rs_bvh* A, const float* d_startsA, const float* d_endsA, const int32_t* d_offsetsA,
                          const int32_t* d_countsA, const int32_t* d_sourcesA, uint64_t nEA,
                          const rs_bvh* B, const float* d_startsB, const float* d_endsB, const int32_t* d_offsetsB,
                          const int32_t* d_countsB, const int32_t* d_sourcesB, uint64_t nEB,
                          int direction, int with_containment, rs_pairset* ps, void* edges_a_ready,
                          void* edges_b_ready, void* stream);

/* Overlap (with_containment = 0) or full intersection join straight from two device
 * geometries (no counterpart in the reference): every object's box is computed, objects
 * whose widened box overlaps no widened object box of the other set are dropped, and each
 * set's BVH (leaf_size as rs_bvh_build) is built over the triangles of its remaining
 * objects only.  Same pair set as rs_bvh_build of both sets + rs_overlap_join, with the
 * same table growth; the BVHs live only inside the call.  Sparse joins build and trace a
 * small fraction of the data. */
int rs_overlap_join_filtered(const float* d_VA, uint64_t nVA, const uint32_t* d_IA, uint64_t nFA,
                             const int32_t* d_TA, const float* d_startsA, const float* d_endsA,
                             const int32_t* d_offsetsA, const int32_t* d_countsA, const int32_t* d_sourcesA,
                             uint64_t nEA, const float* d_VB, uint64_t nVB, const uint32_t* d_IB, uint64_t nFB,
                             const int32_t* d_TB, const float* d_startsB, const float* d_endsB,
                             const int32_t* d_offsetsB, const int32_t* d_countsB, const int32_t* d_sourcesB,
                             uint64_t nEB, int direction, int with_containment, int leaf_size, rs_pairset* ps,
                             void* stream);

/* Broad phase of rs_overlap_join (no counterpart in the reference), on by default: each
 * object's box is tested against the other set's triangle boxes, both widened by more
 * than the edge payload's quantisation and the slab arithmetic's rounding; edges whose
 * source objects overlap nothing are not traced.  The pair set is the same with it on or
 * off; rs_set_overlap_cull(0) traces every edge. */
int rs_set_overlap_cull(int on);

/* Status text for a code. */
const char* rs_status_string(int status);

/* Batched queries in one persistent launch (no counterpart in the reference, which
 * launches and synchronises per query: RayLauncher.cpp:39-64, MeshIntersectionLauncher.cpp:
 * 279-328).  Point-in-mesh queries and edge-ray directions of any sizes are split into
 * chunks that the warps of one persistent kernel pull from a global counter; rays with
 * more than 8 crossings are resolved exactly by a second launch.  An unchanged batch is
 * captured as a CUDA graph on its first submit (on a non-default stream) and replayed
 * afterwards.  Inputs, outputs and pair sets stay owned by the caller and must outlive
 * the batch; edge queries insert into their pair set, which the caller clears. */
typedef struct rs_batch rs_batch;
int rs_batch_create(rs_batch** out);
int rs_batch_destroy(rs_batch* batch);
int rs_batch_add_pim(rs_batch* batch, const rs_bvh* bvh, const float* d_points, uint64_t n, float dx, float dy,
                     float dz, int32_t* d_obj, uint8_t* d_inside, int* index);
int rs_batch_add_edges(rs_batch* batch, const rs_bvh* target, const float* d_starts, const float* d_ends,
                       const int32_t* d_offsets, const int32_t* d_counts, const int32_t* d_sources, uint64_t nE,
                       int swap, rs_pairset* ps, int* index);
/* chunk: rays a warp takes per pull (multiple of 32, default 64); stack_depth: 32 or 64
 * traversal stack entries (default 64); use_graph: capture and replay (default 1). */
int rs_batch_set_options(rs_batch* batch, int chunk, int stack_depth, int use_graph);
int rs_batch_submit(rs_batch* batch, void* stream);
/* Waits for the last submit; per-query statuses into h_status (nullable); returns the
 * first failing one. */
int rs_batch_wait(rs_batch* batch, int* h_status);
/* Times the batch over BVH leaf sizes {2,4,8,16}, chunks {32,64,128} and stack depths
 * {32,64} (three runs each, configurations whose queries fail are skipped), keeps the
 * fastest (rebuilding the batch's BVHs with its leaf size when it differs from the
 * caller's) and reports it. */
int rs_batch_autotune(rs_batch* batch, int* h_leaf_size, int* h_chunk, int* h_stack_depth, double* h_ms,
                      void* stream);

/* Grid statistics on the GPU (generateGridStats, preprocess/src/preprocess_dataset.cpp:37-181)
 * for a triangle set in device memory: d_cells receives resolution^3 GridCell records
 * (16 B: u32 CenterCount, u32 TouchCount, f32 AvgSizeMean, f32 VolRatio; index
 * (z*R+y)*R+x); the frame is [0, world_size]^3, or the bounds of all vertices when
 * world_size <= 0 (h_bounds6 receives min xyz, max xyz; nullable).  Objects are ids
 * 0..n_obj-1 (RS_ERR_INVALID if a valid triangle names another).  Bit-identical to the
 * reference: per-object volumes are summed in triangle order and per-cell float sums in the
 * reference's object visit order (its std::unordered_map iteration order). */
int rs_grid_stats(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                  const int32_t* d_tri2obj, uint64_t n_obj, int resolution, float world_size, void* d_cells,
                  float* h_bounds6, void* stream);

/* Legacy per-triangle overlap, one direction (mesh_overlap.cu:126-179, compiled but not
 * launched by the reference's mains): every edge of every source triangle, in the
 * triangle's own orientation (v0v1, v1v2, v2v0) and with the triangle's object as its
 * source, is traced against `target` like an edge of rs_edge_join; shared edges are traced
 * once per triangle.  Needs no precomputed edge payload.  RS_ERR_INVALID (pairs of the valid
 * triangles still inserted) when a source index is >= nV. */
int rs_triangle_join(const rs_bvh* target, const float* d_vertices, uint64_t nV, const uint32_t* d_indices,
                     uint64_t nF, const int32_t* d_tri2obj, int swap, rs_pairset* ps, void* stream);

/* Unique-edge payload on the GPU (EdgePreprocessor::extractEdges,
 * preprocess/src/EdgePreprocessor.cpp:41-119), identical to the reference's: edges keyed by
 * their endpoints quantised with llround(x * 1e5) and ordered as the reference's std::map
 * orders the keys; each edge's endpoints are those of its first occurrence (triangle order,
 * edges v0v1, v1v2, v2v0) in that occurrence's orientation; sources are the distinct objects
 * in first-seen order.  Triangles with an index >= nV are skipped.  Outputs: d_starts and
 * d_ends (float3 per edge), d_offsets and d_counts (int32 per edge) and d_sources (int32 per
 * source), each with room for `capacity` entries (3 * nF always suffices).  *h_nE and *h_nS
 * receive the edge and source counts; RS_ERR_OUTPUT_OVERFLOW (outputs untouched) when either
 * exceeds capacity; RS_ERR_TOO_LARGE above 715,827,882 triangles. */
int rs_extract_edges(const float* d_vertices, uint64_t nV, const uint32_t* d_indices, uint64_t nF,
                     const int32_t* d_tri2obj, float* d_starts, float* d_ends, int32_t* d_offsets,
                     int32_t* d_counts, int32_t* d_sources, uint64_t capacity, uint64_t* h_nE, uint64_t* h_nS,
                     void* stream);

/* Learned selectivity estimator (no counterpart in the reference): a
 * 32768 -> 512 -> 512 -> 1 ReLU MLP on pooled grid features predicting log1p(pairs),
 * trained and evaluated with the engine's BF16 tensor-core GEMM kernels (FP32 accumulate,
 * FP32 master weights, Adam).  Features (rs_mlp_features): each grid pooled to 16^3
 * blocks x {log1p sum CenterCount, log1p sum TouchCount, log1p TouchCount-weighted
 * AvgSizeMean, TouchCount-weighted VolRatio}, side A then side B (32768 floats).
 * Parameters are one FP32 array of rs_mlp_num_params() values: W1[512][32768], b1[512],
 * W2[512][512], b2[512], W3[512], b3[1]. */
typedef struct rs_mlp rs_mlp;
int rs_mlp_create(uint64_t seed, rs_mlp** out);
int rs_mlp_destroy(rs_mlp* mlp);
uint64_t rs_mlp_num_params(void);
int rs_mlp_get_params(const rs_mlp* mlp, float* h_params, float* h_grads);
int rs_mlp_set_params(rs_mlp* mlp, const float* h_params);
int rs_mlp_features(const void* d_cellsA, const void* d_cellsB, int resolution, float* d_out32768, void* stream);
/* d_X: B rows of 32768 FP32 features; d_y: B predictions (log1p pairs). */
int rs_mlp_forward(rs_mlp* mlp, const float* d_X, int B, float* d_y, void* stream);
/* Mean squared error against d_target and its gradients (read with rs_mlp_get_params). */
int rs_mlp_gradients(rs_mlp* mlp, const float* d_X, const float* d_target, int B, float* h_loss, void* stream);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on a minibatch. */
int rs_mlp_train_step(rs_mlp* mlp, const float* d_X, const float* d_target, int B, float lr, float* h_loss,
                      void* stream);
/* GEMM path of the MLP: 0 (default) runs the products whose operands are both K-major -- the
 * forward pass -- on the tcgen05 tensor cores (TMA-fed shared memory, tensor-memory
 * accumulators) and the rest on mma.sync tiles; 1 runs every product on mma.sync.  Calls
 * return RS_ERR_ITER_LIMIT if a tcgen05 kernel's bounded wait ran out. */
int rs_mlp_set_gemm(int mode);
/* The MLP's GEMM alone: C[m][n] = sum_k A[m][k] B[n][k] (BF16 row-major A [M][lda], B [N][ldb],
 * FP32 C [M][ldc], all on the device); mode 0 tcgen05 (RS_ERR_INVALID unless N % 256 == 0,
 * K % 64 == 0, 16-byte aligned operands and lda, ldb multiples of 8), mode 1 mma.sync. */
int rs_mlp_gemm(const void* d_A, int lda, const void* d_B, int ldb, float* d_C, int ldc, int M, int N, int K,
                int mode, void* stream);
/* Decoupled weight decay of W1, W2 and W3 in rs_mlp_train_step (default 0; no counterpart
 * in the reference). */
int rs_mlp_set_weight_decay(rs_mlp* mlp, float weight_decay);
/* Grid-estimator prior (no counterpart in the reference): with on != 0, rs_estimate_mlp
 * adds the network's output to log1p(grid estimate) of the same two grids (rs_estimate_grid
 * with cell_volume, epsilon, gamma, then rs_estimate_pairs_from_raw with alpha_correction),
 * so the network is trained on the correction of the grid estimator rather than on the
 * count itself.  Off by default. */
int rs_mlp_set_prior(rs_mlp* mlp, int on, float cell_volume, float epsilon, float gamma, int alpha_correction);
/* Estimated pair count of two grids (expm1 of the prediction, rounded; h_log1p nullable). */
int rs_estimate_mlp(rs_mlp* mlp, const void* d_cellsA, const void* d_cellsB, int resolution, int64_t* h_estimate,
                    double* h_log1p, void* stream);

/* Diagnostics (no counterpart in the reference).  rs_launch_count: kernels launched by this
 * library since load.  rs_profile_*: when enabled, device time of the main kernels is
 * accumulated with CUDA events on the launching stream; ids 0 edge join, 1 containment,
 * 2 point-in-mesh, 3 BVH build (whole), 4 pair finalisation, 5 estimator, 6 the build's
 * bottom-up tree kernel alone, 7 the learned estimator's GEMMs (with their split-K sums). */
uint64_t rs_launch_count(void);
/* Device allocations the library has requested from its stream-ordered memory pool since
 * it was loaded (diagnostics; no counterpart in the reference). */
uint64_t rs_alloc_count(void);
int rs_profile_enable(int on);
int rs_profile_reset(void);
int rs_profile_read(int kernel, double* total_ms, uint64_t* launches);

/* Recheck rate of the exact hit contract (no counterpart in the reference): the number of
 * edge signs the FP32 error filter could not decide and that were re-evaluated exactly
 * (always counted), and the number of ray/triangle tests (counted while enabled; costs one
 * atomic per ray).  Rate = exact_signs / (3 * triangle_tests) at most. */
int rs_recheck_enable(int on);
int rs_recheck_reset(void);
int rs_recheck_read(uint64_t* exact_signs, uint64_t* triangle_tests);

/* ========================================================================== */
/* 2. Reference-compatible helpers (same names and signatures as the reference) */
/* ========================================================================== */

/* query/src/cuda/scan_utils.h:7-9 -- exclusive scan of int counts into int64 offsets; returns the total. */
long long exclusive_scan_gpu(const int* d_input, long long* d_output, int num_elements);

/* query/src/cuda/mesh_query_deduplication.h:6-18.  Pairs are MeshQueryResult{int,int} (8 bytes).
 * merge: concatenates both inputs into d_merged_output, sorts them as little-endian u64 and
 * removes duplicates; returns the unique count.  compact: copies occupied slots of a pair
 * table, in slot order, to d_output; returns min(count, max_output_size). */
long long merge_and_deduplicate_pairs_gpu(const void* d_results1, long long num_results1,
                                          const void* d_results2, long long num_results2,
                                          void* d_merged_output);
int compact_hash_table_pairs(const unsigned long long* d_hash_table, unsigned long long table_size,
                             void* d_output, int max_output_size);

/* query/src/cuda/result_compaction.h:5-22.  RayResult{int ray_id; int polygon_index}. */
int count_hits_gpu(const void* d_results, int num_results);
void compact_hits_gpu(const void* d_input, void* d_output, int num_results, int* h_num_hits);

/* The estimators of query/src/cuda/estimated_overlap.h:6-13 and estimated_intersection.h:6-13
 * with C linkage (no counterpart in the reference, for C and FFI callers): host GridCell
 * arrays (16 B records), returns the raw estimate (-1.0f if device memory cannot be
 * allocated).  The raw sum is accumulated in double in a fixed order and rounded to float
 * once; the reference's thrust::reduce sums the per-cell floats in float in its own order,
 * so the two can differ in the last bits of the float. */
float rs_estimate_overlap_selectivity(const void* h_gridA, const void* h_gridB, int numCells, float cellVolume,
                                      float epsilon, float gamma);
float rs_estimate_intersection_selectivity(const void* h_gridA, const void* h_gridB, int numCells,
                                           float cellVolume, float epsilon, float gamma);

#ifdef __cplusplus
}

/* The same two estimators with the reference's exact C++ declarations
 * (query/src/cuda/estimated_overlap.h:6-13, estimated_intersection.h:6-13; GridCell as
 * common/include/GridCell.h:5-10 defines it), so the reference's mains
 * (raytracer_overlap_estimated_main.cpp:266, raytracer_overlap_direct_estimation_main.cpp:384)
 * link against this library unchanged.  Include either this header or the reference's
 * estimated_*.h in one translation unit, not both (both give default arguments). */
struct GridCell;
float estimateOverlapSelectivity(const GridCell* h_gridA, const GridCell* h_gridB, int numCells, float cellVolume,
                                 float epsilon = 0.001f, float gamma = 0.8f);
float estimateIntersectionSelectivity(const GridCell* h_gridA, const GridCell* h_gridB, int numCells,
                                      float cellVolume, float epsilon = 0.001f, float gamma = 0.8f);
#endif

#endif /* RAYSPACE3D_H */
