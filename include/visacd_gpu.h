/*
 * visacd_gpu.h — C ABI of the GB300 (sm_103a) visibility-edge decomposition kernels.
 *
 * Plain C types only: host-owned handles, raw pointers, sizes and an int status
 * (0 = ok, otherwise a visacd_status code; visacd_last_error() returns the message
 * of the calling thread's most recent failure). Nothing here calls exit().
 *
 * Threading: a visacd_ctx owns one CUDA stream and a set of grow-only device
 * buffers. A context is not thread-safe; use one per host thread. Calls taking
 * `device_ptrs = 0` read and write host memory and return after the result is
 * on the host. Calls taking `device_ptrs = 1` read and write device memory and
 * are asynchronous on the context stream unless they also return host-side
 * counts (documented per call).
 *
 * Reference interfaces these entry points replace (paths inside the VisACD
 * source tree):
 *   classify_and_rate_planes ........ lib/cuda/plane_intersections.cu:71-133
 *   visacd_score_planes ............. same, with FP64 scores, exact crossing
 *                                     classification and a first-max argmax
 *                                     (lib/src/process.cpp:123-134)
 *   visacd_bvh_build ................ optixAccelBuild, lib/src/intersections.cpp:131-180
 *   visacd_visibility ............... run_optix + the host scan of
 *                                     compute_intersection_matrix,
 *                                     lib/src/intersections.cpp:75-385 and
 *                                     lib/ptx/ray_segments.cu:49-125
 *   visacd_compute_intersection_matrix  compute_intersection_matrix,
 *                                     lib/include/intersections.hpp:24
 *   visacd_candidate_planes ......... get_candidate_planes after the draws,
 *                                     lib/src/process.cpp:28-72
 *   visacd_split_search ............. the split search of decompose_iteration,
 *                                     lib/src/process.cpp:96-134
 *   visacd_learned_split_search ..... the same split search with the learned
 *                                     proposer (no reference counterpart) in
 *                                     place of most of the candidate draw
 *   visacd_convex_hulls ............. Mesh::compute_ch for a batch of parts,
 *                                     lib/src/core.cpp:59-111 (qhull replaced
 *                                     by this project's QuickHull)
 *   visacd_hull_distances ........... mesh_dist of multimerge_ch,
 *                                     lib/src/cost.cpp:125-159
 */
#ifndef VISACD_GPU_H
#define VISACD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VISACD_ABI_VERSION 1

typedef enum {
  VISACD_OK = 0,
  VISACD_ERR_INVALID_ARG = 1,  /* bad size, null pointer, index out of range */
  VISACD_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  VISACD_ERR_NO_MEMORY = 3,    /* device or pinned allocation failed */
  VISACD_ERR_CAPACITY = 4,     /* caller's output buffer is too small */
  VISACD_ERR_DEVICE = 5        /* a kernel reported a bounded-loop overrun */
} visacd_status;

typedef struct visacd_ctx visacd_ctx;
typedef struct visacd_bvh visacd_bvh;
typedef struct visacd_batch visacd_batch;

/* Counters of one visibility call. */
typedef struct {
  int64_t pairs_tested;   /* pairs whose segment was traced (mask applied) */
  int64_t n_edges;        /* visibility edges: cage hit and no self hit */
  int64_t self_hits;      /* pairs whose segment leaves the cage and crosses the part */
  int64_t cage_hits;      /* pairs whose segment leaves the cage (tested first) */
  int64_t fp64_rechecks;  /* segment-triangle tests re-decided in FP64 */
  int64_t degenerate;     /* pairs with coincident endpoints (never edges) */
  int64_t node_visits;    /* BVH node records fetched (per warp packet) */
  int64_t tri_tests;      /* segment-triangle tests started (per segment) */
} visacd_vis_stats;

/* Sizes of one clip result (the cap is triangulated by the caller). */
typedef struct {
  int32_t n_pos, n_neg;        /* triangles of the positive / negative part, without the cap */
  int32_t nv_pos, nv_neg;      /* original vertices kept by each part */
  int32_t n_border;            /* border points (appended after the kept vertices of both parts) */
  int32_t n_border_edges;      /* unique border edges, 1-based border point pairs */
  int32_t n_touching;          /* triangles touching the plane (resolved in order) */
} visacd_clip_result;

/* Counters of one scoring call. */
typedef struct {
  int32_t quantum_exp;    /* edge lengths are summed in units of 2^quantum_exp */
  int32_t argmax;         /* first plane with the maximum score, -1 if P == 0 */
  int64_t band_blocks;    /* (plane, edge block) pairs re-decided in FP64 */
  int64_t skipped_edges;  /* edges with an out-of-range index or non-finite endpoint */
} visacd_score_stats;

/* ---- errors, version ---------------------------------------------------- */
const char* visacd_last_error(void);
int visacd_abi_version(void);

/* ---- context ------------------------------------------------------------ */
/* cuda_stream: a cudaStream_t to run on, or NULL to create a private stream. */
int visacd_ctx_create(int device, void* cuda_stream, visacd_ctx** out);
int visacd_ctx_destroy(visacd_ctx* ctx);
int visacd_ctx_synchronize(visacd_ctx* ctx);
/* Per-kernel CUDA-event timing on the context stream (off by default). */
int visacd_ctx_set_timing(visacd_ctx* ctx, int enable);
/* How this context's calls wait for the GPU: 0 (default) spins, the lowest
   latency for a single caller; 1 sleeps on a blocking-sync event, leaving the
   cores to other host threads when many contexts share one machine. */
int visacd_ctx_set_blocking_wait(visacd_ctx* ctx, int enable);
int visacd_ctx_reset_times(visacd_ctx* ctx);
/* Accumulated time and launch count per kernel name since the last reset.
   Synchronizes the stream. names[i] stay valid for the life of the library. */
int visacd_ctx_kernel_times(visacd_ctx* ctx, const char** names, double* total_ms,
                            int64_t* launches, int capacity, int* n_kernels);
/* Number of kernel launches issued on this context since creation. */
int64_t visacd_ctx_launch_count(const visacd_ctx* ctx);
int visacd_ctx_sm_count(const visacd_ctx* ctx);
/* The device sort the BVH build and the visibility ordering use: a stable
   sort of (keys[i], vals[i]) by key (keys below 2^key_bits), host arrays
   sorted in place. Up to 512 pairs: a bitonic sort in one CTA's shared
   memory; up to 32768: one CTA running every 8-bit LSD pass; beyond: three
   launches per pass. Synchronizes. */
int visacd_radix_sort_pairs(visacd_ctx* ctx, uint64_t* keys, uint32_t* vals, int32_t n, int key_bits);

/* How host threads wait for this process's work on `device`: blocking = 1
   makes waiting threads sleep until the GPU finishes (cudaDeviceScheduleBlockingSync)
   instead of spinning, which frees host cores when many threads drive the GPU
   (process_batch); 0 restores the default (automatic) policy. Per process. */
int visacd_set_blocking_sync(int device, int blocking);

/* FP32 FMA throughput of this GPU in TFLOP/s (packed f32x2 FMA loop, best of
   3 timed launches): the denominator of the FP32-bound rooflines. */
int visacd_measure_fp32_peak(visacd_ctx* ctx, double* tflops);
/* Texture fetch rate of this GPU (G fetches/s, point-sampled tex3D<float> from
   a cache-resident texture), the denominator of the free-space walk's
   roofline: coherent = a warp reads an 8 x 4 block of neighbouring texels (the
   best case), divergent = every lane walks its own line through the texture.
   Synchronizes. */
int visacd_measure_tex_peak(visacd_ctx* ctx, double* coherent_gfetch, double* divergent_gfetch);

/* ---- BVH ---------------------------------------------------------------- */
/* Linear BVH over a triangle mesh: 63-bit Morton codes of triangle centroids,
   LSD radix sort, Karras (2012) hierarchy, bottom-up AABB fit. verts is nv x 3
   float32, tris is nt x 3 uint32 (indices < nv, else VISACD_ERR_INVALID_ARG).
   device_ptrs selects host or device input. The BVH keeps the vertex indices
   of every triangle so a visibility query can skip triangles incident to the
   segment's endpoints. Synchronizes. */
int visacd_bvh_build(visacd_ctx* ctx, const float* verts, int32_t nv, const uint32_t* tris,
                     int32_t nt, int device_ptrs, visacd_bvh** out);
int visacd_bvh_destroy(visacd_bvh* bvh);
int visacd_bvh_info(const visacd_bvh* bvh, int32_t* n_tris, int32_t* depth);

/* ---- visibility --------------------------------------------------------- */
/* For every unordered vertex pair i < j of pts (n x 3 float32) — or, when
   is_new != NULL, every pair with at least one is_new[] != 0 endpoint — trace
   the segment p_i -> p_j over t in [0.001 / |p_j - p_i|, 1]. The pair is a
   visibility edge iff the segment hits cage_bvh and does not hit self_bvh,
   where triangles of self_bvh incident to i or j are skipped (the end-vertex
   policy). Segment-triangle tests run in FP32 with a rigorous rounding bound;
   tests inside the bound are re-decided in FP64. Edges are kept on the device
   in row-major (i, j) order; fetch them with visacd_visibility_edges*.
   Returns the edge count in *n_edges. Synchronizes. */
int visacd_visibility(visacd_ctx* ctx, const float* pts, int32_t n, const uint8_t* is_new,
                      int device_ptrs, const visacd_bvh* self_bvh, const visacd_bvh* cage_bvh,
                      int64_t* n_edges, visacd_vis_stats* stats);
/* Copy the last visibility result (2 x n_edges uint32, i < j) to host memory. */
int visacd_visibility_edges(visacd_ctx* ctx, uint32_t* edges_out, int64_t capacity_edges);
/* Several parts in one call: the pending sub-parts of a decomposition step.
   Part p has n_pts[p] points pts[p] (float32 n x 3, host), an optional is_new
   mask (is_new may be NULL, or is_new[p] NULL for an unmasked part), its own
   BVH and its cage BVH. Each part is prepared on its own (Morton order, the
   masked rows), then one persistent visibility launch covers the work items of
   all parts and one compaction emits every part's edges, parts in order, each
   as visacd_visibility would (row-major, its own vertex indices). n_edges[p]
   gets part p's edge count; visacd_visibility_edges then returns all of them
   concatenated. stats (may be NULL) sums the counters over the parts. Results
   equal one visacd_visibility call per part. Replaces the per-part
   compute_intersection_matrix calls of lib/src/process.cpp:165-178. */
int visacd_visibility_batch(visacd_ctx* ctx, int32_t n_parts, const float* const* pts,
                            const int32_t* n_pts, const uint8_t* const* is_new,
                            const visacd_bvh* const* self_bvhs, const visacd_bvh* const* cage_bvhs,
                            int64_t* n_edges, visacd_vis_stats* stats);
/* Device pointer to the last visibility result (valid until the next call). */
int visacd_visibility_edges_device(visacd_ctx* ctx, const uint32_t** d_edges, int64_t* n_edges);

/* Launch shapes of the visibility kernel (tile rows x columns per warp and the
   resident-CTA target). variant -1 restores automatic choice: the autotuned
   shape for the call's shape class if one was measured, else variant 1 (8 x 4
   tiles, 8 resident CTAs per SM). */
int visacd_vis_variant_count(void);
int visacd_ctx_set_vis_variant(visacd_ctx* ctx, int variant);
/* Autotuner: times every launch shape on this exact call (twice each, CUDA
   events on the context stream), caches the fastest for the call's shape class
   (log2 buckets of n and of both triangle counts, masked or not) in the
   context, and reports it. ms_per_variant (optional) gets
   visacd_vis_variant_count() entries. Resets the context's kernel timers. */
int visacd_autotune_visibility(visacd_ctx* ctx, const float* pts, int32_t n, const uint8_t* is_new,
                               int device_ptrs, const visacd_bvh* self_bvh,
                               const visacd_bvh* cage_bvh, int* best_variant,
                               double* ms_per_variant);

/* Free-space walks (on by default). A visibility call (or a part of a
   batched call) with at least 2^22 pairs first walks each segment through a grid over its cage that bounds,
   per cell, the distance to the cage's triangles (built once per cage BVH,
   kept with it): a segment whose whole length the walk covers cannot hit the
   cage and skips the cage BVH; every other segment is traced as before. The
   edges are the same either way. visacd_ctx_vis_trace_counts reports, for the
   context's last visacd_visibility call, the segments cleared this way and
   the grid cells read. */
int visacd_ctx_set_vis_trace(visacd_ctx* ctx, int enable);
int visacd_ctx_vis_trace_counts(const visacd_ctx* ctx, int64_t* cleared, int64_t* grid_reads);

/* One call that builds both BVHs, runs visacd_visibility and copies the edges
   out: the C form of compute_intersection_matrix(mesh, cage). If the edge
   count exceeds capacity_edges, *n_edges holds the count and the call returns
   VISACD_ERR_CAPACITY without writing edges_out. Host pointers. */
int visacd_compute_intersection_matrix(visacd_ctx* ctx, const float* verts, int32_t nv,
                                       const uint32_t* tris, int32_t nt, const uint8_t* is_new,
                                       const float* cage_verts, int32_t ncv,
                                       const uint32_t* cage_tris, int32_t nct,
                                       uint32_t* edges_out, int64_t capacity_edges,
                                       int64_t* n_edges, visacd_vis_stats* stats);

/* ---- plane scoring ------------------------------------------------------ */
/* score[p] = sum over edges e = (i, j) of |p_j - p_i| where the endpoints lie
   strictly on opposite sides of plane p: side(x) = +1 if a x + b y + c z + d >
   1e-6f, -1 if < -1e-6f, else 0 (lib/cuda/plane_intersections.cu:44-57). The
   side test is exact with respect to FP64 evaluation of the FP32 inputs
   (FP32 fast path, FP64 re-decision inside the rounding band). Edge lengths
   are FP32 (IEEE ops, no contraction) quantized to 2^quantum_exp and summed in
   integers, so scores are deterministic and independent of launch shape.
   planes P x 4, points N x 3 float32, edges E x 2 uint32; edges with an index
   >= N are skipped as in the reference. scores is P float64. If device_ptrs
   is 1 the call is asynchronous unless stats != NULL. An asynchronous call
   cannot rerun or raise: if its FP64 re-decision queue fills up, or a
   bulk-copy wait in the kernel times out, every score it writes is NaN. With
   stats != NULL (or host pointers) the library reruns a full queue with room
   for every block and returns VISACD_ERR_DEVICE on a timeout. */
int visacd_score_planes(visacd_ctx* ctx, const float* planes, int32_t P, const float* points,
                        int32_t N, const uint32_t* edges, int64_t E, int device_ptrs,
                        double* scores, visacd_score_stats* stats);
/* Planes per scoring thread (1, 2, 4 or 8; the scores do not depend on it):
   visacd_ctx_set_score_k forces one (0: the autotuned choice of the call's
   shape class if one was measured, else a rule on P). visacd_autotune_scoring
   times each on this exact call (twice, CUDA events on the context stream),
   caches the fastest for the call's shape class (log2 buckets of P and E) in
   the context and reports it; ms_per_k (optional) gets 4 entries. Resets the
   context's kernel timers. */
int visacd_ctx_set_score_k(visacd_ctx* ctx, int k);
int visacd_autotune_scoring(visacd_ctx* ctx, const float* planes, int32_t P, const float* points,
                            int32_t N, const uint32_t* edges, int64_t E, int device_ptrs, int* best_k,
                            double* ms_per_k);

/* ---- candidate planes and the split search -------------------------------- */
/* Candidate split planes from drawn visibility edges. Replaces the plane
   construction and near-duplicate filter of get_candidate_planes
   (lib/src/process.cpp:28-72); the draws themselves stay with the caller's
   random engine. draws[k] is the edge index of draw k (the reference's
   uniform_int_distribution(0, E - 1) outputs, in order; pass the most the
   reference could use, 5 num_planes). For each draw, in order, the plane with
   unit normal n = unit(p2 - p1) and d = -n . midpoint (FP64, the reference's
   operation order) is kept unless |p2 - p1| < 1e-6 or a kept plane has
   |n . n'| > cos 5 deg and |d - d'| < 1e-3; drawing stops once num_planes are
   kept. verts n x 3 float64, edges E x 2 uint32, host pointers. planes_out:
   num_planes x 4 float64 (a, b, c, d); *n_planes gets the count kept and
   *draws_used how many draws the reference's loop consumed (advance the
   engine by exactly those draws). Bit-identical to the reference. */
int visacd_candidate_planes(visacd_ctx* ctx, const double* verts, int32_t n, const uint32_t* edges,
                            int64_t E, const int32_t* draws, int32_t n_draws, int32_t num_planes,
                            double* planes_out, int32_t* n_planes, int32_t* draws_used);

typedef struct visacd_split_info {
  int32_t best_index;    /* in [candidates..., flat planes...]; -1 when nothing was scored */
  int32_t n_candidates;  /* candidate planes kept */
  int32_t draws_used;    /* draws the reference's candidate loop consumed */
  int32_t pad;
  double best_score;     /* the winning float score (flat planes: times flat_k) */
} visacd_split_info;

/* The split-plane search of one part (lib/src/process.cpp:96-134) in one
   call: the candidate planes of visacd_candidate_planes, then the flat-surface
   planes (n_flat x 4 float64), all scored by visacd_score_planes' kernels
   (FP32 points from the FP64 vertices). As in the reference, the scores are
   compared as float: flat scores are multiplied by flat_k in double and
   rounded to float, and the first maximum in that order wins. best_plane: 4
   float64 (the chosen candidate's FP64 coefficients, or the flat plane's).
   Host pointers, synchronous. */
int visacd_split_search(visacd_ctx* ctx, const double* verts, int32_t n, const uint32_t* edges,
                        int64_t E, const int32_t* draws, int32_t n_draws, int32_t num_planes,
                        const double* flat_planes, int32_t n_flat, double flat_k,
                        double* best_plane, visacd_split_info* info);

/* ---- batched visibility + scoring ----------------------------------------- */
/* A batch of parts of uneven size, each with its points (n x 3 float32, host),
   its own BVH (built from those points), its cage BVH and its candidate planes
   (P x 4 float32, host). visacd_batch_run then computes every part's
   visibility edges (all pairs i < j) and scores every part's planes against
   them in one fixed kernel sequence whose sizes live in device memory; with
   use_graph it is captured once as a CUDA graph and replayed. edge_capacity
   bounds the edges of all parts together (0 = total pairs / 64 + 4096). The
   BVHs must outlive the batch. Results equal per-part visacd_visibility +
   visacd_score_planes. Not thread-safe; one run at a time per batch. */
int visacd_batch_create(visacd_ctx* ctx, int32_t n_parts, const float* const* pts,
                        const int32_t* n_pts, const visacd_bvh* const* self_bvhs,
                        const visacd_bvh* const* cage_bvhs, const float* const* planes,
                        const int32_t* n_planes, int64_t edge_capacity, visacd_batch** out);
/* Enqueue one run on the context stream (asynchronous). */
int visacd_batch_run(visacd_ctx* ctx, visacd_batch* b, int use_graph);
/* Wait for the run and copy results: per-part edge counts, all scores
   (float64, parts concatenated in order), per-part first argmax, and
   optionally all edges (parts concatenated, part-local vertex ids). */
int visacd_batch_results(visacd_ctx* ctx, visacd_batch* b, int64_t* n_edges, double* scores,
                         int32_t* argmax, uint32_t* edges, int64_t edge_capacity);
int visacd_batch_info(const visacd_batch* b, int64_t* total_pairs, int64_t* total_planes);
int visacd_batch_destroy(visacd_batch* b);

/* ---- per-part clipping --------------------------------------------------- */
/* Split a mesh (float64 vertices nv x 3, int32 triangles nt x 3) by the plane
   a x + b y + c z + d = 0 (plane = {a, b, c, d}), as lib/src/clip.cpp:190-741
   does before its cap triangulation: 1e-6 side test, triangles wholly on one
   side kept, touching triangles split at the plane, border points deduplicated
   by vertex key, edge key and position (1e-4, first match). Output triangles
   index part-local vertices: the kept original vertices in input order, then
   the border points. Host pointers; results stay on the device until
   visacd_clip_fetch. The caller triangulates the cap from the border points
   and edges. Synchronizes. */
int visacd_clip(visacd_ctx* ctx, const double* verts, int32_t nv, const int32_t* tris, int32_t nt,
                const double* plane, visacd_clip_result* res);
/* Copy the last clip result to host memory (any pointer may be NULL):
   triangles 3 x n_pos / 3 x n_neg, 1-based vertex maps nv each (0 = absent),
   border points 3 x n_border, border edges 2 x n_border_edges. */
int visacd_clip_fetch(visacd_ctx* ctx, int32_t* pos_tris, int32_t* neg_tris, int32_t* pos_map,
                      int32_t* neg_map, double* border, int32_t* border_edges);

/* ---- concavity metric ---------------------------------------------------- */
/* Sampled symmetric face Hausdorff distance between surfaces A and B
   (lib/include/hausdorff.hpp:214-298): for every sample of one surface, the
   smallest FP64 distance to the triangles its 10 nearest samples on the other
   surface were drawn from (the nearest-sample distance if that exceeds 10);
   *out = the largest over both directions. Meshes: float64 vertices, int32
   triangles; samples: float64 xyz with the id of the triangle each was drawn
   from. Host pointers; synchronizes. */
int visacd_face_hausdorff(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                          int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                          const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                          const double* xb, const int32_t* idb, int32_t nb, double* out);

/* visacd_face_hausdorff for a caller that only needs values at or above
   `floor` (the largest of several concavities, lib/src/process.cpp:208-236):
   *out is the exact distance when that is >= floor, and otherwise some value
   strictly below floor. Sample terms whose upper bound lies below floor are
   not evaluated. floor <= 0 gives the exact distance. */
int visacd_face_hausdorff_floor(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                                int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                                const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                                const double* xb, const int32_t* idb, int32_t nb, double floor,
                                double* out);

/* Many face Hausdorff distances in one call: job j compares surface A_j (mesh
   2j, samples of set 2j) with surface B_j (mesh 2j + 1, set 2j + 1). Meshes
   are concatenated: vertices 3 x vert_off[2J] float64, triangles 3 x
   tri_off[2J] int32 with indices local to their mesh; samples 3 x
   sample_off[2J] float64 with the (local) triangle each was drawn from.
   Offsets have 2J + 1 entries starting at 0; every surface and sample set
   must be non-empty.
   independent != 0: out[j] is every job's exact distance H_j.
   independent == 0 (the part selection of lib/src/process.cpp:208-236): with
   lower[j] a known lower bound of job j's concavity (NULL: 0) and
   M = max(floor, max_j max(lower[j], H_j)), out[j] = H_j for every job with
   H_j = M and out[j] <= H_j otherwise, so max(lower[j], out[j]) is exact for
   the jobs that attain M and below M for the rest. Sample terms that cannot
   reach the running maximum are not evaluated. Host pointers; synchronizes. */
int visacd_face_hausdorff_batch(visacd_ctx* ctx, int32_t njobs, const double* verts,
                                const int64_t* vert_off, const int32_t* tris, const int64_t* tri_off,
                                const double* samples, const int32_t* sample_tri,
                                const int64_t* sample_off, const double* lower, double floor,
                                int32_t independent, double* out);

/* Independent segment-triangle decisions with the visibility kernel's test
   (FP32 filter with a rigorous rounding bound, FP64 re-decision inside it;
   lib/ptx/ray_segments.cu:49-111 semantics, tmin 0.001): seg S x 6 (p, q),
   tri S x 9 (a, b, c) float32, host. hit_out[k] = 1 when segment k meets
   triangle k over t in [0.001 / |q - p|, 1]; *n_fp64 = tests decided in FP64.
   Synchronizes. */
int visacd_segment_triangle_tests(visacd_ctx* ctx, const float* seg, const float* tri, int64_t S,
                                  uint8_t* hit_out, int64_t* n_fp64);

/* ---- SDF remeshing (cages) ------------------------------------------------ */
/* The iso-surface at distance `level` outside the mesh on a grid of voxel size
   1/scale: the manifold / cage step of lib/src/preprocess.cpp:18-67 (OpenVDB
   meshToSignedDistanceField + volumeToMesh there). Narrow-band exact distance,
   inside/outside by the majority of x/y/z ray-crossing parities, surface-nets
   vertices and quads split in two triangles; the same mesh, bit for bit, as
   this project's host restatement. verts nv x 3 float64, tris nt x 3 int32
   (host). Writes the output sizes; the mesh stays on the device until
   visacd_sdf_fetch. Synchronizes. */
int visacd_sdf_remesh(visacd_ctx* ctx, const double* verts, int32_t nv, const int32_t* tris,
                      int32_t nt, double scale, double level, int32_t* out_nv, int32_t* out_nt);
/* Copies the last remesh result: verts out_nv x 3 float64, tris out_nt x 3 int32. */
int visacd_sdf_fetch(visacd_ctx* ctx, double* verts, int32_t* tris);

/* ---- convex hulls ---------------------------------------------------------- */
/* Convex hulls of many point sets in one launch: Mesh::compute_ch
   (lib/src/core.cpp:59-111) for every part of a batch, this project's
   QuickHull standing in for qhull "Qt Pp". Part k owns the points
   [offsets[k], offsets[k+1]) of points (float64 xyz, host, finite, at most
   2^22 a part). Its hull triangles (indices into its own points, every input
   point stays a vertex as with qhull) go to tris + 6 * offsets[k] (host; tris
   holds 6 * offsets[nparts] int32, room for 2 triangles a point) and their
   number to counts[k]; with fix_normals every triangle faces away from the
   point centroid (lib/src/core.cpp:33-57). The triangles, and their order,
   equal the host QuickHull's; coplanar input gives the two-sided fan of its 2D
   hull, and fewer than 3 points or collinear input no triangle. One warp per
   part; a part that outgrows its working room (a multiple of its point count)
   runs again with four times the room. Synchronizes. */
int visacd_convex_hulls(visacd_ctx* ctx, const double* points, const int64_t* offsets, int32_t nparts,
                        int32_t fix_normals, int32_t* tris, int32_t* counts);

/* ---- hull merging ---------------------------------------------------------- */
/* Exact minimum vertex-to-vertex distance between pairs of hulls: the
   mesh_dist gate of multimerge_ch (lib/src/postprocess.cpp:64-200,
   lib/src/cost.cpp:125-159). Hull h owns vertices [offsets[h], offsets[h+1])
   of verts (float64 xyz, host); pairs is P x 2 hull indices; out[k] (host, P)
   = the distance of pair k, equal bit for bit to the host's nearest-neighbour
   result, or DBL_MAX when a hull is empty or the pair's bounding boxes are
   farther apart than cutoff (pass DBL_MAX to compute every pair).
   Synchronizes. */
int visacd_hull_distances(visacd_ctx* ctx, const double* verts, const int64_t* offsets, int32_t H,
                          const int32_t* pairs, int64_t P, double cutoff, double* out);

/* ---- learned plane proposer ---------------------------------------------- */
/* No counterpart in the reference: a small network that proposes split planes
   in place of the random candidate draw of lib/src/process.cpp:28-72, whose
   proposals the exact scoring above still ranks. Per part, 2048 visibility
   edges are sampled (edge floor(s*E/2048), or s mod E when E < 2048) and
   described by 7 features in the part's frame x' = (x - center) / scale:
   midpoint, unit direction with its largest component positive, length.
   Network: 7 (padded to 16) -> 64 -> 128 -> 256 shared per-edge layers (ReLU),
   max over the edges, 256 -> 128 -> 64 (ReLU) -> 64 = 16 planes (normal xyz,
   offset). BF16 tensor-core operands, FP32 accumulation, FP32 master weights.
   Parameters are laid out layer by layer, each as W (out x in, row-major)
   followed by b (out): 87,744 floats. */
#define VISACD_LP_POINTS 2048
#define VISACD_LP_FEATURES 7
#define VISACD_LP_PLANES 16
typedef struct visacd_lp visacd_lp;

int visacd_lp_param_count(void);
/* params: 87,744 floats, or NULL for a seeded He-uniform initialisation. The
   proposer runs on ctx's stream. Destroying ctx first releases the proposer's
   device memory: later calls on it fail and visacd_lp_destroy only frees its
   host side. */
int visacd_lp_create(visacd_ctx* ctx, const float* params, uint32_t seed, visacd_lp** out);
int visacd_lp_destroy(visacd_lp* lp);
int visacd_lp_get_params(visacd_lp* lp, float* out);
/* Features of one part (points n x 3 float32, edges E x 2 uint32, host) into
   feats_out (2048 x 7 float32, host). */
int visacd_lp_features(visacd_lp* lp, const float* points, int32_t n, const uint32_t* edges,
                       int64_t E, const float* center, float scale, float* feats_out);
/* Planes for B parts from their features (B x 2048 x 7): planes_out B x 16 x 4
   float32 (unit normal, offset) in each part's normalised frame. */
int visacd_lp_forward(visacd_lp* lp, const float* feats, int32_t B, float* planes_out);
/* Features + forward for one part; planes_out 16 x 4 float64 in the input frame. */
int visacd_lp_propose(visacd_lp* lp, const float* points, int32_t n, const uint32_t* edges,
                      int64_t E, const float* center, float scale, double* planes_out);
/* Loss and gradients for B parts with L label planes each (labels B x L x 4
   float32 in the normalised frame, weights B x L; weight 0 = unused slot).
   Loss per part: sum_l w_l min_q D(q,l) / sum_l w_l + 0.1/16 sum_q min_l D(q,l)
   with D = min over the normal's sign of |n_q - n_l|^2 + (d_q - d_l)^2; the
   batch loss is the mean. grads_out: 87,744 floats or NULL. */
int visacd_lp_grads(visacd_lp* lp, const float* feats, const float* labels, const float* lw,
                    int32_t B, int32_t L, float* grads_out, float* loss_out);
/* Forward per-edge layers on the Blackwell tensor-core path (tcgen05.mma with
   the accumulator in tensor memory, the default) or on mma.sync (enable = 0). */
int visacd_lp_set_tcgen05(visacd_lp* lp, int enable);
/* visacd_lp_grads followed by one Adam step (beta 0.9 / 0.999, eps 1e-8). */
int visacd_lp_train_step(visacd_lp* lp, const float* feats, const float* labels, const float* lw,
                         int32_t B, int32_t L, float lr, float* loss_out);

/* The learned split search of one part in one call, in place of the candidate
   draw and scoring of lib/src/process.cpp:96-134 when the proposer is on:
    1. the proposer's 16 planes, as visacd_lp_propose (center, scale);
    2. refinement: per proposal, the refine_k (0..32) perpendicular-bisector
       planes of visibility edges (the reference's candidate form,
       lib/src/process.cpp:45-53; edges shorter than 1e-6 have none) nearest
       under D = 2 - 2|n_q . n_e| + ((s d_q - d_e) / half)^2 with
       s = sign(n_q . n_e), ties by edge index; their union in edge order;
    3. a probe: the candidates visacd_candidate_planes keeps from probe_draws
       with num_planes = probe_planes;
    4. the exact scores (visacd_score_planes) of [proposals, refined, probe,
       flat planes], the flat scores times flat_k;
    5. the decision: info->fallback = 1 when the best proposal or refined score
       is below (1 - tolerance) x the best probe score (0 without probe
       planes): the caller then runs the full search (visacd_split_search)
       with the draws after info->draws_used. best_plane and best_index are
       the first maximum of all scores in the order of step 4 either way.
   Planes and scores are FP64 and equal, bit for bit, to those of the separate
   calls. verts n x 3 float64, edges E x 2 uint32 (E > 0), probe_draws and
   flat_planes (n_flat x 4 float64) are host arrays. Synchronizes twice. */
typedef struct {
  int32_t best_index;  /* in step 4's order: [0,16) proposals, then refined, probe, flat */
  int32_t n_refined;
  int32_t n_probe;     /* probe candidates kept */
  int32_t draws_used;  /* probe draws consumed */
  int32_t fallback;
  int32_t reserved;
  double best_score;
  double best_proposal_score; /* over the proposals and the refined planes */
  double best_probe_score;    /* 0 without probe planes */
} visacd_learned_split_info;
int visacd_learned_split_search(visacd_lp* lp, const double* verts, int32_t n, const uint32_t* edges,
                                int64_t E, const float* center, float scale, double half,
                                int32_t refine_k, const int32_t* probe_draws, int32_t n_probe_draws,
                                int32_t probe_planes, const double* flat_planes, int32_t n_flat,
                                double flat_k, double tolerance, double* best_plane,
                                visacd_learned_split_info* info);

/* Allocation-free variant of visacd_score_planes. No counterpart in the
   reference: it exists for callers that cannot allocate — code running under a
   fixed, pre-reserved memory budget, or a latency-bound loop where cudaMalloc's
   implicit synchronisation is not acceptable. It calls no cudaMalloc/cudaFree
   or other allocating routine: all scratch lives in one static device array
   of 10,518,784 bytes that every GPU loading the library reserves until exit.
   Inputs (planes P x 4, points N x 3, edges E x 2) and outputs (scores P
   float64, argmax one int32 or NULL) are device pointers; the call is
   asynchronous on cuda_stream (NULL = the legacy default stream). Limits:
   P <= 4096 and E <= 65536, larger sizes return VISACD_ERR_CAPACITY. The first
   call on a device looks up the array's device address (do it before any
   stream capture); the address is cached per device for the life of the
   process, so do not use this call across cudaDeviceReset. Calls share the
   array: calls that overlap on the GPU race, so serialise them. The queue
   holds every (plane, edge block) pair and cannot fill up; if a bulk-copy
   wait inside the kernel times out, every score is NaN and argmax is -2 (the
   call itself returns before the GPU runs, so the failure is reported in the
   outputs). Otherwise results equal visacd_score_planes bit for bit. */
int visacd_score_planes_noalloc(const float* planes, int32_t P, const float* points, int32_t N,
                                const uint32_t* edges, int64_t E, double* scores,
                                int32_t* argmax, void* cuda_stream);

/* Drop-in for the reference's host wrapper: same signature and meaning
   (host pointers, synchronous, float scores), run on a process-wide default
   context on device 0. Errors are recorded in visacd_last_error() and leave
   scores at zero, as the reference does on a launch error. */
void classify_and_rate_planes(const float* planes, const float* points,
                              const unsigned int* edges, float* scores, int numPlanes,
                              int numPoints, int numEdges);

#ifdef __cplusplus
}
#endif
#endif /* VISACD_GPU_H */
