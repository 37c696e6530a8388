/*
 * gsq.h -- C ABI of the GB300-native spatial-query library (libgsq.so).
 *
 * Drop-in boundary for LLNL/axom's spatial-query hot path:
 *   - spin::BVH<3, Exec, double>           (src/axom/spin/BVH.hpp:129-568)
 *   - quest::SignedDistance<3, Exec>       (src/axom/quest/SignedDistance.hpp:147-605)
 *   - the quest C API / shroud wrappers     (src/axom/quest/interface/signed_distance.hpp:88-319,
 *                                            src/axom/quest/interface/c_fortran/wrapQUEST.h:84-129;
 *                                            their QUEST_signed_distance_* entry points themselves
 *                                            are declared in gsq_quest.h)
 *
 * Conventions
 *   - Every function returns an int status: GSQ_OK (0) on success, a negative
 *     GSQ_ERR_* code otherwise; gsq_last_error() describes the last failure of
 *     the calling thread.  Nothing aborts (the reference's SLIC_ERROR does).
 *   - Coordinates are IEEE double.  Indices and counts are int32, as axom's
 *     default IndexType (src/cmake/AxomOptions.cmake:25).
 *   - Array arguments may live in host memory or in device memory of the
 *     current CUDA device; each pointer is classified on entry.  Host inputs
 *     are staged to the device and device results copied back to host outputs.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  Calls are synchronous with respect to that stream, like the
 *     reference's SYNCHRONOUS execution policies: outputs are complete when the
 *     call returns.
 *   - Boxes are 6 doubles {xmin, ymin, zmin, xmax, ymax, zmax}, the memory
 *     layout of primal::BoundingBox<double,3> (BoundingBox.hpp:363-367), so an
 *     array of reference boxes can be passed as is.  Points are 3 doubles, the
 *     layout of primal::Point<double,3>.
 *   - Device work runs on the CUDA device that is current when the handle is
 *     created; a handle must be used with that device current.
 *   - Like the reference's const BVH::find* and SignedDistance::
 *     computeDistances, gsq_bvh_find_* and gsq_sdf_eval may run concurrently
 *     on one handle from several host threads (each on its own stream): a
 *     call that finds the handle's scratch in use allocates its own.  Builds,
 *     option changes and destruction must not overlap other calls on the
 *     handle.
 */
#ifndef GSQ_H_
#define GSQ_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GSQ_OK 0
#define GSQ_ERR_INVALID -1  /* bad argument; also BVH_BUILD_FAILED (spin/BVH.hpp:39-43) */
#define GSQ_ERR_CUDA -2     /* a CUDA runtime call failed */
#define GSQ_ERR_NOMEM -3    /* device or host allocation failed */
#define GSQ_ERR_DEVICE -4   /* a kernel reported an error (stack overflow, bounded wait expired) */
#define GSQ_ERR_STATE -5    /* call out of order (e.g. query before build) */

/* Precision forms of the signed-distance query. */
#define GSQ_PRECISION_FP64 0  /* op-for-op FP64 restatement of the reference */
#define GSQ_PRECISION_MIXED 1 /* FP32 outward-rounded traversal, FP64 refine and sign */

typedef struct gsq_bvh gsq_bvh;
typedef struct gsq_sdf gsq_sdf;

/* Message of the last failed call on this thread ("" if none). */
const char* gsq_last_error(void);

/* Self-test of the kernels' bounded waits (no reference counterpart): runs
 * one block of the radix sort's onesweep pass on the second tile of a
 * two-tile input while the first tile is never processed, so that its
 * decoupled look-back waits for a flag nothing sets.  The wait gives up after
 * its poll limit (about a second), the kernel finishes without writing
 * outside its buffers, and the call returns GSQ_ERR_DEVICE with "expired
 * bounded wait" in gsq_last_error(); the CUDA context stays usable. */
int gsq_selftest_bounded_wait(void* stream);

/* Library version string. */
const char* gsq_version(void);

/* Number of CUDA kernels this library has launched in this process (for
 * launch accounting in benchmarks).  No reference counterpart. */
int64_t gsq_kernel_launches(void);

/* Frees a candidate array returned by a gsq_bvh_find_* call, wherever it lives. */
int gsq_free(void* ptr);

/* Copies bytes between any two host or device pointers (cudaMemcpyDefault),
 * e.g. a device candidate array into a caller buffer.  No reference
 * counterpart: axom::copy (core/memory_management.hpp) plays this role there. */
int gsq_memcpy(void* dst, const void* src, size_t bytes);

/* ---- spin::BVH -------------------------------------------------------- */

/* Replaces spin::BVH::BVH() (spin/BVH.hpp:185); default scale factor
 * 1.000123 and tolerance DBL_EPSILON (spin/BVH.hpp:410-412). */
int gsq_bvh_create(gsq_bvh** out);
int gsq_bvh_destroy(gsq_bvh* bvh);

/* Replaces BVH::setScaleFactor / getScaleFactor (spin/BVH.hpp:269-275). */
int gsq_bvh_set_scale_factor(gsq_bvh* bvh, double scale);
int gsq_bvh_get_scale_factor(const gsq_bvh* bvh, double* scale);
/* Replaces BVH::setTolerance / getTolerance (spin/BVH.hpp:283-289); the
 * tolerance is the ray test's near-zero direction threshold. */
int gsq_bvh_set_tolerance(gsq_bvh* bvh, double tol);
int gsq_bvh_get_tolerance(const gsq_bvh* bvh, double* tol);

/* Replaces BVH::initialize(boxes, numItems) (spin/BVH.hpp:424-477):
 * Morton codes, stable radix sort, Karras hierarchy, bottom-up refit.
 * boxes: n x 6 doubles.  n may be 0 or 1 (padded as the reference does). */
int gsq_bvh_build(gsq_bvh* bvh, const double* boxes, int32_t n, void* stream);

/* Replaces BVH::getBounds (spin/BVH.hpp:297-309): global bounds of the
 * scaled input boxes.  lo/hi are host arrays of 3. */
int gsq_bvh_bounds(const gsq_bvh* bvh, double* lo, double* hi);

/* Number of leaves stored (after padding of 0/1 boxes to 2). */
int gsq_bvh_num_leaves(const gsq_bvh* bvh, int32_t* n);

/* Candidate queries.  Replace BVH::findBoundingBoxes / findPoints / findRays
 * (spin/BVH.hpp:480-568, policy/LinearBVH.hpp:271-402).
 *   offsets, counts : m int32 each, caller-owned (host or device).
 *   *candidates     : allocated by the library in the memory space of
 *                     `offsets` (free with gsq_free); query i's candidate ids
 *                     are candidates[offsets[i] .. offsets[i]+counts[i]).
 *   total           : host int64, the number of candidates (nullable).
 * Candidate order within a query is the reference traversal order. */
int gsq_bvh_find_boxes(const gsq_bvh* bvh, const double* query_boxes, int32_t m, int32_t* offsets,
                       int32_t* counts, int32_t** candidates, int64_t* total, void* stream);
/* points: m x 3 doubles. */
int gsq_bvh_find_points(const gsq_bvh* bvh, const double* points, int32_t m, int32_t* offsets,
                        int32_t* counts, int32_t** candidates, int64_t* total, void* stream);
/* origins, directions: m x 3 doubles.  Directions are the rays' stored unit
 * directions, as primal::Ray keeps them (primal/geometry/Ray.hpp:123-128);
 * gsq_ray_normalize gives the same normalisation for raw directions. */
int gsq_bvh_find_rays(const gsq_bvh* bvh, const double* origins, const double* directions, int32_t m,
                      int32_t* offsets, int32_t* counts, int32_t** candidates, int64_t* total, void* stream);

/* Host helper: primal::Vector::unitVector (primal/geometry/Vector.hpp:477-493)
 * applied to m raw directions (host arrays, m x 3). */
int gsq_ray_normalize(const double* raw, int32_t m, double* unit);

/* Debug export of the built hierarchy in the reference's LinearBVH layout
 * (policy/LinearBVH.hpp:170-188, 225-266), to host arrays (each nullable):
 *   node_boxes   2(n-1) x 6 : child boxes of inner node i at rows 2i, 2i+1
 *   children     2(n-1)     : 2*c for inner child c, -(leafpos+1) for a leaf
 *   leaf_ids     n          : original box id of each sorted leaf position
 *   codes        n          : sorted Morton codes (build_radix_tree.hpp:146-260)
 * where n = gsq_bvh_num_leaves. */
int gsq_bvh_export(const gsq_bvh* bvh, double* node_boxes, int32_t* children, int32_t* leaf_ids,
                   uint32_t* codes);

/* Replaces BVH::getTraverser (spin/BVH.hpp:319): device pointers to the built
 * tree for user kernels, traversed with gsq::device::traverse_tree
 * (include/gsq_device.cuh).  Valid until the next build or destroy.
 *   nodes      num_leaves - 1 node records of 128 bytes (gsq::device::Node)
 *   leaf_ids   num_leaves original box ids, by sorted leaf position */
typedef struct gsq_bvh_view {
  const void* nodes;
  const int32_t* leaf_ids;
  int32_t num_leaves;
  int32_t reserved;
} gsq_bvh_view;
int gsq_bvh_get_view(const gsq_bvh* bvh, gsq_bvh_view* view);

/* Milliseconds of device time taken by the last gsq_bvh_build on this
 * handle (CUDA events around the build's kernels). */
int gsq_bvh_last_build_ms(const gsq_bvh* bvh, float* ms);

/* Milliseconds of device time taken by the last find on this handle: its two
 * traversal passes and the offsets scan (CUDA events on the call's stream;
 * the host wait for the candidate count between them is not included). */
int gsq_bvh_last_find_ms(const gsq_bvh* bvh, float* ms);

/* ---- quest::SignedDistance --------------------------------------------- */

typedef struct gsq_sdf_opts {
  int32_t precision;      /* GSQ_PRECISION_FP64 (default) or GSQ_PRECISION_MIXED */
  int32_t sort_queries;   /* 1: process queries in Morton order (default 1) */
  int32_t block_size;     /* threads per block of the query kernel (0 = default) */
  int32_t audit;          /* MIXED only: 1 re-checks every FP32 skip in FP64 and counts
                             violations and FP64 fallbacks (gsq_sdf_mixed_stats); slow */
  int32_t queue_depth;    /* MIXED only: FP64 refinements a lane queues before they run
                             (1, 4 or 16; 0 = default 4) */
  int32_t reserved[3];
} gsq_sdf_opts;

/* Fills opts with the defaults. */
int gsq_sdf_opts_init(gsq_sdf_opts* opts);

/* Replaces SignedDistance(const mint::Mesh*, isWatertight, computeSign)
 * and setMesh (quest/SignedDistance.hpp:410-504): mesh box, per-cell boxes
 * and the BVH build.  The mesh is an unstructured single-shape surface mesh:
 *   x, y, z         : nverts node coordinates
 *   cells           : ncells x nodes_per_cell node ids (int32), ncells < 2^28
 *   nodes_per_cell  : 3 (triangles) or 4 (quads, split as the reference does)
 * The handle keeps its own device copy of the mesh (the reference borrows
 * the mint mesh).  opts nullable. */
int gsq_sdf_create(gsq_sdf** out, const double* x, const double* y, const double* z, int32_t nverts,
                   const int32_t* cells, int32_t ncells, int32_t nodes_per_cell, int32_t watertight,
                   int32_t compute_sign, const gsq_sdf_opts* opts, void* stream);
int gsq_sdf_destroy(gsq_sdf* sdf);

/* Changes the options of an existing handle (precision, query order, ...). */
int gsq_sdf_set_opts(gsq_sdf* sdf, const gsq_sdf_opts* opts);

/* Replaces SignedDistance::computeDistances(npts, queryPts, outSgnDist,
 * outClosestPts, outNormals) (quest/SignedDistance.hpp:527-605) and the C
 * API's signed_distance_evaluate (quest/interface/signed_distance.hpp:290,
 * quest/interface/signed_distance.cpp:432-465).
 *   qx, qy, qz : query coordinates; element i is q*[i * stride]
 *                (stride 1 = three SoA arrays, as ZipPoint / the C API;
 *                 stride 3 with qy = qx+1, qz = qx+2 = an array of points)
 *   out        : m signed distances
 *   closest    : m x 3 closest points (nullable)
 *   normals    : m x 3 unit pseudo-normals (nullable) */
int gsq_sdf_eval(const gsq_sdf* sdf, const double* qx, const double* qy, const double* qz, int32_t stride,
                 int32_t m, double* out, double* closest, double* normals, void* stream);

/* Allocation-free evaluation, for callers that must not allocate device
 * memory while evaluating: applications whose own pool allocator owns all
 * device memory, and loops beside other streams that must not be stalled by
 * the implicit device-wide synchronisation of cudaMalloc/cudaFree.  No
 * counterpart in the reference.
 *   - qx, qy, qz (with `stride`, as gsq_sdf_eval) and out (m doubles) must be
 *     device memory; no closest points or normals.
 *   - Runs on the handle's device, which must be the current device
 *     (else GSQ_ERR_INVALID).  Returns after its stream has finished (it
 *     reads the device error flag), as gsq_sdf_eval does.
 *   - m <= GSQ_NOALLOC_MAX_QUERIES, else GSQ_ERR_INVALID and nothing runs.
 *   - Calls no cudaMalloc/cudaFree or allocating library routine.  Its only
 *     scratch (the Morton-order sort of the points and the query kernel's
 *     work counter) is one fixed array of about 4.3 MB in the library's
 *     device image, which every GPU that loads the library holds until the
 *     process exits.
 *   - The first call on each device looks the array's device address up once
 *     (cudaGetSymbolAddress) and keeps it; make that first call before any
 *     stream capture.  A cudaDeviceReset after it is not supported (it also
 *     invalidates every handle).
 *   - Every call shares that one array: calls of this entry point whose GPU
 *     work overlaps (other streams or host threads, on the same device) race
 *     and corrupt each other's results.  Serialise them.  (A gsq_sdf_eval
 *     running at the same time does not use the array.)
 *   - The precision and query-order options of the handle apply; outputs equal
 *     gsq_sdf_eval's. */
#define GSQ_NOALLOC_MAX_QUERIES 262144
int gsq_sdf_eval_noalloc(const gsq_sdf* sdf, const double* qx, const double* qy, const double* qz, int32_t stride,
                         int32_t m, double* out, void* stream);

/* Replaces signed_distance_get_mesh_bounds (quest/interface/signed_distance.hpp:308):
 * bounding box of the mesh nodes (host lo[3], hi[3]). */
int gsq_sdf_mesh_bounds(const gsq_sdf* sdf, double* lo, double* hi);

/* The BVH built over the mesh cells (SignedDistance::getBVHTree,
 * quest/SignedDistance.hpp:337).  Owned by the sdf handle. */
int gsq_sdf_get_bvh(const gsq_sdf* sdf, const gsq_bvh** bvh);

/* Milliseconds of device time of the last gsq_sdf_eval's query kernel. */
int gsq_sdf_last_eval_ms(const gsq_sdf* sdf, float* ms);

/* Adjoint of gsq_sdf_eval for a loss L(d): given grad_dist = dL/dd (m), returns
 *   grad_points   m x 3      dL/dq = dL/dd * s * (q - cp) / |q - cp|     (nullable)
 *   grad_vertices nverts x 3 dL/dV_k = sum over points of -dL/dd * s * b_k * (q - cp)/|q - cp|
 *                            where b are the barycentric weights of cp on its
 *                            closest triangle (nullable)
 * s is the point's sign; at |q - cp| = 0 the contribution is 0.  The vertex
 * sum is reduced deterministically (stable sort by vertex id, segment sums in
 * point order), so repeated calls agree bit for bit.  The closest triangles
 * are those of the forward pass (same traversal).  No counterpart in the
 * reference, which has no gradient. */
int gsq_sdf_backward(const gsq_sdf* sdf, const double* qx, const double* qy, const double* qz, int32_t stride,
                     int32_t m, const double* grad_dist, double* grad_points, double* grad_vertices, void* stream);

/* gsq_sdf_eval of the signed distances (no closest points or normals) that
 * also returns each point's closest triangle, the one whose closest point the
 * distance is measured to: triangles[i] = c for triangle cell c, 2c or 2c+1
 * for the first (nodes 0, 1, 2) or second (nodes 0, 2, 3) triangle of quad
 * cell c, -1 when the mesh has no valid cell.  In MIXED precision the query
 * runs with 128 threads per block, queue depth 4 and no audit whatever the
 * handle's options; distances equal gsq_sdf_eval's.  Saved by a forward pass
 * for gsq_sdf_backward_tri.  No counterpart in the reference. */
int gsq_sdf_eval_tri(const gsq_sdf* sdf, const double* qx, const double* qy, const double* qz, int32_t stride,
                     int32_t m, double* out, int32_t* triangles, void* stream);

/* gsq_sdf_backward given the forward pass's signed distances `dist` and
 * closest triangles (gsq_sdf_eval_tri on the same points): the same outputs,
 * bit for bit, without a second traversal. */
int gsq_sdf_backward_tri(const gsq_sdf* sdf, const double* qx, const double* qy, const double* qz, int32_t stride,
                         int32_t m, const double* dist, const int32_t* triangles, const double* grad_dist,
                         double* grad_points, double* grad_vertices, void* stream);

/* Counters of the last audited MIXED evaluation (opts.audit = 1), host int64[4]:
 *   [0] FP32 skips that the FP64 re-check contradicts (must be 0)
 *   [1] node visits decided in FP64   [2] leaves refined in FP64
 *   [3] leaves skipped on the FP32 certificate.
 * No reference counterpart (the reference has only the FP64 form). */
int gsq_sdf_mixed_stats(const gsq_sdf* sdf, int64_t* counters);

/* ---- Surface-mesh input --------------------------------------------------
 * Replaces quest::STLReader::read + getMesh (quest/readers/STLReader.cpp) as
 * used by signed_distance_init(file) (quest/interface/internal/
 * QuestHelpers.cpp:287-320): reads an ASCII or binary STL file (binary iff the
 * file size is 84 + 50 n for the triangle count n in its header).  Every
 * triangle gets its own three nodes in file order (no merging, as the
 * reference); cell i is (3i, 3i+1, 3i+2).  Host arrays, freed with gsq_free:
 *   xyz    nnodes x 3 coordinates (AoS)
 *   cells  ncells x 3 node ids
 * The mesh feeds gsq_sdf_create with stride-3 coordinate pointers. */
int gsq_stl_read(const char* path, double** xyz, int32_t* nnodes, int32_t** cells, int32_t* ncells);

/* ---- Closest object point ----------------------------------------------
 * Replaces the local step of quest::DistributedClosestPoint
 * (quest/detail/DistributedClosestPointImpl.hpp: generateBVHTreeImpl 883-901,
 * computeLocalClosestPoints 1002-1050): a BVH over the object points (one
 * degenerate box each, default scale factor), then per query point the closest
 * object point within a distance threshold.  MPI exchange and conduit
 * plumbing are not part of it (one GPU, one domain set).
 *   points      n x 3 object points (host or device); domain_ids n ints (nullable = 0)
 *   sq_threshold  squared distance threshold (the reference's
 *               setDistanceThreshold(t) stores t*t; DBL_MAX = none)
 *   idx, dom    m ints: the closest object point and its domain, -1 if none
 *   pos, dist   m x 3 and m doubles: its coordinates and distance, NaN if none
 *   precision   GSQ_PRECISION_FP64 or GSQ_PRECISION_MIXED (FP32-certified node
 *               decisions); both give the same bits.
 * Ties keep the first point the traversal reaches, as the reference does. */
typedef struct gsq_cpq gsq_cpq;
int gsq_cpq_create(gsq_cpq** out, const double* points, int32_t n, const int32_t* domain_ids, void* stream);
int gsq_cpq_destroy(gsq_cpq* cpq);
int gsq_cpq_query(const gsq_cpq* cpq, const double* points, int32_t m, double sq_threshold, int32_t precision,
                  int32_t* idx, int32_t* dom, double* pos, double* dist, void* stream);
/* Milliseconds of device time of the last query kernel. */
int gsq_cpq_last_ms(const gsq_cpq* cpq, float* ms);

/* ---- Batched signed distance -------------------------------------------
 * Many independent surface meshes, each with its own set of query points of
 * any size, evaluated together.  One run rebuilds the BVH of every mesh (a
 * segmented build: each build kernel covers all meshes at once) and then
 * evaluates every point against its own mesh with one persistent launch of
 * the mixed-precision query kernel (FP32 certified traversal, FP64 refine and
 * sign).  The whole sequence is captured once as a CUDA graph and replayed by
 * each run.  Every mesh's distances and closest points equal gsq_sdf_eval on
 * that mesh alone, and hence the reference's SignedDistance, bit for bit.
 * No counterpart in the reference, which handles one mesh per object.
 *
 * Mesh sizes, connectivity and the number of points per mesh are fixed when
 * the batch is created; vertex coordinates and point coordinates may change
 * between runs (each run rebuilds the trees from the current coordinates). */
typedef struct gsq_batch gsq_batch;

typedef struct gsq_batch_opts {
  int32_t block_size;      /* threads per block of the query kernel: 32..128, multiple of 32 (0 = 128) */
  int32_t queue_depth;     /* FP64 refinements a lane queues: 1, 4 or 16 (0 = 4) */
  int32_t stack_depth;     /* traversal stack entries: 32 or 64 (0 = 64, the reference's).  32
                              needs every tree's deepest leaf at depth <= 31; a run that
                              overflows it is repeated with 64 and the option set to 64 */
  int32_t morton_bits;     /* bits of each point's Morton code in the processing order,
                              1..30; with the mesh id they must fit 32 bits
                              (0 = as many as fit) */
  int32_t leaf_size;       /* boxes per BVH leaf.  Only 1, the reference's: larger leaves
                              change which triangles the traversal examines and so can
                              change pseudo-normal sums; 0 = 1 */
  int32_t closest_points;  /* 1: runs also produce closest points (set at creation) */
  int32_t reserved[2];
} gsq_batch_opts;

/* Fills opts with the defaults. */
int gsq_batch_opts_init(gsq_batch_opts* opts);

/* Creates a batch of nmeshes meshes.  Host arrays:
 *   vert_offsets  nmeshes+1 int64: mesh k's vertices are [vert_offsets[k], vert_offsets[k+1])
 *   cell_offsets  nmeshes+1 int64: mesh k's cells likewise; every mesh needs >= 2 cells
 *   cells         cell_offsets[nmeshes] x nodes_per_cell vertex ids, local to the mesh
 *                 (0 = the mesh's first vertex)
 *   query_offsets nmeshes+1 int64: mesh k's points are [query_offsets[k], query_offsets[k+1])
 * Totals: fewer than 2^30 cells and 2^30 points, at most 65536 meshes, fewer
 * than 2^28 cells per mesh.
 * watertight / compute_sign apply to every mesh.  Device buffers for all of it
 * are allocated here, once.  opts nullable. */
int gsq_batch_create(gsq_batch** out, int32_t nmeshes, const int64_t* vert_offsets, const int64_t* cell_offsets,
                     const int32_t* cells, int32_t nodes_per_cell, const int64_t* query_offsets, int32_t watertight,
                     int32_t compute_sign, const gsq_batch_opts* opts, void* stream);
int gsq_batch_destroy(gsq_batch* batch);

/* Vertex coordinates of all meshes (vert_offsets[nmeshes] each; host or device). */
int gsq_batch_set_vertices(gsq_batch* batch, const double* x, const double* y, const double* z, void* stream);

/* Query points of all meshes, query_offsets[nmeshes] x 3 (host or device). */
int gsq_batch_set_points(gsq_batch* batch, const double* points, void* stream);

/* Rebuilds every tree and evaluates every point: one graph launch.
 *   out      query_offsets[nmeshes] signed distances (host or device; null keeps them
 *            in the batch's device buffer, see gsq_batch_device_output)
 *   closest  query_offsets[nmeshes] x 3 closest points (nullable; needs closest_points) */
int gsq_batch_run(gsq_batch* batch, double* out, double* closest, void* stream);

/* Device buffers holding the last run's distances and closest points (null if
 * not produced); valid until the next run or destroy. */
int gsq_batch_device_output(const gsq_batch* batch, const double** dist, const double** closest);

/* Chooses block size, queue depth, stack depth and Morton width by timing the
 * query kernel on a sample of the current points (every candidate in turn),
 * after one build of the current meshes; the next run re-captures its graph.
 * The chosen options are readable with gsq_batch_get_opts. */
int gsq_batch_tune(gsq_batch* batch, void* stream);

int gsq_batch_get_opts(const gsq_batch* batch, gsq_batch_opts* opts);
/* Replaces the options (closest_points stays as created); the next run re-captures. */
int gsq_batch_set_opts(gsq_batch* batch, const gsq_batch_opts* opts);

/* Milliseconds of device time of the last run (the whole graph), and the
 * deepest leaf over all trees as of the last tune (-1 before). */
int gsq_batch_last_ms(const gsq_batch* batch, float* ms);
int gsq_batch_max_depth(const gsq_batch* batch, int32_t* depth);

#ifdef __cplusplus
}
#endif
#endif /* GSQ_H_ */
