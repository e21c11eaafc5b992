/*
 * cuspatial_gb300 — C ABI of the GB300 (sm_103a) quadtree spatial join.
 *
 * Each entry point replaces one libcuspatial column-API function; the comment
 * on each names the reference declaration it stands in for (paths relative to
 * the cuSpatial 25.06 source tree).  Differences from the reference:
 *   - columns are raw device pointers plus element counts; coordinates carry a
 *     dtype code (float32 / float64) where cuDF columns carried a type id;
 *   - offsets are 32-bit unsigned (cuDF INT32 offsets are accepted as-is: the
 *     values are non-negative, so the bits are the same);
 *   - cuspatial::logic_error / cuda_error become status codes, with the
 *     reference's message text available from cspt_last_error_message();
 *   - outputs whose size is only known on the device are allocated through a
 *     caller-supplied allocator (rmm's device_async_resource_ref in the
 *     reference); passing NULL uses the library's own stream-ordered pool
 *     (one per device, created on first use; freed memory stays in it for
 *     later calls until cspt_pool_trim; like the library's other per-device
 *     state it does not survive cudaDeviceReset);
 *   - every call takes an explicit stream (a cudaStream_t passed as void*).
 *     Calls that return a size the host must know (quadtree node count, pair
 *     counts) synchronise that stream once; the others are asynchronous.
 *
 * Thread safety: calls are reentrant; the last-error message is per thread.
 */
#ifndef CUSPATIAL_GB300_H
#define CUSPATIAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CSPT_OK               = 0,
  CSPT_INVALID_ARGUMENT = 1, /* cuspatial::logic_error */
  CSPT_OUT_OF_MEMORY    = 2, /* rmm::out_of_memory */
  CSPT_CUDA_ERROR       = 3, /* cuspatial::cuda_error */
  CSPT_TIMEOUT          = 4, /* a bounded device-side wait gave up */
  CSPT_UNSUPPORTED      = 5  /* non-floating-point coordinates (CUDF_FAIL) */
} cspt_status;

typedef enum { CSPT_FLOAT32 = 0, CSPT_FLOAT64 = 1 } cspt_dtype;

/* Point-in-polygon / nearest-linestring arithmetic.
 *   CSPT_METHOD_EXACT    : every edge test in the input precision, evaluated
 *                          exactly as the reference does (the drop-in).
 *   CSPT_METHOD_FILTERED : float64 inputs are first tested in float32 with a
 *                          forward error bound; only undecided candidates are
 *                          re-evaluated with the float64 reference expression.
 *                          Results are identical to CSPT_METHOD_EXACT.
 */
typedef enum { CSPT_METHOD_EXACT = 0, CSPT_METHOD_FILTERED = 1 } cspt_method;

/* Device allocator.  allocate must return 256-byte aligned device memory or
 * NULL; deallocate receives the same size and stream.  Memory is
 * stream-ordered: a block allocated for `stream` is used only by work on that
 * stream (or by work ordered after it), and once deallocated it may be handed
 * out again only to work ordered after that stream's pending work (a call
 * may allocate for more than one stream). */
typedef struct {
  void* ctx;
  void* (*allocate)(void* ctx, size_t bytes, void* stream);
  void (*deallocate)(void* ctx, void* ptr, size_t bytes, void* stream);
} cspt_allocator;

/* Quadtree columns (cpp/include/cuspatial/point_quadtree.hpp:40-58):
 * key u32, level u8, is_internal_node u8 (0/1), length u32, offset u32. */
typedef struct {
  uint32_t* key;
  uint8_t* level;
  uint8_t* is_internal_node;
  uint32_t* length;
  uint32_t* offset;
  size_t num_nodes;
} cspt_quadtree;

/* Message of the last failed call on this thread ("" if none). */
const char* cspt_last_error_message(void);

/* Library version string. */
const char* cspt_version(void);

/* Number of candidates that the last CSPT_METHOD_FILTERED point-in-polygon
 * call on this thread re-evaluated in float64.  Diagnostic with no
 * counterpart in the reference. */
uint64_t cspt_last_refined_count(void);

/* Number of (polygon, quadrant) pairs that the last CSPT_METHOD_FILTERED
 * float64 point-in-polygon call on this thread decided whole: no edge comes
 * within the filter's margin of the quadrant's points, so one point's
 * result holds for all of them.  Diagnostic with no counterpart in the
 * reference. */
uint64_t cspt_last_edge_free_pairs(void);

/* Paths taken by the last CSPT_METHOD_FILTERED float64 nearest-linestring
 * call on this thread: points whose fold ran over every candidate in
 * float64 (their listed candidates reached a zero distance, or none),
 * groups of pairs sharing a quadrant that were scanned point by point
 * instead of through their leaf's segment list, and listed segments whose
 * distance was evaluated in float64.  Any pointer may be NULL.  Diagnostic
 * with no counterpart in the reference. */
void cspt_last_nearest_stats(uint64_t* points_folded_whole, uint64_t* groups_scanned,
                             uint64_t* float64_segments);

/* Number of kernels this library has launched since load.  Diagnostic with
 * no counterpart in the reference. */
uint64_t cspt_launch_count(void);

/* Event timing of the library's named kernels on their launching streams
 * ("pip_bits", "pip_expand", "join_count", "join_write", "nearest",
 * "quadtree_build").  Enabling (or disabling) clears the totals; reading
 * waits for the recorded events.  Diagnostics with no counterpart in the
 * reference. */
void cspt_profile_enable(int on);
int cspt_profile_read(const char* name, double* total_ms, uint64_t* launches);

/* Releases a buffer returned by this library (same allocator as the call). */
void cspt_free(const cspt_allocator* mr, void* ptr, size_t bytes, void* stream);

/* Returns memory of the library's pool on the current device (used when a
 * call gets no allocator) to the CUDA driver, keeping at most min_bytes_to_keep;
 * synchronises the device first.  No reference counterpart. */
cspt_status cspt_pool_trim(size_t min_bytes_to_keep);

/* Releases the five columns of a quadtree returned by cspt_quadtree_on_points. */
void cspt_quadtree_free(const cspt_allocator* mr, cspt_quadtree* tree, void* stream);

/*
 * Replaces cuspatial::quadtree_on_points
 * (cpp/include/cuspatial/point_quadtree.hpp:68-78; behaviour
 * cpp/src/indexing/point_quadtree.cu:154-180 and
 * cpp/include/cuspatial/detail/point_quadtree.cuh:237-272).
 * Outputs point_indices[num_points] and the quadtree, both allocated with mr.
 * max_depth is clamped to [0, 15], max_size to >= 1 and scale to
 * >= max(dx, dy) / ((1 << max_depth) + 2), as the reference does.
 */
cspt_status cspt_quadtree_on_points(const void* x, const void* y, size_t num_points,
                                    cspt_dtype dtype, double x_min, double x_max, double y_min,
                                    double y_max, double scale, int8_t max_depth,
                                    int32_t max_size, const cspt_allocator* mr, void* stream,
                                    uint32_t** out_point_indices, cspt_quadtree* out_tree);

/*
 * cspt_quadtree_on_points for points in host memory: the points are copied
 * into the caller's device arrays device_x / device_y (num_points elements
 * each, for the calls that follow) in chunks, and the Morton keys of each
 * chunk are computed while the next chunk is copied, so with page-locked host
 * arrays the copy overlaps the key computation.  Outputs as
 * cspt_quadtree_on_points.
 */
cspt_status cspt_quadtree_on_points_host(const void* host_x, const void* host_y,
                                         size_t num_points, cspt_dtype dtype, double x_min,
                                         double x_max, double y_min, double y_max, double scale,
                                         int8_t max_depth, int32_t max_size, void* device_x,
                                         void* device_y, const cspt_allocator* mr, void* stream,
                                         uint32_t** out_point_indices, cspt_quadtree* out_tree);

/*
 * The points in quadtree order: writes out_xy[2 i] = x[point_indices[i]] and
 * out_xy[2 i + 1] = y[point_indices[i]] for i < num_point_indices (out_xy is
 * the caller's device array of 2 * num_point_indices elements of dtype,
 * starting on a 16-byte boundary for float64, 8-byte for float32).  An index
 * at or beyond num_points gives NaN coordinates.  Asynchronous.
 * No counterpart in the reference: its quadtree_point_in_polygon and
 * quadtree_point_to_nearest_linestring read every point through
 * point_indices on every call (an index read and two random reads per
 * point).  A caller that keeps a quadtree for one or more joins pays that
 * gather once here and passes the result to the *_ordered entry points,
 * which then read each leaf's points contiguously.
 */
cspt_status cspt_points_in_quadtree_order(const uint32_t* point_indices,
                                          size_t num_point_indices, const void* x, const void* y,
                                          size_t num_points, cspt_dtype dtype, void* out_xy,
                                          void* stream);

/*
 * cspt_quadtree_on_points and cspt_quadtree_on_points_host that also write
 * the points in quadtree order to out_ordered_xy (what
 * cspt_points_in_quadtree_order writes; the caller's device array of
 * 2 * num_points elements of dtype, 16-byte aligned for float64, 8-byte for
 * float32).  The key pass writes the points interleaved as it reads them,
 * so the gather after the sort reads one vector per point.  Tree and
 * point_indices are those of the calls they stand beside.  No counterpart in
 * the reference (see cspt_points_in_quadtree_order).
 */
cspt_status cspt_quadtree_on_points_ordered(const void* x, const void* y, size_t num_points,
                                            cspt_dtype dtype, double x_min, double x_max,
                                            double y_min, double y_max, double scale,
                                            int8_t max_depth, int32_t max_size,
                                            const cspt_allocator* mr, void* stream,
                                            uint32_t** out_point_indices,
                                            cspt_quadtree* out_tree, void* out_ordered_xy);
cspt_status cspt_quadtree_on_points_host_ordered(
  const void* host_x, const void* host_y, size_t num_points, cspt_dtype dtype, double x_min,
  double x_max, double y_min, double y_max, double scale, int8_t max_depth, int32_t max_size,
  void* device_x, void* device_y, const cspt_allocator* mr, void* stream,
  uint32_t** out_point_indices, cspt_quadtree* out_tree, void* out_ordered_xy);

/*
 * Replaces cuspatial::polygon_bounding_boxes
 * (cpp/include/cuspatial/bounding_boxes.hpp:79-85;
 * cpp/src/bounding_boxes/polygon_bounding_boxes.cu:132-159).
 * poly_offsets[num_poly_offsets] index rings, ring_offsets[num_ring_offsets]
 * index vertices.  Writes num_poly_offsets-1 rows to the caller's four
 * arrays (dtype of x/y).  A polygon without vertices yields no row and later
 * rows move up, as reduce_by_key does in the reference; left-over rows are NaN.
 */
cspt_status cspt_polygon_bounding_boxes(const uint32_t* poly_offsets, size_t num_poly_offsets,
                                        const uint32_t* ring_offsets, size_t num_ring_offsets,
                                        const void* x, const void* y, size_t num_vertices,
                                        cspt_dtype dtype, double expansion_radius,
                                        void* out_min_x, void* out_min_y, void* out_max_x,
                                        void* out_max_y, void* stream);

/*
 * cspt_polygon_bounding_boxes_noalloc: same arguments and results as
 * cspt_polygon_bounding_boxes, but the call allocates no device memory.  It
 * has no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: code that runs while a stream is being captured into a CUDA
 * graph or inside a latency-bound loop (cudaMalloc synchronises the device),
 * and hosts that hand out all device memory themselves.  Its scratch is a
 * fixed file-scope device array of 4 MiB + 2 KiB that every GPU loading the
 * library keeps until exit, so inputs are limited to 1,048,576 polygons;
 * larger inputs are rejected with CSPT_INVALID_ARGUMENT.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current: make that first call before any stream capture.  The
 * address is kept per device ordinal for the life of the process; it does
 * not survive cudaDeviceReset (or another reset of the device's primary
 * context), after which this entry point must not be called again.  All
 * calls on a device share the one array (each call rewrites what it reads),
 * so calls whose work overlaps on the GPU (different streams, no ordering
 * between them) race and must not be issued.
 */
cspt_status cspt_polygon_bounding_boxes_noalloc(
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* x, const void* y, size_t num_vertices, cspt_dtype dtype,
  double expansion_radius, void* out_min_x, void* out_min_y, void* out_max_x, void* out_max_y,
  void* stream);

/*
 * Replaces cuspatial::linestring_bounding_boxes
 * (cpp/include/cuspatial/bounding_boxes.hpp:52-57;
 * cpp/src/bounding_boxes/linestring_bounding_boxes.cu).
 */
cspt_status cspt_linestring_bounding_boxes(const uint32_t* linestring_offsets,
                                           size_t num_linestring_offsets, const void* x,
                                           const void* y, size_t num_vertices, cspt_dtype dtype,
                                           double expansion_radius, void* out_min_x,
                                           void* out_min_y, void* out_max_x, void* out_max_y,
                                           void* stream);

/*
 * Replaces cuspatial::join_quadtree_and_bounding_boxes
 * (cpp/include/cuspatial/spatial_join.hpp:66-75;
 * cpp/src/join/quadtree_bbox_filtering.cu:90-126).
 * Output pairs (bbox_offset, quad_offset) sorted by the leaf's first point,
 * then by bbox index — the reference's order.  Allocated with mr.
 */
cspt_status cspt_join_quadtree_and_bounding_boxes(
  const cspt_quadtree* tree, const void* bbox_min_x, const void* bbox_min_y,
  const void* bbox_max_x, const void* bbox_max_y, size_t num_bboxes, cspt_dtype dtype,
  double x_min, double x_max, double y_min, double y_max, double scale, int8_t max_depth,
  const cspt_allocator* mr, void* stream, uint32_t** out_bbox_offset,
  uint32_t** out_quad_offset, size_t* out_num_pairs);

/*
 * Replaces cuspatial::quadtree_point_in_polygon
 * (cpp/include/cuspatial/spatial_join.hpp:116-126;
 * cpp/src/join/quadtree_point_in_polygon.cu:143-191).
 * Output (polygon_index, point_index) in (pair order, point position) order;
 * point_index is a position in point_indices.  Allocated with mr.
 */
cspt_status cspt_quadtree_point_in_polygon(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* poly_offsets,
  size_t num_poly_offsets, const uint32_t* ring_offsets, size_t num_ring_offsets,
  const void* poly_x, const void* poly_y, size_t num_poly_vertices, cspt_dtype dtype,
  cspt_method method, const cspt_allocator* mr, void* stream, uint32_t** out_polygon_index,
  uint32_t** out_point_index, size_t* out_num_pairs);

/*
 * The whole quadtree point-in-polygon join, host columns in and host rows
 * out, in one call: cspt_quadtree_on_points_host, polygon bounding boxes,
 * cspt_join_quadtree_and_bounding_boxes and
 * cspt_quadtree_point_in_polygon_host with the corners ordered and the scale
 * clamped as the reference's Python join does (join.py:163-180).  The
 * polygons' copy, boxes and slab index run on a second stream while the
 * quadtree is built from the points; rows go to host_polygon_index and
 * host_point_index (host_capacity each) chunk by chunk.  Rows are those of
 * the separate calls, in their order, except that the point column holds
 * each point's row in the input columns (point_indices[point_index] of the
 * separate calls; the quadtree itself stays internal).  *out_num_rows
 * receives the row count; above host_capacity the call returns
 * CSPT_INVALID_ARGUMENT.  Host arrays should be page-locked for the copies
 * to overlap the work.  No counterpart in the reference.
 */
cspt_status cspt_point_in_polygon_join_host(
  const void* host_x, const void* host_y, size_t num_points, cspt_dtype dtype, double x_min,
  double x_max, double y_min, double y_max, double scale, int8_t max_depth, int32_t max_size,
  const uint32_t* host_poly_offsets, size_t num_poly_offsets, const uint32_t* host_ring_offsets,
  size_t num_ring_offsets, const void* host_poly_x, const void* host_poly_y,
  size_t num_poly_vertices, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* host_polygon_index, uint32_t* host_point_index, size_t host_capacity,
  size_t* out_num_rows);

/*
 * cspt_quadtree_point_in_polygon with the rows written to host memory, for a
 * caller whose results go to the host (the reference's column API followed by
 * a device-to-host copy of both columns).  Rows go to host_polygon_index and
 * host_point_index (host_capacity rows each), in the same order.  The pairs
 * are evaluated in chunks and each chunk's rows are copied while the next is
 * evaluated, so with page-locked host arrays the copies overlap the
 * evaluation.  Returns once the rows are in host memory.  *out_num_pairs
 * receives the row count; when it exceeds host_capacity the call returns
 * CSPT_INVALID_ARGUMENT (the message gives both counts) and the arrays hold
 * no complete result.
 */
cspt_status cspt_quadtree_point_in_polygon_host(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* poly_offsets,
  size_t num_poly_offsets, const uint32_t* ring_offsets, size_t num_ring_offsets,
  const void* poly_x, const void* poly_y, size_t num_poly_vertices, cspt_dtype dtype,
  cspt_method method, const cspt_allocator* mr, void* stream, uint32_t* host_polygon_index,
  uint32_t* host_point_index, size_t host_capacity, size_t* out_num_pairs);

/*
 * Replaces cuspatial::quadtree_point_to_nearest_linestring
 * (cpp/include/cuspatial/spatial_join.hpp:166-175;
 * cpp/src/join/quadtree_point_to_nearest_linestring.cu:142-187).
 * Writes num_point_indices rows into the caller's arrays and sets *out_num_rows
 * to num_point_indices (0 for the reference's empty-input cases).  Rows of
 * points that have no candidate get (position, 0xFFFFFFFF, 0).  Scratch
 * memory comes from mr.
 */
cspt_status cspt_quadtree_point_to_nearest_linestring(
  const uint32_t* pair_linestring, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* linestring_offsets,
  size_t num_linestring_offsets, const void* ls_x, const void* ls_y, size_t num_ls_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* out_point_index, uint32_t* out_linestring_index, void* out_distance,
  size_t* out_num_rows);

/*
 * cspt_quadtree_point_in_polygon, cspt_quadtree_point_in_polygon_host and
 * cspt_quadtree_point_to_nearest_linestring with the points given in
 * quadtree order (ordered_xy: num_points interleaved (x, y) pairs from
 * cspt_points_in_quadtree_order) in place of point_indices, x and y.  The
 * results, row order, validation and empty-input rules are those of the
 * calls they stand beside (point_index is still a position in
 * point_indices).  No counterpart in the reference (see
 * cspt_points_in_quadtree_order).
 */
cspt_status cspt_quadtree_point_in_polygon_ordered(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* poly_x, const void* poly_y, size_t num_poly_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t** out_polygon_index, uint32_t** out_point_index, size_t* out_num_pairs);
cspt_status cspt_quadtree_point_in_polygon_host_ordered(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* poly_x, const void* poly_y, size_t num_poly_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* host_polygon_index, uint32_t* host_point_index, size_t host_capacity,
  size_t* out_num_pairs);
cspt_status cspt_quadtree_point_to_nearest_linestring_ordered(
  const uint32_t* pair_linestring, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* linestring_offsets, size_t num_linestring_offsets, const void* ls_x,
  const void* ls_y, size_t num_ls_vertices, cspt_dtype dtype, cspt_method method,
  const cspt_allocator* mr, void* stream, uint32_t* out_point_index,
  uint32_t* out_linestring_index, void* out_distance, size_t* out_num_rows);

/*
 * Replaces cuspatial::point_in_polygon
 * (cpp/include/cuspatial/point_in_polygon.hpp:75-82;
 * cpp/src/point_in_polygon/point_in_polygon.cu:108-150).
 * Every point against every polygon (at most 31): out[i] bit p is set when
 * point i is inside polygon p.  out holds num_points int32 values (caller's
 * device memory).  poly_offsets holds num_polygons + 1 ring offsets.
 */
cspt_status cspt_point_in_polygon(const void* x, const void* y, size_t num_points,
                                  const uint32_t* poly_offsets, size_t num_poly_offsets,
                                  const uint32_t* ring_offsets, size_t num_ring_offsets,
                                  const void* poly_x, const void* poly_y,
                                  size_t num_poly_vertices, cspt_dtype dtype, cspt_method method,
                                  const cspt_allocator* mr, void* stream, int32_t* out);

/*
 * Replaces cuspatial::pairwise_point_in_polygon
 * (cpp/include/cuspatial/point_in_polygon.hpp:124-131;
 * cpp/src/point_in_polygon/point_in_polygon.cu:108-150 with pairwise).
 * Point i against polygon i: out[i] = 1 inside, 0 outside (num_points
 * uint8 values, caller's device memory); num_points must equal the number
 * of polygons.
 */
cspt_status cspt_pairwise_point_in_polygon(const void* x, const void* y, size_t num_points,
                                           const uint32_t* poly_offsets, size_t num_poly_offsets,
                                           const uint32_t* ring_offsets, size_t num_ring_offsets,
                                           const void* poly_x, const void* poly_y,
                                           size_t num_poly_vertices, cspt_dtype dtype,
                                           cspt_method method, const cspt_allocator* mr,
                                           void* stream, uint8_t* out);

/*
 * contains_properly in quadtree mode
 * (python/cuspatial/cuspatial/core/binpreds/contains.py:19-74): the
 * reference's parameters (max_depth 15, max_size ceil(sqrt(num_points)), the
 * polygons' vertex extent as the tree's box and the smallest unclamped
 * scale) run through cspt_quadtree_on_points, cspt_polygon_bounding_boxes,
 * cspt_join_quadtree_and_bounding_boxes and cspt_quadtree_point_in_polygon.
 * Rows in the join's order: out_point_index is the point's index in the
 * input (point_indices[point_index], contains.py:65-67), out_part_index the
 * polygon (part), out_geometry_index the multipolygon owning the part
 * (core/binpreds/contains_geometry_processor.py:72-116; equal to the part
 * when geometry_offsets is null).  Arrays allocated with mr.
 */
cspt_status cspt_quadtree_contains_properly(
  const void* x, const void* y, size_t num_points, const uint32_t* geometry_offsets,
  size_t num_geometry_offsets, const uint32_t* part_offsets, size_t num_part_offsets,
  const uint32_t* ring_offsets, size_t num_ring_offsets, const void* poly_x, const void* poly_y,
  size_t num_poly_vertices, cspt_dtype dtype, cspt_method method, const cspt_allocator* mr,
  void* stream, uint32_t** out_point_index, uint32_t** out_part_index,
  uint32_t** out_geometry_index, size_t* out_num_pairs);

/*
 * Replaces cuspatial::pairwise_point_linestring_distance
 * (cpp/include/cuspatial/distance.hpp:167-170;
 * cpp/src/distance/point_linestring_distance.cu:80-110).
 * Pair i: multipoint i (points [point_geometry_offsets[i], [i+1]) or, with
 * point_geometry_offsets NULL, point i) against multilinestring i (parts
 * [linestring_geometry_offsets[i], [i+1]) or, NULL, part i; part j has the
 * vertices [linestring_part_offsets[j], [j+1])).  Writes one distance per
 * pair (dtype of the coordinates) to the caller's device array.
 */
cspt_status cspt_pairwise_point_linestring_distance(
  const uint32_t* point_geometry_offsets, size_t num_point_geometry_offsets, const void* x,
  const void* y, size_t num_points, const uint32_t* linestring_geometry_offsets,
  size_t num_linestring_geometry_offsets, const uint32_t* linestring_part_offsets,
  size_t num_linestring_part_offsets, const void* ls_x, const void* ls_y,
  size_t num_ls_vertices, cspt_dtype dtype, cspt_method method, void* stream,
  void* out_distance);

/*
 * Replaces cuspatial::pairwise_point_linestring_nearest_points
 * (cpp/include/cuspatial/nearest_points.hpp:36-51 and :150-160;
 * cpp/src/nearest_points/point_linestring_nearest_points.cu:210-245).
 * Same inputs as cspt_pairwise_point_linestring_distance.  Per pair: the
 * point's index within its multipoint, the linestring's index within its
 * multilinestring, the segment's index within its linestring and the
 * nearest point (x, y interleaved).  out_point_geometry_id and
 * out_linestring_geometry_id may be NULL.  Pairs without a segment get
 * 0, 0, 0, (0, 0) (the reference leaves them unset).
 */
cspt_status cspt_pairwise_point_linestring_nearest_points(
  const uint32_t* point_geometry_offsets, size_t num_point_geometry_offsets, const void* x,
  const void* y, size_t num_points, const uint32_t* linestring_geometry_offsets,
  size_t num_linestring_geometry_offsets, const uint32_t* linestring_part_offsets,
  size_t num_linestring_part_offsets, const void* ls_x, const void* ls_y,
  size_t num_ls_vertices, cspt_dtype dtype, cspt_method method, void* stream,
  int32_t* out_point_geometry_id, int32_t* out_linestring_geometry_id, int32_t* out_segment_id,
  void* out_nearest_xy);

/* ------------------------------------------------------------------------
 * GeoArrow ingestion (python/cuspatial/cuspatial/io/pygeoarrow.py:9-70 and
 * core/_column/geocolumn.py): a geometry array handed over through the
 * Arrow C data interface becomes device columns with this library's offset
 * layout (geometry -> part -> ring -> point, x and y apart).  Accepted:
 *   - the reference's dense union of points / multipoints / linestrings /
 *     polygons (one type per column; points as list<double> of length 2);
 *   - native GeoArrow: points as fixed_size_list<double or float>[2] or
 *     struct<x, y>, nested in (large) lists, the type from the
 *     "ARROW:extension:name" metadata (geoarrow.point ... geoarrow.
 *     multipolygon) or from `kind`.
 * The Arrow buffers must be in host memory; no nulls.
 * ------------------------------------------------------------------------ */
#ifndef ARROW_C_DATA_INTERFACE
#define ARROW_C_DATA_INTERFACE
#define ARROW_FLAG_DICTIONARY_ORDERED 1
#define ARROW_FLAG_NULLABLE 2
#define ARROW_FLAG_MAP_KEYS_SORTED 4
struct ArrowSchema {
  const char* format;
  const char* name;
  const char* metadata;
  int64_t flags;
  int64_t n_children;
  struct ArrowSchema** children;
  struct ArrowSchema* dictionary;
  void (*release)(struct ArrowSchema*);
  void* private_data;
};
struct ArrowArray {
  int64_t length;
  int64_t null_count;
  int64_t offset;
  int64_t n_buffers;
  int64_t n_children;
  const void** buffers;
  struct ArrowArray** children;
  struct ArrowArray* dictionary;
  void (*release)(struct ArrowArray*);
  void* private_data;
};
#endif

/* Geometry kinds, in the order of the reference's union children.
 * LINESTRING and POLYGON columns carry multi-geometries too (geometry
 * offsets over parts). */
enum {
  CSPT_GEOM_POINT      = 0,
  CSPT_GEOM_MULTIPOINT = 1,
  CSPT_GEOM_LINESTRING = 2,
  CSPT_GEOM_POLYGON    = 3
};

typedef struct {
  int kind;
  int multi;        /* 1: multi-geometries (an extra list level) */
  int interleaved;  /* 1: xy interleaved in the Arrow buffer */
  cspt_dtype dtype;
  size_t num_geometries;
  size_t num_geometry_offsets, num_part_offsets, num_ring_offsets, num_points;
} cspt_geoarrow_layout;

/* Device columns: geometry_offsets (multipoint -> points, multilinestring
 * -> parts, multipolygon -> polygons; 0..n for single linestrings and
 * polygons, NULL for points), part_offsets (linestring -> points, polygon ->
 * rings), ring_offsets (ring -> points, polygons only), x, y. */
typedef struct {
  int kind;
  cspt_dtype dtype;
  size_t num_geometries;
  uint32_t* geometry_offsets;
  size_t num_geometry_offsets;
  uint32_t* part_offsets;
  size_t num_part_offsets;
  uint32_t* ring_offsets;
  size_t num_ring_offsets;
  void* x;
  void* y;
  size_t num_points;
} cspt_geometry_column;

/* Layout and sizes of a GeoArrow array (host only, no device work).
 * kind: a CSPT_GEOM_* value, or -1 to take it from the union or metadata. */
cspt_status cspt_geoarrow_describe(const struct ArrowSchema* schema,
                                   const struct ArrowArray* array, int kind,
                                   cspt_geoarrow_layout* out);

/* The same columns written to caller host buffers sized by
 * cspt_geoarrow_describe (no device work; NULL for absent levels). */
cspt_status cspt_geoarrow_read_host(const struct ArrowSchema* schema,
                                    const struct ArrowArray* array, int kind,
                                    uint32_t* geometry_offsets, uint32_t* part_offsets,
                                    uint32_t* ring_offsets, void* x, void* y);

/* Copies a GeoArrow array to device columns allocated with mr (one
 * host->device copy per buffer; interleaved coordinates are split on the
 * device).  Synchronises the stream.  The caller keeps ownership of the
 * Arrow structures (they are not released). */
cspt_status cspt_geoarrow_import(const struct ArrowSchema* schema, const struct ArrowArray* array,
                                 int kind, const cspt_allocator* mr, void* stream,
                                 cspt_geometry_column* out);

/* Releases the device columns of cspt_geoarrow_import (same allocator). */
void cspt_geometry_column_free(const cspt_allocator* mr, cspt_geometry_column* col, void* stream);

/* ------------------------------------------------------------------------
 * Batched point-in-polygon join (no counterpart in the reference, which
 * joins one point set with one polygon set per call).
 *
 * Many independent instances, each with its own points, polygons and
 * quadtree parameters, are planned together: one tree build over all
 * points, one box join over all polygons, one polygon index.  Running the
 * plan evaluates every instance's candidate pairs in the same kernels and
 * writes, per instance, exactly the rows that
 *   cspt_quadtree_on_points -> cspt_polygon_bounding_boxes (radius 0) ->
 *   cspt_join_quadtree_and_bounding_boxes -> cspt_quadtree_point_in_polygon
 * return for that instance alone with its parameters.
 *
 * Inputs (device, float64): x/y of all points, instance i owning points
 * [point_offsets[i], point_offsets[i+1]); a polygon column whose
 * poly_offsets index ring_offsets and whose ring_offsets index poly_x/poly_y
 * (global offsets), instance i owning polygons
 * [polygon_offsets[i], polygon_offsets[i+1]).  point_offsets,
 * polygon_offsets (num_instances + 1 entries each, starting at 0) and params
 * are HOST arrays.  Every polygon must have at least one vertex.  Inputs are
 * borrowed for the plan's lifetime.
 * ------------------------------------------------------------------------ */
typedef struct cspt_instance_params {
  double x_min, x_max, y_min, y_max; /* quadtree area: x_min < x_max, y_min < y_max */
  double scale;                      /* raised to max(dx, dy) / ((1 << max_depth) + 2) */
  int32_t max_depth;                 /* 1..15 */
  int32_t max_size;                  /* raised to 1 */
} cspt_instance_params;

typedef struct cspt_batched_pip cspt_batched_pip;

/* Results of a plan (device pointers owned by the plan).  Rows of instance i
 * are [row_offsets[i], row_offsets[i+1]); polygon_index is local to the
 * instance's polygons and point_index is a position in the instance's
 * point_indices.  point_indices holds instance i's sorted point order at
 * [point_offsets[i], point_offsets[i+1]) with instance-local values; tree
 * holds instance i's nodes at [node_offsets[i], node_offsets[i+1]) with
 * instance-local child and point offsets.  Rows are valid once a run has
 * completed. */
typedef struct cspt_batched_pip_info {
  size_t num_instances, num_points, num_polygons, num_nodes, num_pairs, num_rows;
  uint64_t kernels_per_run; /* kernel launches one graph replay makes (0 before capture) */
  const uint32_t* polygon_index;
  const uint32_t* point_index;
  const uint64_t* row_offsets;
  const uint32_t* point_indices;
  cspt_quadtree tree;
  const uint64_t* node_offsets;
} cspt_batched_pip_info;

/* Builds the trees, joins the boxes, builds the polygon index and sizes the
 * outputs by one evaluation; synchronises `stream`.  method selects plain
 * float64 or float32-filtered evaluation (same rows).  ordered_index != 0
 * sorts each slab's crossing edges and keeps per-(slab, x-bin) windows: a
 * longer plan and faster runs (for plans run many times); 0 keeps the
 * one-shot index and its quadrant fast path (the shortest plan + run).
 * block_threads (a multiple of 32 up to 256; 256 is a good default) is the
 * block size of the per-pair kernels with the ordered index (the one-shot
 * index's kernel takes 256).  Device memory comes from mr on `stream`, which
 * must stay valid until cspt_batched_pip_free. */
cspt_status cspt_batched_pip_plan(
  size_t num_instances, const uint64_t* point_offsets, const void* x, const void* y,
  const uint64_t* polygon_offsets, const uint32_t* poly_offsets, size_t num_poly_offsets,
  const uint32_t* ring_offsets, size_t num_ring_offsets, const void* poly_x, const void* poly_y,
  size_t num_poly_vertices, const cspt_instance_params* params, cspt_dtype dtype,
  cspt_method method, int ordered_index, int block_threads, const cspt_allocator* mr,
  void* stream, cspt_batched_pip** out_plan);

/* Evaluates all instances on `stream` (asynchronous; allocates nothing).
 * The first run after the plan reuses the plan's sizing evaluation and only
 * writes the rows; later runs evaluate again.  With use_graph != 0 a full
 * evaluation is recorded into a CUDA graph on the first such call that
 * evaluates and replayed as one graph launch afterwards. */
cspt_status cspt_batched_pip_run(cspt_batched_pip* plan, int use_graph, void* stream);

cspt_status cspt_batched_pip_get_info(const cspt_batched_pip* plan, cspt_batched_pip_info* out);

/* Candidates re-evaluated in float64 by the last run (filtered method);
 * synchronises `stream`. */
cspt_status cspt_batched_pip_refined_count(const cspt_batched_pip* plan, void* stream,
                                           uint64_t* out);

/* Frees the plan; runs issued on it must have completed. */
void cspt_batched_pip_free(cspt_batched_pip* plan);

/* ------------------------------------------------------------------------
 * Serving form (no counterpart in the reference): a device-resident polygon
 * set answering point-in-polygon requests that arrive over time.
 *
 * A request is a host array of float64 points plus its quadtree parameters.
 * Its answer is exactly what cspt_quadtree_on_points ->
 * cspt_polygon_bounding_boxes (whole set) -> cspt_join_quadtree_and_bounding_boxes
 * -> cspt_quadtree_point_in_polygon return for those points against the whole
 * set: (polygon_index into the set, point_index = position in the request's
 * point_indices) rows in the reference's order, plus point_indices.  The
 * answer does not depend on which other requests share its batch.
 *
 * The server queues requests on submit; worker threads, one CUDA stream
 * each, take batches of queued requests in arrival order as soon as a worker
 * is free and the estimated device memory of all batches in flight stays
 * within memory_budget_bytes.  Device memory of batches comes from a byte
 * budget of that size; a batch that runs out is split and its requests are
 * retried one at a time.  A request that cannot fit even alone fails with
 * CSPT_OUT_OF_MEMORY; other requests are unaffected.
 * ------------------------------------------------------------------------ */
typedef struct cspt_polygon_set cspt_polygon_set;
typedef struct cspt_server cspt_server;

/* Copies the polygon column (device, float64; every polygon must have a
 * vertex) into a resident set with its boxes, cell grid and point-in-polygon
 * index.  Memory comes from mr on `stream`, which must stay valid until the
 * set is freed; synchronises `stream`. */
cspt_status cspt_polygon_set_create(const uint32_t* poly_offsets, size_t num_poly_offsets,
                                    const uint32_t* ring_offsets, size_t num_ring_offsets,
                                    const void* poly_x, const void* poly_y,
                                    size_t num_poly_vertices, cspt_dtype dtype,
                                    const cspt_allocator* mr, void* stream,
                                    cspt_polygon_set** out);
/* Frees the set; servers using it must be freed first. */
void cspt_polygon_set_free(cspt_polygon_set* set);

typedef struct cspt_server_options {
  size_t memory_budget_bytes; /* device memory all batches in flight may hold */
  int num_streams;            /* worker threads, one CUDA stream each */
  size_t max_batch_points;    /* points per batch (a larger request runs alone) */
  size_t max_batch_requests;  /* requests per batch */
  cspt_method method;
  int block_threads;          /* per-pair kernel block size: multiple of 32, <= 256 */
} cspt_server_options;

typedef struct cspt_server_stats {
  uint64_t submitted, completed, failed, batches, split_batches, queued;
  size_t reserved_bytes, peak_device_bytes, memory_budget_bytes;
  uint64_t max_batch_requests_seen;
} cspt_server_stats;

typedef struct cspt_request_result {
  int status;        /* cspt_status of the request */
  const char* error; /* message when status != CSPT_OK */
  const uint32_t* polygon_index;
  const uint32_t* point_index;
  size_t num_rows;
  const uint32_t* point_indices;
  size_t num_points;
  double submit_s, admit_s, done_s; /* server clock (cspt_server_now) */
  uint64_t batch;
  uint32_t batch_requests;
} cspt_request_result;

cspt_status cspt_server_create(const cspt_polygon_set* set, const cspt_server_options* options,
                               cspt_server** out);
/* Queues a request.  x and y (host) must stay valid until the request
 * completes; parameters are validated here (same messages as the join). */
cspt_status cspt_server_submit(cspt_server* server, uint64_t request_id, const double* x,
                               const double* y, size_t num_points,
                               const cspt_instance_params* params);
/* Ids of requests completed since the last poll (waits up to timeout_s for
 * the first). */
size_t cspt_server_poll(cspt_server* server, uint64_t* ids, size_t max_ids, double timeout_s);
/* Result of a completed request; pointers stay valid until release. */
cspt_status cspt_server_result(cspt_server* server, uint64_t request_id,
                               cspt_request_result* out);
void cspt_server_release(cspt_server* server, uint64_t request_id);
double cspt_server_now(const cspt_server* server);
cspt_status cspt_server_get_stats(cspt_server* server, cspt_server_stats* out);
/* Finishes the queued requests, then stops the workers. */
void cspt_server_free(cspt_server* server);

#ifdef __cplusplus
}
#endif

#endif /* CUSPATIAL_GB300_H */
