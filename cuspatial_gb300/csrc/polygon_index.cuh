// Device-resident polygon index used by the point-in-polygon join.
//
// For every polygon the index holds
//   * its vertex bounding box and an anchor (box centre),
//   * each vertex's edge (previous vertex -> vertex, ring-cyclic) as float32
//     offsets from the anchor, plus the largest offset magnitude,
//   * a partition of [ymin, ymax) into slabs, each listing the edges whose
//     y-range (widened by a margin) meets the slab,
//   * the sorted x values of its exactly vertical edges.
//
// Why this is exact against the reference's ring walk
// (detail/algorithm/is_point_in_polygon.cuh:45-100):
//   1. For coordinates of normal magnitude, float_equal(b - a, 0) holds only
//      for b == a, and equality is transitive, so the reference's skipped
//      vertices are exactly those equal to their predecessor and its edges
//      are (p[i-1], p[i]) for the other vertices.  Polygons where a vertex
//      difference is non-zero but within 4 ULP of zero (denormal scale) are
//      flagged and always walked with the reference loop.
//   2. The result is "no on-edge hit" AND the XOR of per-edge toggles, so the
//      edges can be visited in any order and any subset that contains every
//      edge able to toggle or to hit is enough.
//   3. A point with py outside [ymin, ymax) sees equal y-flags on every edge:
//      no toggle, result false.
//   4. An edge toggles only if its y-range contains py; a non-vertical edge
//      can be "collinear and within x-range" only if py lies within
//      2^-48 * |rise| of its y-range.  Each edge is binned over its y-range
//      widened by 2^-36 of its height, which covers both.
//   5. An exactly vertical edge reports "on edge" for any py whenever
//      px == its x (x-range check only, is_point_in_polygon.cuh:75-83); that
//      case is caught by a lookup in the sorted vertical-x list.
//   6. Slab coordinates are float32 roundings of the float64 (y - ymin) *
//      inv_h (2.5e-4 slab at most); edges are further widened by 1/32 of a
//      slab, which covers that and the float32 slab lookup of the filter
//      (below 1e-2 slab under its guard), so every lookup finds every edge.
//
// Anchors lie on a power-of-two grid (2^(e-22) for coordinates below 2^e), so
// the offset between a polygon anchor and a leaf anchor on the same grid is
// exact in float64 and, when below 2^24 grid steps, in float32.
#pragma once

#include <memory>

#include "common.cuh"

namespace cspt {

// x-bins per slab of the float32 index (window records per slab)
constexpr int kSlabBins = 8;
// slab entries: vertex id in bits 0-30, bit 31 set when the edge crosses the
// whole slab (float32 index)
constexpr uint32_t kEntryCrossing = 1u << 31;
constexpr uint32_t kEntryVertex   = kEntryCrossing - 1u;

template <typename T>
struct PolygonIndexView {
  // polygon topology (caller's arrays)
  uint32_t const* poly_offsets;
  uint32_t const* ring_offsets;
  T const* vx;
  T const* vy;
  size_t num_polygons;
  // per polygon
  T const* pminx;
  T const* pminy;
  T const* pmaxx;
  T const* pmaxy;
  T const* anchor_x;           // box centre rounded to the grid
  T const* anchor_y;
  T const* grid;               // device scalar: the anchor grid step
  long long const* anchor_ix;  // anchors in grid steps
  long long const* anchor_iy;
  float const* inv_slab_h32;   // inv_slab_h rounded to float
  T const* inv_slab_h;         // slabs per unit of y
  float const* max_offset;     // largest |float32 offset| over the polygon's vertices
  float4 const* box32;         // vertex box as float32 offsets from the anchor
  uint32_t const* num_slabs;
  uint32_t const* slab_base;   // first slab of the polygon in slab_start
  uint8_t const* exact_only;   // 1: walk the reference loop, no index
  uint32_t const* vert_begin;  // sorted vertical-edge x values, per polygon range
  uint32_t const* vert_end;
  T const* vert_x;
  float const* vert_x32;
  // per slab: entries [slab_start[s], slab_start[s+1])
  uint32_t const* slab_start;
  uint32_t const* slab_edges;  // vertex index of the edge's end point | kEntryCrossing
  float4 const* slab_e32;      // the entry's edge (ax, ay, bx, by) as float32 offsets
  // per vertex
  uint32_t const* prev_vertex;
  float4 const* edge32;        // (ax, ay, bx, by) offsets from the anchor
  // float32 index: per slab, the entries crossing the whole slab come first
  // (sorted left to right); per (slab, x-bin) a window record
  // lo | hi << 15 | parity << 30 (see slab_order_kernel)
  uint32_t const* slab_nfull;  // null: slabs not ordered
  uint32_t const* slab_bins;
  float const* inv_bin_w32;    // x-bins per unit of x (0: no bins)
};

template <typename T>
class PolygonIndex {
 public:
  // order_slabs (float32 index only): sort each slab's crossing edges and
  // build the per-(slab, x-bin) windows.  It costs a pass over all slab
  // entries and pays off where the index is evaluated many times (batched
  // plans, resident polygon sets).
  // defer_fill: return once the per-polygon boxes, slab counts and the anchor
  // grid are enqueued (array sizes come from bounds on the host, so the call
  // does not wait for the device); fill() then writes the slab entries.  Work
  // that needs only grid() can run on another stream meanwhile, once it waits
  // for the calling stream.
  PolygonIndex(uint32_t const* poly_offsets, size_t num_poly_offsets,
               uint32_t const* ring_offsets, size_t num_ring_offsets, T const* vx, T const* vy,
               size_t num_vertices, bool build_float32, Allocator const& alloc,
               bool order_slabs = false, bool defer_fill = false);
  ~PolygonIndex();
  PolygonIndex(PolygonIndex const&)            = delete;
  PolygonIndex& operator=(PolygonIndex const&) = delete;
  void fill();
  // device scalar: the anchor grid step (valid before fill())
  T const* grid() const { return grid_.data(); }
  PolygonIndexView<T> view() const { return v_; }

 private:
  struct Sizing;  // state carried from the sizing pass to fill()
  std::unique_ptr<Sizing> sizing_;
  Buffer<T> pminx_, pminy_, pmaxx_, pmaxy_, ax_, ay_, invh_, vert_x_, grid_;
  Buffer<float> maxoff_, vert_x32_, invh32_;
  Buffer<long long> aix_, aiy_;
  Buffer<uint32_t> nslab_, slab_base_, vbeg_, vend_, slab_start_, slab_edges_, prev_;
  Buffer<uint8_t> exact_;
  Buffer<float4> edge32_, box32_, slab_e32_;
  Buffer<uint32_t> slab_nfull_, slab_bins_;
  Buffer<float> invw32_;
  PolygonIndexView<T> v_{};
};

// A planned float64 point-in-polygon evaluation (defined in pip.cu).
class PipExec {
 public:
  PipExec(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t npairs,
          uint32_t const* qlen, uint32_t const* qoff, uint32_t const* point_indices, size_t npi,
          double const* x, double const* y, PolygonIndexView<double> const& ix, bool filtered,
          unsigned block_threads, Allocator const& alloc);
  ~PipExec();
  PipExec(PipExec const&)            = delete;
  PipExec& operator=(PipExec const&) = delete;
  void execute(cudaStream_t s, uint32_t* out_poly, uint32_t* out_point, uint64_t cap);
  void evaluate(cudaStream_t s);  // bits, counts and output offsets
  void expand(cudaStream_t s, uint32_t* out_poly, uint32_t* out_point, uint64_t cap);
  uint64_t const* total() const;             // device: number of output pairs
  uint64_t const* pair_out_offsets() const;  // device: first output of each pair
  int const* overflow() const;               // device: 1 when total > cap
  unsigned long long const* refined() const;

 private:
  class Impl;
  Impl* impl_;
};

}  // namespace cspt
