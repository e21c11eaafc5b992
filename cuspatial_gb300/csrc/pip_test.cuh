// Per-candidate point-in-polygon tests shared by the quadtree join
// (pip.cu) and the unindexed calls (point_in_polygon.cu).
//
// Reference: detail/algorithm/is_point_in_polygon.cuh:45-100.  The exact
// tests evaluate the reference's float64 (or float32) expressions; the
// float32 filter decides a candidate only where a forward error bound proves
// the reference's answer, and hands the rest to the exact tests.
#pragma once

#include "common.cuh"
#include "polygon_index.cuh"

namespace cspt {
namespace {  // one copy per translation unit

// detail/algorithm/is_point_in_polygon.cuh:45-100, literally: rings in
// order, the degenerate-edge skip keeps b, the first b is the ring's last
// vertex, any on-edge hit makes the polygon false.
template <typename T>
__device__ bool ring_walk(T px, T py, PolygonIndexView<T> const& ix, uint32_t poly)
{
  bool within  = false;
  bool on_edge = false;
  uint32_t const r0 = ix.poly_offsets[poly], r1 = ix.poly_offsets[poly + 1];
  for (uint32_t r = r0; r < r1; ++r) {
    uint32_t const v0 = ix.ring_offsets[r], v1 = ix.ring_offsets[r + 1];
    if (v1 <= v0) continue;
    T bx    = ix.vx[v1 - 1];
    T by    = ix.vy[v1 - 1];
    bool y0 = by > py;
    for (uint32_t v = v0; v < v1; ++v) {
      T const ax = ix.vx[v], ay = ix.vy[v];
      T const run = bx - ax, rise = by - ay;
      if (float_equal(run, T{0}) && float_equal(rise, T{0})) continue;
      T const rtp  = py - ay;
      T const rtpx = px - ax;
      if (float_equal(run * rtp, rtpx * rise)) {
        T mn = ax, mx = bx;
        if (mn > mx) {
          T const t = mn;
          mn        = mx;
          mx        = t;
        }
        if (mn <= px && px <= mx) {
          on_edge = true;
          break;
        }
      }
      bool const y1 = ay > py;
      if (y1 != y0) {
        T const lhs = (px - ax) * rise;
        T const rhs = run * rtp;
        if ((lhs < rhs) != y1) within = !within;
      }
      bx = ax;
      by = ay;
      y0 = y1;
    }
    if (on_edge) return false;
  }
  return within;
}

template <typename V>
__device__ inline bool sorted_has(V const* a, uint32_t b, uint32_t e, V x)
{
  uint32_t lo = b, hi = e;
  while (lo < hi) {
    uint32_t const m = (lo + hi) >> 1;
    if (a[m] < x)
      lo = m + 1;
    else
      hi = m;
  }
  return lo < e && a[lo] == x;
}

template <typename T>
__device__ inline uint32_t point_slab(T py, PolygonIndexView<T> const& ix, uint32_t poly)
{
  uint32_t const ns = ix.num_slabs[poly];
  T const f         = (py - ix.pminy[poly]) * ix.inv_slab_h[poly];
  if (!(f > T{0})) return 0;
  if (f >= static_cast<T>(ns)) return ns - 1;
  uint32_t const j = static_cast<uint32_t>(f);
  return j < ns ? j : ns - 1;
}

// One effective edge (b -> a) of the reference's ring walk
// (is_point_in_polygon.cuh:61-90), in the input precision: 2 when the point
// is on the edge, 1 when the edge toggles the crossing parity, 0 otherwise.
template <typename T>
__device__ inline int exact_edge(T px, T py, T ax, T ay, T bx, T by)
{
  T const run = bx - ax, rise = by - ay;
  T const rtp = py - ay, rtpx = px - ax;
  if (float_equal(run * rtp, rtpx * rise)) {
    T const mn = ax < bx ? ax : bx;
    T const mx = ax < bx ? bx : ax;
    if (mn <= px && px <= mx) return 2;
  }
  bool const y1 = ay > py;
  bool const y0 = by > py;
  if (y1 != y0 && ((rtpx * rise < run * rtp) != y1)) return 1;
  return 0;
}

// The reference's test restricted to the edges of the point's slab.
template <typename T>
__device__ bool pip_exact(T px, T py, PolygonIndexView<T> const& ix, uint32_t poly)
{
  if (!(py >= ix.pminy[poly]) || !(py < ix.pmaxy[poly])) return false;
  if (ix.exact_only[poly]) return ring_walk<T>(px, py, ix, poly);
  if (sorted_has<T>(ix.vert_x, ix.vert_begin[poly], ix.vert_end[poly], px)) return false;
  uint32_t const s  = ix.slab_base[poly] + point_slab<T>(py, ix, poly);
  uint32_t const e0 = ix.slab_start[s], e1 = ix.slab_start[s + 1];
  bool within       = false;
  for (uint32_t k = e0; k < e1; ++k) {
    uint32_t const v  = ix.slab_edges[k] & kEntryVertex;
    uint32_t const pv = ix.prev_vertex[v];
    T const ax = ix.vx[v], ay = ix.vy[v], bx = ix.vx[pv], by = ix.vy[pv];
    T const run = bx - ax, rise = by - ay;
    T const rtp = py - ay, rtpx = px - ax;
    if (float_equal(run * rtp, rtpx * rise)) {
      T const mn = ax < bx ? ax : bx;
      T const mx = ax < bx ? bx : ax;
      if (mn <= px && px <= mx) return false;
    }
    bool const y1 = ay > py;
    bool const y0 = by > py;
    if (y1 != y0) {
      T const lhs = rtpx * rise;
      T const rhs = run * rtp;
      if ((lhs < rhs) != y1) within = !within;
    }
  }
  return within;
}

constexpr int kUndecided = 2;

// float32 filter, in a frame anchored on the polygon grid (a quadrant's
// leaf frame, or a single point's own frame).
//
// Maps: a point goes through f_l(v) = fl32(fl32(v - A_l) - d) with d the
// exact offset between the grid-rounded polygon and leaf anchors, so
// |f_l(p) - (p - A_p)| <= 2 u32 M; edge ends were stored as
// f_p(v) = fl32(v - A_p), |f_p(v) - (v - A_p)| <= u32 M, where M bounds the
// offsets involved (the polygon's, the leaf's and the point's).  Hence:
//   * the box reject compares f_l with f_l (monotone) and needs px beyond the
//     box by more than the float64 rounding of the reference's comparison
//     (2^-44 M): tol = 2^-21 M covers it and the mapping error;
//   * f_l against f_p comparisons (y-flags, x-ranges, vertical x) are certain
//     beyond tol (> 3 u32 M) and undecided within it;
//   * |cross32 - (lhs64 - rhs64)| <= 56 u32 M^2 (point and edge roundings
//     through the differences, products and FMA) + 2^-49 M^2 (float64
//     rounding and the 4-ULP collinear band); the test uses
//     2^-17 M^2 = 128 u32 M^2, plus 2^-120 for float32 underflow;
//   * the float32 slab index is off by at most 8 u32 M invh + 2 u32 nslab
//     slabs; edges are binned 1/64 slab wide of their range, so the filter
//     requires M invh <= 2^14.
// Undecided points are re-evaluated with pip_exact.  The polygon box is kept
// in the polygon's frame (f_p), so the box reject is a cross-frame comparison
// with tol as well.

// The float32-filtered crossing test of one point against one polygon (the
// bounds are stated above).  (qx, qy): the point's float32 offset from the
// polygon's anchor; mp: the polygon's largest offset; mlf: the largest offset
// of the point's own frame; load(px, py) fetches the point's float64
// coordinates when an edge or the whole test needs the reference's float64
// arithmetic; nref counts those.
template <bool Ordered, class Load>
__device__ __forceinline__ bool filtered_test(PolygonIndexView<double> const& ix, uint32_t poly,
                                              float qx, float qy, float mp, float mlf,
                                              float4 const& bx, float invh, float invw,
                                              uint32_t ns, uint32_t slab0, uint32_t vb,
                                              uint32_t ve, Load const& load, uint32_t& nref)
{
  int r       = kUndecided;  // 0/1 decided, kUndecided: run the whole exact test
  bool have64 = false;
  double px64 = 0.0, py64 = 0.0;
  float const m   = fmaxf(fmaxf(mp, mlf), fmaxf(fabsf(qx), fabsf(qy)));
  float const tol = 4.76837158203125e-07f * m;  // 2^-21 M
  if (qx < bx.x - tol || qx > bx.z + tol || qy < bx.y - tol || qy > bx.w + tol) {
    r = 0;
  } else if (m * invh <= 16384.0f) {
    r = -1;  // in progress
    if (vb < ve) {
      // a vertical edge within tol: decide the px == x quirk exactly
      uint32_t lo = vb, hi = ve;
      float const key = qx - tol;
      while (lo < hi) {
        uint32_t const mid = (lo + hi) >> 1;
        if (ix.vert_x32[mid] < key)
          lo = mid + 1;
        else
          hi = mid;
      }
      if (lo < ve && ix.vert_x32[lo] <= qx + tol) {
        load(px64, py64);
        have64 = true;
        if (sorted_has<double>(ix.vert_x, vb, ve, px64)) r = 0;
      }
    }
    if (r == -1) {
      float const eb = __fmaf_rn(7.62939453125e-06f * m, m, 7.52316384526264e-37f);
      float const fs = (qy - bx.y) * invh;
      uint32_t sj    = 0;
      if (fs > 0.0f) sj = fs >= static_cast<float>(ns) ? ns - 1 : static_cast<uint32_t>(fs);
      if (sj >= ns) sj = ns - 1;
      uint32_t const sidx = slab0 + sj;
      uint32_t const e0 = ix.slab_start[sidx], e1 = ix.slab_start[sidx + 1];
      // crossing edges [e0, e0 + nf): only the point's x-bin window
      // [wlo, whi) is tested, those after it all toggle (parity bit);
      // the other edges [e0 + nf, e1) are all tested
      uint32_t const nf = Ordered ? ix.slab_nfull[sidx] : 0u;
      uint32_t wlo = 0, whi = nf;
      bool within = false;
      if (Ordered && nf > 0 && m * invw <= 16384.0f) {
        float const fb   = (qx - bx.x) * invw;
        uint32_t const top = static_cast<uint32_t>(kSlabBins - 1);
        uint32_t const b   = fb > 0.0f ? (fb < static_cast<float>(top)
                                            ? static_cast<uint32_t>(fb)
                                            : top)
                                       : 0u;
        uint32_t const rec = ix.slab_bins[static_cast<size_t>(sidx) * kSlabBins + b];
        wlo    = rec & 0x7FFFu;
        whi    = (rec >> 15) & 0x7FFFu;
        within = (rec >> 30) & 1u;
      }
      uint32_t const nwin = whi - wlo;
      uint32_t const ntot = nwin + (e1 - e0 - nf);
      for (uint32_t t = 0; t < ntot; ++t) {
        uint32_t const k2 =
          Ordered ? (t < nwin ? e0 + wlo + t : e0 + nf + (t - nwin)) : e0 + t;
        float4 const e = ix.slab_e32[k2];  // (ax, ay, bx, by)
        float const ya = e.y - qy, yb = e.w - qy;
        bool const y1  = ya > 0.0f;
        bool const y0  = yb > 0.0f;
        float const cr = __fmaf_rn(qx - e.x, e.w - e.y, -((e.z - e.x) * (qy - e.y)));
        bool const undecided =
          fabsf(ya) <= tol || fabsf(yb) <= tol ||
          (fabsf(cr) <= eb &&
           (y1 != y0 || !(qx < fminf(e.x, e.z) - tol || qx > fmaxf(e.x, e.z) + tol)));
        if (!undecided) {
          if (y1 != y0 && ((cr < 0.0f) != y1)) within = !within;
          continue;
        }
        // this edge only, with the reference's float64 expression
        ++nref;
        if (!have64) {
          load(px64, py64);
          have64 = true;
        }
        uint32_t const v  = ix.slab_edges[k2] & kEntryVertex;
        uint32_t const pv = ix.prev_vertex[v];
        int const ee =
          exact_edge<double>(px64, py64, ix.vx[v], ix.vy[v], ix.vx[pv], ix.vy[pv]);
        if (ee == 2) {
          r = 0;  // on an edge: outside
          break;
        }
        if (ee == 1) within = !within;
      }
      if (r == -1) r = within ? 1 : 0;
    }
  }
  if (r == kUndecided) {
    ++nref;
    if (!have64) load(px64, py64);
    return pip_exact<double>(px64, py64, ix, poly);
  }
  return r == 1;
}

}  // namespace
}  // namespace cspt
