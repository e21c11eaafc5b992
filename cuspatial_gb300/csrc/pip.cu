// Quadtree point-in-polygon join on sm_103a.
//
// Reference: cpp/include/cuspatial/detail/join/quadtree_point_in_polygon.cuh:
// 104-235 (candidate enumeration and compaction), get_quad_and_local_point_
// indices.cuh:26-45 and detail/algorithm/is_point_in_polygon.cuh:45-100 (the
// per-pair test).
//
// Layout of the work: one warp per (polygon, quadrant) pair, lanes over the
// quadrant's points 32 at a time.  Each 32-point chunk produces one ballot
// word in a bitmask laid out pair by pair; a scan of per-pair hit counts then
// places every pair's hits, and an expansion kernel writes
// (polygon, point position) in the reference's order: pair order, then
// ascending position.  Only the bitmask (one bit per candidate) and the
// exact-size output touch HBM, never a candidate-sized pair buffer.
//
// Per candidate test (see polygon_index.cuh for why it equals the reference):
//   exact    : y-range reject, vertical-x lookup, then the reference's
//              float64 edge test over the edges of the point's slab;
//   filtered : the same edges in float32 on anchored coordinates with a
//              forward error bound; any undecided edge sends the candidate
//              to the exact test.
#include "common.cuh"
#include "leaf_frame.cuh"
#include "polygon_index.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

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
constexpr int kPipBlock = 256;
// resident blocks per SM the registers are sized for (filtered / exact)
#ifndef CSPT_PIP_MIN_BLOCKS
#define CSPT_PIP_MIN_BLOCKS 6
#endif
#ifndef CSPT_PIP_MIN_BLOCKS_EXACT
#define CSPT_PIP_MIN_BLOCKS_EXACT 8
#endif
constexpr int kPipMinBlocksFiltered = CSPT_PIP_MIN_BLOCKS;
constexpr int kPipMinBlocksExact    = CSPT_PIP_MIN_BLOCKS_EXACT;

// resident blocks of a pair kernel: the persistent grid
template <typename K>
unsigned pair_grid(K kernel, unsigned block, size_t npairs)
{
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, static_cast<int>(block), 0) !=
        cudaSuccess ||
      per_sm < 1) {
    (void)cudaGetLastError();
    per_sm = 1;
  }
  size_t const want = (npairs * 32 + block - 1) / block;
  size_t const cap  = static_cast<size_t>(num_sms()) * static_cast<size_t>(per_sm);
  return static_cast<unsigned>(want < 1 ? 1 : (want < cap ? want : cap));
}
// float32 filter, in the leaf's frame (used by pip_group_kernel below).
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

// One warp per (polygon, quadrant) pair, lanes over the quadrant's points.
// Filtered: float32 test in the leaf frame (bounds above), undecided points
// re-evaluated with pip_exact.  Exact: pip_exact on float64 coordinates.
//
// Pairs are handed out dynamically: each warp takes the next pair index from
// a device counter (zeroed before the launch), so warps that drew cheap pairs
// keep working while others finish long ones; the grid holds only as many
// blocks as are resident.
// Ordered: the index's slabs are ordered (slab_order_kernel) and the
// per-(slab, x-bin) windows are used.
template <bool Filtered, bool Ordered = false>
__global__ void __launch_bounds__(kPipBlock, Filtered ? kPipMinBlocksFiltered : kPipMinBlocksExact)
  pip_pair_kernel(uint32_t const* __restrict__ pair_poly, uint32_t const* __restrict__ pair_quad,
                  uint32_t const* __restrict__ pair_group, size_t npairs,
                  uint32_t const* __restrict__ qlen, uint32_t const* __restrict__ qoff,
                  uint32_t const* __restrict__ point_indices, size_t npi,
                  double const* __restrict__ x, double const* __restrict__ y,
                  float2 const* __restrict__ u, LeafFrame const* __restrict__ frames,
                  PolygonIndexView<double> ix, uint64_t const* __restrict__ word_off,
                  uint32_t* __restrict__ bits, uint32_t* __restrict__ counts,
                  unsigned long long* __restrict__ refined,
                  unsigned long long* __restrict__ next_pair)
{
  int const lane      = threadIdx.x & 31;
  float const gf      = Filtered ? static_cast<float>(*ix.grid) : 0.0f;
  bool const gok      = gf >= 1.17549435e-38f && gf < 1.0e30f;  // normal float grid step
  uint32_t nref       = 0;
  for (;;) {
    unsigned long long kk = 0;
    if (lane == 0) kk = atomicAdd(next_pair, 1ull);
    size_t const k = static_cast<size_t>(__shfl_sync(0xFFFFFFFFu, kk, 0));
    if (k >= npairs) break;
    uint32_t const poly = pair_poly[k];
    uint32_t const quad = pair_quad[k];
    uint32_t const len  = qlen[quad];
    uint64_t const off  = qoff[quad];
    uint64_t const wb   = word_off[k];
    uint32_t const nw   = (len + 31) >> 5;
    uint32_t cnt        = 0;
    if (poly >= ix.num_polygons) {
      for (uint32_t w = lane; w < nw; w += 32) bits[wb + w] = 0u;
      if (lane == 0) counts[k] = 0;
      continue;
    }
    if constexpr (Filtered) {
      LeafFrame const lf = frames[pair_group[k]];
      // anchor offset in grid steps: exact in float32 below 2^24 steps
      long long const dix = ix.anchor_ix[poly] - lf.ix;
      long long const diy = ix.anchor_iy[poly] - lf.iy;
      bool const exact    = ix.exact_only[poly] || lf.nonfinite || !gok ||
                         dix <= -16777216LL || dix >= 16777216LL || diy <= -16777216LL ||
                         diy >= 16777216LL;
      float const dx = exact ? 0.0f : static_cast<float>(static_cast<int>(dix)) * gf;
      float const dy = exact ? 0.0f : static_cast<float>(static_cast<int>(diy)) * gf;
      float4 const bx = ix.box32[poly];  // polygon box in its own frame
      float const mp  = ix.max_offset[poly];
      // whole quadrant outside the polygon's box (beyond the tolerance)
      if (!exact) {
        float const qxmin = lf.uxmin - dx, qxmax = lf.uxmax - dx;
        float const qymin = lf.uymin - dy, qymax = lf.uymax - dy;
        float const mall  = fmaxf(fmaxf(mp, lf.m), fmaxf(fmaxf(fabsf(qxmin), fabsf(qxmax)),
                                                        fmaxf(fabsf(qymin), fabsf(qymax))));
        float const tol   = 4.76837158203125e-07f * mall;
        if (qxmax < bx.x - tol || qxmin > bx.z + tol || qymax < bx.y - tol ||
            qymin > bx.w + tol) {
          for (uint32_t w = lane; w < nw; w += 32) bits[wb + w] = 0u;
          if (lane == 0) counts[k] = 0;
          continue;
        }
      }
      float const invh     = ix.inv_slab_h32[poly];
      float const invw     = Ordered ? ix.inv_bin_w32[poly] : 0.0f;
      uint32_t const ns    = ix.num_slabs[poly];
      uint32_t const slab0 = ix.slab_base[poly];
      uint32_t const vb = ix.vert_begin[poly], ve = ix.vert_end[poly];
      for (uint32_t c = 0; c < len; c += 32) {
        uint64_t const pos = off + c + lane;
        bool hit           = false;
        if (c + lane < len && pos < npi) {
          // r: 0/1 decided, kUndecided: run the whole exact test
          int r       = kUndecided;
          bool have64 = false;
          double px64 = 0.0, py64 = 0.0;
          if (!exact) {
            float2 const uv = u[pos];
            float const qx = uv.x - dx, qy = uv.y - dy;
            float const m   = fmaxf(fmaxf(mp, lf.m), fmaxf(fabsf(qx), fabsf(qy)));
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
                  uint32_t const pi = point_indices[pos];
                  px64              = x[pi];
                  py64              = y[pi];
                  have64            = true;
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
                    uint32_t const pi = point_indices[pos];
                    px64              = x[pi];
                    py64              = y[pi];
                    have64            = true;
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
          }
          if (r == kUndecided) {
            ++nref;
            if (!have64) {
              uint32_t const pi = point_indices[pos];
              px64              = x[pi];
              py64              = y[pi];
            }
            hit = pip_exact<double>(px64, py64, ix, poly);
          } else {
            hit = r == 1;
          }
        }
        unsigned const w = __ballot_sync(0xFFFFFFFFu, hit);
        if (lane == 0) bits[wb + (c >> 5)] = w;
        cnt += __popc(w);
      }
    } else {
      for (uint32_t c = 0; c < len; c += 32) {
        uint64_t const pos = off + c + lane;
        bool hit           = false;
        if (c + lane < len && pos < npi) {
          uint32_t const pi = point_indices[pos];
          hit               = pip_exact<double>(x[pi], y[pi], ix, poly);
        }
        unsigned const w = __ballot_sync(0xFFFFFFFFu, hit);
        if (lane == 0) bits[wb + (c >> 5)] = w;
        cnt += __popc(w);
      }
    }
    if (lane == 0) counts[k] = cnt;
  }
  if (Filtered && refined) {
    for (int o = 16; o > 0; o >>= 1) nref += __shfl_xor_sync(0xFFFFFFFFu, nref, o);
    if (lane == 0 && nref) atomicAdd(refined, static_cast<unsigned long long>(nref));
  }
}

// float inputs: the reference's test in float, one warp per pair.
__global__ void __launch_bounds__(256)
  pip_pair_kernel_f32(uint32_t const* __restrict__ pair_poly,
                      uint32_t const* __restrict__ pair_quad, size_t npairs,
                      uint32_t const* __restrict__ qlen, uint32_t const* __restrict__ qoff,
                      uint32_t const* __restrict__ point_indices, size_t npi,
                      float const* __restrict__ x, float const* __restrict__ y,
                      PolygonIndexView<float> ix, uint64_t const* __restrict__ word_off,
                      uint32_t* __restrict__ bits, uint32_t* __restrict__ counts)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t k = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; k < npairs;
       k += warps) {
    uint32_t const poly = pair_poly[k];
    uint32_t const quad = pair_quad[k];
    uint32_t const len  = qlen[quad];
    uint64_t const off  = qoff[quad];
    uint64_t const wb   = word_off[k];
    uint32_t cnt        = 0;
    for (uint32_t c = 0; c < len; c += 32) {
      uint64_t const pos = off + c + lane;
      bool hit           = false;
      if (c + lane < len && pos < npi && poly < ix.num_polygons) {
        uint32_t const pi = point_indices[pos];
        hit               = pip_exact<float>(x[pi], y[pi], ix, poly);
      }
      unsigned const w = __ballot_sync(0xFFFFFFFFu, hit);
      if (lane == 0) bits[wb + (c >> 5)] = w;
      cnt += __popc(w);
    }
    if (lane == 0) counts[k] = cnt;
  }
}

__global__ void __launch_bounds__(256)
  pip_expand_kernel(uint32_t const* __restrict__ pair_poly, uint32_t const* __restrict__ pair_quad,
                    size_t npairs, uint32_t const* __restrict__ qlen,
                    uint32_t const* __restrict__ qoff, uint64_t const* __restrict__ word_off,
                    uint32_t const* __restrict__ bits, uint64_t const* __restrict__ out_off,
                    uint32_t* __restrict__ out_poly, uint32_t* __restrict__ out_point,
                    uint64_t cap)
{
  int const lane     = threadIdx.x & 31;
  unsigned const lt  = (1u << lane) - 1u;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t k = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; k < npairs;
       k += warps) {
    uint32_t const poly = pair_poly[k];
    uint32_t const len  = qlen[pair_quad[k]];
    uint32_t const off  = qoff[pair_quad[k]];
    uint64_t const wb   = word_off[k];
    uint64_t o          = out_off[k];
    for (uint32_t c = 0; c < len; c += 32) {
      unsigned const w = bits[wb + (c >> 5)];
      if (w == 0) continue;
      if (w & (1u << lane)) {
        uint64_t const d = o + __popc(w & lt);
        if (d < cap) {
          out_poly[d]  = poly;
          out_point[d] = off + c + lane;
        }
      }
      o += __popc(w);
    }
  }
}

template <typename T>
void run(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t npairs,
         cspt_quadtree const* tree, uint32_t const* point_indices, size_t npi, T const* x,
         T const* y, uint32_t const* po, size_t npo, uint32_t const* ro, size_t nro,
         T const* vx, T const* vy, size_t nv, cspt_method method, Allocator const& alloc,
         uint32_t** out_poly, uint32_t** out_point, size_t* out_n, uint64_t* out_refined)
{
  cudaStream_t const s = alloc.stream();
  bool const filtered  = method == CSPT_METHOD_FILTERED && std::is_same<T, double>::value;
  PolygonIndex<T> index(po, npo, ro, nro, vx, vy, nv, filtered, alloc);
  uint32_t const* qlen = tree->length;
  uint32_t const* qoff = tree->offset;

  // words of the bitmask per pair
  Buffer<uint64_t> word_off(alloc, npairs + 1);
  uint64_t* wo = word_off.data();
  scan_apply<uint64_t>(
    [pair_quad, qlen] __device__(size_t k) {
      return static_cast<uint64_t>((qlen[pair_quad[k]] + 31u) >> 5);
    },
    [wo] __device__(size_t k, uint64_t e, uint64_t) { wo[k] = e; }, npairs, wo + npairs, alloc);
  size_t const nwords = read_back(wo + npairs, s);
  Buffer<uint32_t> bits(alloc, nwords);
  Buffer<uint32_t> counts(alloc, npairs);
  Buffer<unsigned long long> refined(alloc, 2);  // [0] refined candidates, [1] next pair
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, 2 * sizeof(unsigned long long), s));
  unsigned const blk = 256;
  unsigned const grd = grid_for(npairs * 32, blk, 152u * 8u * 4u);
  if constexpr (std::is_same<T, double>::value) {
    Buffer<uint32_t> gstart, pgroup;
    Buffer<float2> u;
    Buffer<LeafFrame> frames;
    if (filtered) {
      // groups of consecutive pairs sharing a quadrant, and each pair's group
      gstart = Buffer<uint32_t>(alloc, npairs + 1);
      pgroup = Buffer<uint32_t>(alloc, npairs);
      uint32_t* gs = gstart.data();
      uint32_t* pg = pgroup.data();
      scan_apply<uint32_t>(
        [pair_quad] __device__(size_t k) {
          return (k == 0 || pair_quad[k] != pair_quad[k - 1]) ? 1u : 0u;
        },
        [gs, pg] __device__(size_t k, uint32_t e, uint32_t f) {
          if (f) gs[e] = static_cast<uint32_t>(k);
          pg[k] = e + f - 1u;
        },
        npairs, gs + npairs, alloc);
      u      = Buffer<float2>(alloc, npi);
      frames = Buffer<LeafFrame>(alloc, npairs);
      KernelTimer timer("leaf_frames", s);
      leaf_frame_kernel<<<grd, blk, 0, s>>>(gs, gs + npairs, pair_quad, qlen, qoff, point_indices,
                                            npi, x, y, index.view().grid, u.data(),
                                            frames.data());
      CSPT_CHECK_LAUNCH();
    }
    KernelTimer timer("pip_bits", s);
    if (filtered)
      pip_pair_kernel<true>
        <<<pair_grid(pip_pair_kernel<true>, kPipBlock, npairs), kPipBlock, 0, s>>>(
          pair_poly, pair_quad, pgroup.data(), npairs, qlen, qoff, point_indices, npi, x, y,
          u.data(), frames.data(), index.view(), word_off.data(), bits.data(), counts.data(),
          refined.data(), refined.data() + 1);
    else
      pip_pair_kernel<false>
        <<<pair_grid(pip_pair_kernel<false>, kPipBlock, npairs), kPipBlock, 0, s>>>(
          pair_poly, pair_quad, nullptr, npairs, qlen, qoff, point_indices, npi, x, y, nullptr,
          nullptr, index.view(), word_off.data(), bits.data(), counts.data(), nullptr,
          refined.data() + 1);
    CSPT_CHECK_LAUNCH();
  } else {
    KernelTimer timer("pip_bits", s);
    pip_pair_kernel_f32<<<grd, blk, 0, s>>>(pair_poly, pair_quad, npairs, qlen, qoff,
                                            point_indices, npi, x, y, index.view(),
                                            word_off.data(), bits.data(), counts.data());
    CSPT_CHECK_LAUNCH();
  }
  Buffer<uint64_t> out_off(alloc, npairs + 1);
  uint64_t* oo        = out_off.data();
  uint32_t const* cnt = counts.data();
  scan_apply<uint64_t>([cnt] __device__(size_t k) { return static_cast<uint64_t>(cnt[k]); },
                       [oo] __device__(size_t k, uint64_t e, uint64_t) { oo[k] = e; }, npairs,
                       oo + npairs, alloc);
  size_t const m = read_back(oo + npairs, s);
  if (out_refined) *out_refined = filtered ? read_back(refined.data(), s) : 0;
  *out_n = m;
  if (m == 0) return;
  Buffer<uint32_t> op(alloc, m), oq(alloc, m);
  {
    KernelTimer timer("pip_expand", s);
    pip_expand_kernel<<<grd, blk, 0, s>>>(pair_poly, pair_quad, npairs, qlen, qoff,
                                          word_off.data(), bits.data(), out_off.data(),
                                          op.data(), oq.data(), m);
    CSPT_CHECK_LAUNCH();
  }
  *out_poly  = op.release();
  *out_point = oq.release();
}

}  // namespace

// ---------------------------------------------------------------------------
// PipExec: a point-in-polygon evaluation over fixed pairs, tree and polygon
// index (float64).  The constructor plans and allocates (and synchronises);
// execute() only launches kernels into those buffers — no allocation, no
// host synchronisation — so it can be captured into a CUDA graph and
// replayed.  Outputs beyond the capacity are dropped and *overflow() tells.
// block_threads (a multiple of 32, at most 256) is the block size of the
// per-pair kernels; grids hold at most 256 warps per SM and stride beyond.
// ---------------------------------------------------------------------------
struct GroupOf {
  uint32_t const* pair_quad;
  __device__ uint32_t operator()(size_t k) const
  {
    return (k == 0 || pair_quad[k] != pair_quad[k - 1]) ? 1u : 0u;
  }
};
struct StoreGroups {
  uint32_t* gs;
  uint32_t* pg;
  __device__ void operator()(size_t k, uint32_t e, uint32_t f) const
  {
    if (f) gs[e] = static_cast<uint32_t>(k);
    pg[k] = e + f - 1u;
  }
};
struct WordsOf {
  uint32_t const* pair_quad;
  uint32_t const* qlen;
  __device__ uint64_t operator()(size_t k) const
  {
    return static_cast<uint64_t>((qlen[pair_quad[k]] + 31u) >> 5);
  }
};
struct CountsOf {
  uint32_t const* c;
  __device__ uint64_t operator()(size_t k) const { return c[k]; }
};
struct Store64 {
  uint64_t* p;
  __device__ void operator()(size_t k, uint64_t e, uint64_t) const { p[k] = e; }
};

__global__ void overflow_kernel(uint64_t const* total, uint64_t cap, int* flag)
{
  *flag = *total > cap ? 1 : 0;
}

class PipExec::Impl {
 public:
  Impl(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t npairs, uint32_t const* qlen,
       uint32_t const* qoff, uint32_t const* point_indices, size_t npi, double const* x,
       double const* y, PolygonIndexView<double> ix, bool filtered, unsigned block,
       Allocator const& alloc)
    : pp_(pair_poly), pq_(pair_quad), np_(npairs), qlen_(qlen), qoff_(qoff),
      pi_(point_indices), npi_(npi), x_(x), y_(y), ix_(ix), filtered_(filtered), blk_(block)
  {
    cudaStream_t const s = alloc.stream();
    size_t const parts   = (npairs + kScanTile - 1) / kScanTile + 1;
    word_off_ = Buffer<uint64_t>(alloc, npairs + 1);
    out_off_  = Buffer<uint64_t>(alloc, npairs + 1);
    partials_ = Buffer<uint64_t>(alloc, parts);
    gpart_    = Buffer<uint32_t>(alloc, parts);
    counts_   = Buffer<uint32_t>(alloc, npairs);
    gstart_   = Buffer<uint32_t>(alloc, npairs + 1);
    pgroup_   = Buffer<uint32_t>(alloc, npairs);
    frames_   = Buffer<LeafFrame>(alloc, npairs);
    u_        = Buffer<float2>(alloc, filtered ? npi : 0);
    refined_  = Buffer<unsigned long long>(alloc, 2);  // [0] refined, [1] next pair
    flag_     = Buffer<int>(alloc, 1);
    grid_true_    = pair_grid(pip_pair_kernel<true>, blk_, npairs);
    grid_ordered_ = pair_grid(pip_pair_kernel<true, true>, blk_, npairs);
    grid_false_ = pair_grid(pip_pair_kernel<false>, blk_, npairs);
    scan_apply_prealloc<uint64_t>(WordsOf{pair_quad, qlen}, Store64{word_off_.data()}, npairs,
                                  word_off_.data() + npairs, partials_.data(), s);
    nwords_ = read_back(word_off_.data() + npairs, s);
    bits_   = Buffer<uint32_t>(alloc, nwords_);
    scan_apply_prealloc<uint32_t>(GroupOf{pair_quad}, StoreGroups{gstart_.data(), pgroup_.data()},
                                  npairs, gstart_.data() + npairs, gpart_.data(), s);
  }

  // the bitmask, counts and output offsets of all pairs
  void evaluate(cudaStream_t s)
  {
    unsigned const blk = blk_;
    unsigned const grd = grid_for(np_ * 32, blk, 152u * 8u * 1024u / blk);
    CSPT_CUDA_TRY(cudaMemsetAsync(refined_.data(), 0, 2 * sizeof(unsigned long long), s));
    if (filtered_) {
      leaf_frame_kernel<<<grd, blk, 0, s>>>(gstart_.data(), gstart_.data() + np_, pq_, qlen_,
                                            qoff_, pi_, npi_, x_, y_, ix_.grid, u_.data(),
                                            frames_.data());
      CSPT_CHECK_LAUNCH();
      if (ix_.slab_nfull)
        pip_pair_kernel<true, true><<<grid_ordered_, blk, 0, s>>>(
          pp_, pq_, pgroup_.data(), np_, qlen_, qoff_, pi_, npi_, x_, y_, u_.data(),
          frames_.data(), ix_, word_off_.data(), bits_.data(), counts_.data(), refined_.data(),
          refined_.data() + 1);
      else
        pip_pair_kernel<true><<<grid_true_, blk, 0, s>>>(
          pp_, pq_, pgroup_.data(), np_, qlen_, qoff_, pi_, npi_, x_, y_, u_.data(),
          frames_.data(), ix_, word_off_.data(), bits_.data(), counts_.data(), refined_.data(),
          refined_.data() + 1);
    } else {
      pip_pair_kernel<false><<<grid_false_, blk, 0, s>>>(
        pp_, pq_, nullptr, np_, qlen_, qoff_, pi_, npi_, x_, y_, nullptr, nullptr, ix_,
        word_off_.data(), bits_.data(), counts_.data(), nullptr, refined_.data() + 1);
    }
    CSPT_CHECK_LAUNCH();
    scan_apply_prealloc<uint64_t>(CountsOf{counts_.data()}, Store64{out_off_.data()}, np_,
                                  out_off_.data() + np_, partials_.data(), s);
  }

  // writes the rows of the last evaluation to op/oq, up to cap entries
  void expand(cudaStream_t s, uint32_t* op, uint32_t* oq, uint64_t cap)
  {
    unsigned const blk = blk_;
    unsigned const grd = grid_for(np_ * 32, blk, 152u * 8u * 1024u / blk);
    pip_expand_kernel<<<grd, blk, 0, s>>>(pp_, pq_, np_, qlen_, qoff_, word_off_.data(),
                                          bits_.data(), out_off_.data(), op, oq, cap);
    CSPT_CHECK_LAUNCH();
    overflow_kernel<<<1, 1, 0, s>>>(out_off_.data() + np_, cap, flag_.data());
    CSPT_CHECK_LAUNCH();
  }

  void execute(cudaStream_t s, uint32_t* op, uint32_t* oq, uint64_t cap)
  {
    evaluate(s);
    expand(s, op, oq, cap);
  }

  uint64_t const* total() const { return out_off_.data() + np_; }
  uint64_t const* pair_out_offsets() const { return out_off_.data(); }
  int const* overflow() const { return flag_.data(); }
  unsigned long long const* refined() const { return refined_.data(); }

 private:
  uint32_t const *pp_, *pq_;
  size_t np_;
  uint32_t const *qlen_, *qoff_, *pi_;
  size_t npi_;
  double const *x_, *y_;
  PolygonIndexView<double> ix_;
  bool filtered_;
  unsigned blk_;
  unsigned grid_true_ = 1, grid_false_ = 1, grid_ordered_ = 1;
  size_t nwords_ = 0;
  Buffer<uint64_t> word_off_, out_off_, partials_;
  Buffer<uint32_t> gpart_, counts_, gstart_, pgroup_, bits_;
  Buffer<LeafFrame> frames_;
  Buffer<float2> u_;
  Buffer<unsigned long long> refined_;
  Buffer<int> flag_;
};

PipExec::PipExec(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t npairs,
                 uint32_t const* qlen, uint32_t const* qoff, uint32_t const* point_indices,
                 size_t npi, double const* x, double const* y, PolygonIndexView<double> const& ix,
                 bool filtered, unsigned block_threads, Allocator const& alloc)
  : impl_(new Impl(pair_poly, pair_quad, npairs, qlen, qoff, point_indices, npi, x, y, ix,
                   filtered, block_threads, alloc))
{
}
PipExec::~PipExec() { delete impl_; }
void PipExec::execute(cudaStream_t s, uint32_t* op, uint32_t* oq, uint64_t cap)
{
  impl_->execute(s, op, oq, cap);
}
void PipExec::evaluate(cudaStream_t s) { impl_->evaluate(s); }
void PipExec::expand(cudaStream_t s, uint32_t* op, uint32_t* oq, uint64_t cap)
{
  impl_->expand(s, op, oq, cap);
}
uint64_t const* PipExec::total() const { return impl_->total(); }
uint64_t const* PipExec::pair_out_offsets() const { return impl_->pair_out_offsets(); }
int const* PipExec::overflow() const { return impl_->overflow(); }
unsigned long long const* PipExec::refined() const { return impl_->refined(); }

void quadtree_point_in_polygon(uint32_t const* pair_poly, uint32_t const* pair_quad,
                               size_t npairs, cspt_quadtree const* tree,
                               uint32_t const* point_indices, size_t npi, void const* x,
                               void const* y, uint32_t const* po, size_t npo, uint32_t const* ro,
                               size_t nro, void const* vx, void const* vy, size_t nv,
                               cspt_dtype dtype, cspt_method method, Allocator const& alloc,
                               uint32_t** out_poly, uint32_t** out_point, size_t* out_n,
                               uint64_t* out_refined)
{
  if (dtype == CSPT_FLOAT64)
    run<double>(pair_poly, pair_quad, npairs, tree, point_indices, npi,
                static_cast<double const*>(x), static_cast<double const*>(y), po, npo, ro, nro,
                static_cast<double const*>(vx), static_cast<double const*>(vy), nv, method, alloc,
                out_poly, out_point, out_n, out_refined);
  else
    run<float>(pair_poly, pair_quad, npairs, tree, point_indices, npi,
               static_cast<float const*>(x), static_cast<float const*>(y), po, npo, ro, nro,
               static_cast<float const*>(vx), static_cast<float const*>(vy), nv, method, alloc,
               out_poly, out_point, out_n, out_refined);
}

}  // namespace cspt
