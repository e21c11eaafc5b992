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
#include <functional>
#include <memory>

#include "common.cuh"
#include "leaf_frame.cuh"
#include "pip_test.cuh"
#include "polygon_index.cuh"
#include "scan.cuh"

namespace cspt {

uint64_t& last_edge_free_pairs()
{
  static thread_local uint64_t n = 0;
  return n;
}

namespace {

constexpr int kPipBlock = 256;
// chunks of pairs when the rows go to host memory (copies overlap the next chunk)
#ifndef CSPT_HOST_CHUNKS
#define CSPT_HOST_CHUNKS 8
#endif
constexpr size_t kHostChunks = CSPT_HOST_CHUNKS;
// the quadrant fast path: list entries per warp (the y-only list grows up
// from the start of the pool, the full list down from its end), slabs per
// quadrant
#ifndef CSPT_FAST_POOL
#define CSPT_FAST_POOL 128
#endif
constexpr uint32_t kFastPool  = CSPT_FAST_POOL;
constexpr uint32_t kFastSlabs = 31;
// the edge-free quadrant test streams at most this many slab entries
constexpr uint32_t kFreeScan = 1024;

// The float32 slab of offset y (the lookup of filtered_test).
__device__ inline uint32_t slab_lookup(float qy, float y0, float invh, uint32_t ns)
{
  float const fs = (qy - y0) * invh;
  uint32_t sj    = 0;
  if (fs > 0.0f) sj = fs >= static_cast<float>(ns) ? ns - 1 : static_cast<uint32_t>(fs);
  return sj >= ns ? ns - 1 : sj;
}
// Blocks of 256 threads per SM for the leaf frames (the index fill that runs
// beside them takes what the frames leave; 2-8 measured within 1%).
#ifndef CSPT_LEAF_BLOCKS_PER_SM
#define CSPT_LEAF_BLOCKS_PER_SM 8
#endif
inline unsigned leaf_frame_grid(size_t npairs)
{
  return grid_for(npairs * 32, 256, static_cast<unsigned>(num_sms()) * CSPT_LEAF_BLOCKS_PER_SM);
}
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
                  PointSource<double> const src, size_t npi,
                  float2 const* __restrict__ u, LeafFrame const* __restrict__ frames,
                  PolygonIndexView<double> ix, uint64_t const* __restrict__ word_off,
                  uint32_t* __restrict__ bits, uint32_t* __restrict__ counts,
                  unsigned long long* __restrict__ refined,
                  unsigned long long* __restrict__ next_pair,
                  unsigned long long* __restrict__ stats)
{
  int const lane      = threadIdx.x & 31;
  int const wid       = threadIdx.x >> 5;
  // the quadrant fast path's edge lists, per warp: entry (the edge, or the
  // y-only list's two y values), its slab entry index and its slab
  __shared__ float4 s_pool[kPipBlock / 32][kFastPool];
  __shared__ uint32_t s_poolk[kPipBlock / 32][kFastPool];
  __shared__ uint8_t s_pools[kPipBlock / 32][kFastPool];
  __shared__ uint8_t s_pbeg[kPipBlock / 32][kFastSlabs + 1];
  __shared__ uint8_t s_fbeg[kPipBlock / 32][kFastSlabs + 1];
  __shared__ uint32_t s_start[kPipBlock / 32][kFastSlabs + 1];
  __shared__ uint32_t s_base[kPipBlock / 32];
  float const gf      = Filtered ? static_cast<float>(*ix.grid) : 0.0f;
  bool const gok      = gf >= 1.17549435e-38f && gf < 1.0e30f;  // normal float grid step
  uint32_t nref       = 0;
  uint32_t nfree      = 0;  // pairs decided by the edge-free test
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
      // the quadrant's points in the polygon's frame lie in this box
      float const qxmin = lf.uxmin - dx, qxmax = lf.uxmax - dx;
      float const qymin = lf.uymin - dy, qymax = lf.uymax - dy;
      float const mall  = fmaxf(fmaxf(mp, lf.m), fmaxf(fmaxf(fabsf(qxmin), fabsf(qxmax)),
                                                      fmaxf(fabsf(qymin), fabsf(qymax))));
      float const tol   = 4.76837158203125e-07f * mall;  // 2^-21 M
      // whole quadrant outside the polygon's box (beyond the tolerance)
      if (!exact && (qxmax < bx.x - tol || qxmin > bx.z + tol || qymax < bx.y - tol ||
                     qymin > bx.w + tol)) {
        for (uint32_t w = lane; w < nw; w += 32) bits[wb + w] = 0u;
        if (lane == 0) counts[k] = 0;
        continue;
      }
      float const invh     = ix.inv_slab_h32[poly];
      float const invw     = Ordered ? ix.inv_bin_w32[poly] : 0.0f;
      uint32_t const ns    = ix.num_slabs[poly];
      uint32_t const slab0 = ix.slab_base[poly];
      uint32_t const vb = ix.vert_begin[poly], ve = ix.vert_end[poly];
      // Quadrant-level edge classification.  Each point's float32 slab
      // lookup is monotone in y, so the quadrant's points fall in slabs
      // j0..j1 and those of slab j in a band of y (the slab's extent widened
      // by the lookup error, 1/32 slab, and tol, and clipped to the box).
      // Per slab the warp classifies the slab's edges once against the box
      // [qxmin, qxmax] x band, with the filter's margins:
      //   x entirely left of the box, or y entirely above / below the band:
      //     never toggles, never on the edge;
      //   x entirely right and y across the whole band: toggles for every
      //     point of the slab (the crossing is right of the point by more
      //     than tol and the edge rises by more than 2 tol, so the
      //     reference's float64 comparison is decided) -> a common parity;
      //   x entirely right, y partly: the toggle is the y-flags test alone;
      //   x overlapping the box: the full per-point test.
      // Exactly vertical edges keep their x-only check (the vertical list).
      // (the ordered index, used by plans evaluated many times, keeps its
      // per-bin windows: its launches use small blocks that these per-warp
      // lists would starve of occupancy)
      bool fast = false, vcheck = false;
      uint32_t base = 0, j0 = 0, jspan = 0, npart_all = 0;
      if constexpr (!Ordered) {
        if (!exact && mall * invh <= 16384.0f) {
          j0                  = slab_lookup(qymin, bx.y, invh, ns);
          uint32_t const j1   = slab_lookup(qymax, bx.y, invh, ns);
          jspan               = j1 - j0;
          // Edge-free quadrant.  When no edge's box, widened by tol, meets
          // the quadrant's point box [qxmin, qxmax] x [qymin, qymax] and no
          // exactly vertical edge lies within tol of its x-range, every
          // point of the quadrant gets the reference's result of any one of
          // them: no point can be on an edge (each edge is more than tol
          // from it in x or in y); edges left of, above or below the box
          // never toggle; an edge right of the box toggles exactly when its
          // y-range holds the point's y, and as y moves through the box that
          // changes only at a vertex right of the box, whose two ring
          // neighbours are then both right of the box (an edge through such
          // a vertex and within the box's y-range can be neither left,
          // above, below nor meeting the box) and flip together.  So the
          // crossing parity is the same for the whole box: the quadrant's
          // first point is tested over its slab (float32 per edge, the
          // reference's float64 for undecided edges) and its result fills
          // every word.
          {
            uint32_t const E0 = ix.slab_start[slab0 + j0];
            uint32_t const E1 = ix.slab_start[slab0 + j1 + 1];
            bool meets        = E1 - E0 > kFreeScan || len == 0 || off >= npi;
            for (uint32_t t0 = E0; t0 < E1 && !meets; t0 += 32) {
              uint32_t const kk = t0 + lane;
              bool m            = false;
              if (kk < E1) {
                float4 const e = ix.slab_e32[kk];
                m = !(fmaxf(e.x, e.z) < qxmin - tol || fminf(e.x, e.z) > qxmax + tol ||
                      fmaxf(e.y, e.w) < qymin - tol || fminf(e.y, e.w) > qymax + tol);
              }
              meets = __any_sync(0xFFFFFFFFu, m);
            }
            if (!meets && vb < ve) {
              uint32_t lo = vb, hi = ve;
              float const key = qxmin - tol;
              while (lo < hi) {
                uint32_t const mid = (lo + hi) >> 1;
                if (ix.vert_x32[mid] < key)
                  lo = mid + 1;
                else
                  hi = mid;
              }
              meets = lo < ve && ix.vert_x32[lo] <= qxmax + tol;
            }
            if (!meets) {
              float2 const uv   = u[off];
              float const qx    = uv.x - dx, qy = uv.y - dy;
              float const eb    = __fmaf_rn(7.62939453125e-06f * mall, mall, 7.52316384526264e-37f);
              uint32_t const jr = slab_lookup(qy, bx.y, invh, ns);
              uint32_t const R0 = ix.slab_start[slab0 + jr];
              uint32_t const R1 = ix.slab_start[slab0 + jr + 1];
              unsigned par      = 0u;
              bool on           = false;
              for (uint32_t t0 = R0; t0 < R1; t0 += 32) {
                uint32_t const kk = t0 + lane;
                bool tg = false, oe = false;
                if (kk < R1) {
                  float4 const e = ix.slab_e32[kk];
                  float const ya = e.y - qy, yb = e.w - qy;
                  bool const y1  = ya > 0.0f;
                  bool const y0  = yb > 0.0f;
                  float const cr = __fmaf_rn(qx - e.x, e.w - e.y, -((e.z - e.x) * (qy - e.y)));
                  bool const undecided =
                    fabsf(ya) <= tol || fabsf(yb) <= tol ||
                    (fabsf(cr) <= eb &&
                     (y1 != y0 || !(qx < fminf(e.x, e.z) - tol || qx > fmaxf(e.x, e.z) + tol)));
                  if (!undecided) {
                    tg = y1 != y0 && ((cr < 0.0f) != y1);
                  } else {
                    ++nref;
                    double px64, py64;
                    src.load(off, px64, py64);
                    uint32_t const v  = ix.slab_edges[kk] & kEntryVertex;
                    uint32_t const pv = ix.prev_vertex[v];
                    int const ee =
                      exact_edge<double>(px64, py64, ix.vx[v], ix.vy[v], ix.vx[pv], ix.vy[pv]);
                    oe = ee == 2;
                    tg = ee == 1;
                  }
                }
                par ^= __ballot_sync(0xFFFFFFFFu, tg);
                on = __any_sync(0xFFFFFFFFu, oe) || on;
              }
              if (!on) {
                // (an on-edge representative contradicts the premise; such a
                // pair takes the paths below)
                bool const all      = (__popc(par) & 1u) != 0u;
                uint64_t const vmax = npi - off < len ? npi - off : len;
                for (uint32_t w = lane; w < nw; w += 32) {
                  uint64_t const b0 = static_cast<uint64_t>(w) * 32u;
                  uint32_t word     = 0u;
                  if (all && vmax > b0)
                    word = vmax - b0 >= 32 ? 0xFFFFFFFFu : (1u << (vmax - b0)) - 1u;
                  bits[wb + w] = word;
                }
                if (lane == 0) counts[k] = all ? static_cast<uint32_t>(vmax) : 0u;
                ++nfree;
                continue;
              }
            }
          }
          if (jspan < kFastSlabs) {
            fast              = true;
            float const hs    = invh > 0.0f ? 1.0f / invh : 0.0f;
            float const dlt   = tol + 0.03125f * hs;
            unsigned const lt = (1u << lane) - 1u;
            // the entries of slabs j0..j1 are contiguous: their starts
            // (jspan + 2 <= 32 values) bound one stream of entries
            uint32_t const st = lane <= jspan + 1 ? ix.slab_start[slab0 + j0 + lane] : 0u;
            if (lane <= jspan + 1) s_start[wid][lane] = st;
            if (lane == 0) s_base[wid] = 0u;
            uint32_t const E0 = __shfl_sync(0xFFFFFFFFu, st, 0);
            uint32_t const E1 = __shfl_sync(0xFFFFFFFFu, st, static_cast<int>(jspan + 1));
            __syncwarp();
            uint32_t npart = 0, nfull = 0;
            for (uint32_t t0 = E0; t0 < E1; t0 += 32) {
              uint32_t const kk = t0 + lane;
              bool const has    = kk < E1;
              // the entry's slab: the last start <= kk
              uint32_t lo = 0, hi = jspan + 1;
              while (hi - lo > 1) {
                uint32_t const mid = (lo + hi) >> 1;
                if (s_start[wid][mid] <= kk)
                  lo = mid;
                else
                  hi = mid;
              }
              uint32_t const jj = lo, j = j0 + lo;
              float const ylo = j == 0 ? qymin : fmaxf(qymin, __fmaf_rn(static_cast<float>(j), hs, bx.y) - dlt);
              float const yhi = j + 1 >= ns ? qymax
                                            : fminf(qymax, __fmaf_rn(static_cast<float>(j + 1), hs, bx.y) + dlt);
              float4 const e    = has ? ix.slab_e32[kk] : make_float4(0.f, 0.f, 0.f, 0.f);
              float const exmin = fminf(e.x, e.z), exmax = fmaxf(e.x, e.z);
              float const eymin = fminf(e.y, e.w), eymax = fmaxf(e.y, e.w);
              int cls = 0;  // 0 none, 1 every point, 2 y-test, 3 full test
              if (has && !(exmax < qxmin - tol) && !(eymin > yhi + tol || eymax < ylo - tol)) {
                if (exmin > qxmax + tol)
                  cls = (eymin < ylo - tol && eymax > yhi + tol) ? 1 : 2;
                else
                  cls = 3;
              }
              if (cls == 1) atomicXor(&s_base[wid], 1u << jj);
              unsigned const bp = __ballot_sync(0xFFFFFFFFu, cls == 2);
              unsigned const bf = __ballot_sync(0xFFFFFFFFu, cls == 3);
              if (npart + nfull + __popc(bp) + __popc(bf) > kFastPool) {
                fast = false;
                break;
              }
              // lanes hold increasing entries, so the lists stay in slab order
              // (the full list's i-th entry sits at kFastPool - 1 - i)
              if (cls == 2) {
                uint32_t const slot = npart + __popc(bp & lt);
                s_pool[wid][slot]   = make_float4(e.y, e.w, 0.0f, 0.0f);
                s_poolk[wid][slot]  = kk;
                s_pools[wid][slot]  = static_cast<uint8_t>(jj);
              }
              if (cls == 3) {
                uint32_t const slot = kFastPool - 1u - (nfull + __popc(bf & lt));
                s_pool[wid][slot]   = e;
                s_poolk[wid][slot]  = kk;
                s_pools[wid][slot]  = static_cast<uint8_t>(jj);
              }
              npart += __popc(bp);
              nfull += __popc(bf);
            }
            __syncwarp();
            if (fast) {
              // each slab's list range: lane jj counts the entries of lower
              // slabs (the lists are sorted by slab)
              if (lane <= jspan + 1) {
                uint32_t lo = 0, hi = npart;
                while (lo < hi) {
                  uint32_t const mid = (lo + hi) >> 1;
                  if (s_pools[wid][mid] < static_cast<uint32_t>(lane))
                    lo = mid + 1;
                  else
                    hi = mid;
                }
                s_pbeg[wid][lane] = static_cast<uint8_t>(lo);
                lo = 0;
                hi = nfull;
                while (lo < hi) {
                  uint32_t const mid = (lo + hi) >> 1;
                  if (s_pools[wid][kFastPool - 1u - mid] < static_cast<uint32_t>(lane))
                    lo = mid + 1;
                  else
                    hi = mid;
                }
                s_fbeg[wid][lane] = static_cast<uint8_t>(lo);
              }
              __syncwarp();
              base      = s_base[wid];
              npart_all = npart + nfull;
            }
            if (fast && vb < ve) {
              // a vertical edge within tol of the box's x-range
              uint32_t lo = vb, hi = ve;
              float const key = qxmin - tol;
              while (lo < hi) {
                uint32_t const mid = (lo + hi) >> 1;
                if (ix.vert_x32[mid] < key)
                  lo = mid + 1;
                else
                  hi = mid;
              }
              vcheck = lo < ve && ix.vert_x32[lo] <= qxmax + tol;
            }
          }
        }
      }
      if (fast && npart_all == 0 && !vcheck) {
        uint32_t const mask = (2u << jspan) - 1u;
        if ((base & mask) == 0u || (base & mask) == mask) {
          // no edge reaches the quadrant's band: every point has the slabs'
          // common parity, the words are written without reading a point
          bool const all      = (base & mask) != 0u;
          uint64_t const vmax = off >= npi ? 0 : (npi - off < len ? npi - off : len);
          for (uint32_t w = lane; w < nw; w += 32) {
            uint64_t const b0 = static_cast<uint64_t>(w) * 32u;
            uint32_t word     = 0u;
            if (all && vmax > b0) word = vmax - b0 >= 32 ? 0xFFFFFFFFu : (1u << (vmax - b0)) - 1u;
            bits[wb + w] = word;
          }
          __syncwarp();
          if (lane == 0) counts[k] = all ? static_cast<uint32_t>(vmax) : 0u;
          continue;
        }
      }
      if (fast) {
        float const eb = __fmaf_rn(7.62939453125e-06f * mall, mall, 7.52316384526264e-37f);
        for (uint32_t c = 0; c < len; c += 32) {
          uint64_t const pos = off + c + lane;
          bool hit           = false;
          if (c + lane < len && pos < npi) {
            float2 const uv = u[pos];
            float const qx = uv.x - dx, qy = uv.y - dy;
            // in [0, jspan]: the lookup is monotone and qy lies in the box
            uint32_t const jj = min(slab_lookup(qy, bx.y, invh, ns) - j0, jspan);
            bool within       = (base >> jj) & 1u;
            uint32_t const pb = s_pbeg[wid][jj], pe = s_pbeg[wid][jj + 1];
            uint32_t const fb = s_fbeg[wid][jj], fe = s_fbeg[wid][jj + 1];
            bool on_edge   = false;
            bool have64    = false;
            double px64 = 0.0, py64 = 0.0;
            auto load = [&] {
              if (!have64) {
                src.load(pos, px64, py64);
                have64 = true;
              }
            };
            auto exact_at = [&](uint32_t kk) {
              ++nref;
              load();
              uint32_t const v  = ix.slab_edges[kk] & kEntryVertex;
              uint32_t const pv = ix.prev_vertex[v];
              return exact_edge<double>(px64, py64, ix.vx[v], ix.vy[v], ix.vx[pv], ix.vy[pv]);
            };
            if (vcheck) {
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
                load();
                on_edge = sorted_has<double>(ix.vert_x, vb, ve, px64);
              }
            }
            for (uint32_t t = pb; t < pe && !on_edge; ++t) {
              float2 const yy = *reinterpret_cast<float2 const*>(&s_pool[wid][t]);
              float const ya = yy.x - qy, yb = yy.y - qy;
              if (fabsf(ya) <= tol || fabsf(yb) <= tol) {
                int const ee = exact_at(s_poolk[wid][t]);
                if (ee == 2) on_edge = true;
                if (ee == 1) within = !within;
              } else if ((ya > 0.0f) != (yb > 0.0f)) {
                within = !within;
              }
            }
            for (uint32_t t = fb; t < fe && !on_edge; ++t) {
              float4 const e = s_pool[wid][kFastPool - 1u - t];
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
              int const ee = exact_at(s_poolk[wid][kFastPool - 1u - t]);
              if (ee == 2) on_edge = true;
              if (ee == 1) within = !within;
            }
            hit = within && !on_edge;
          }
          unsigned const w = __ballot_sync(0xFFFFFFFFu, hit);
          if (lane == 0) bits[wb + (c >> 5)] = w;
          cnt += __popc(w);
        }
        __syncwarp();  // the next pair rewrites this warp's edge lists
        if (lane == 0) counts[k] = cnt;
        continue;
      }
      for (uint32_t c = 0; c < len; c += 32) {
        uint64_t const pos = off + c + lane;
        bool hit           = false;
        if (c + lane < len && pos < npi) {
          if (!exact) {
            float2 const uv = u[pos];
            hit = filtered_test<Ordered>(
              ix, poly, uv.x - dx, uv.y - dy, mp, lf.m, bx, invh, invw, ns, slab0, vb, ve,
              [&](double& px, double& py) { src.load(pos, px, py); },
              nref);
          } else {
            ++nref;
            double px, py;
            src.load(pos, px, py);
            hit = pip_exact<double>(px, py, ix, poly);
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
          double px, py;
          src.load(pos, px, py);
          hit = pip_exact<double>(px, py, ix, poly);
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
    if (lane == 0 && nfree) atomicAdd(stats, static_cast<unsigned long long>(nfree));
  }
}

// float inputs: the reference's test in float, one warp per pair.
__global__ void __launch_bounds__(256)
  pip_pair_kernel_f32(uint32_t const* __restrict__ pair_poly,
                      uint32_t const* __restrict__ pair_quad, size_t npairs,
                      uint32_t const* __restrict__ qlen, uint32_t const* __restrict__ qoff,
                      PointSource<float> const src, size_t npi, PolygonIndexView<float> ix, uint64_t const* __restrict__ word_off,
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
        float px, py;
        src.load(pos, px, py);
        hit = pip_exact<float>(px, py, ix, poly);
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
                    uint64_t cap, uint32_t const* __restrict__ id_map)
{
  // A warp takes 32 consecutive pairs at a time: lane j loads pair j's
  // header, and each pair's bitmask words are loaded 32 at a time, one per
  // lane, then broadcast word by word, so the loads of a batch are issued
  // together instead of one dependent load per word.
  int const lane     = threadIdx.x & 31;
  unsigned const lt  = (1u << lane) - 1u;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t k0 = ((blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5) * 32;
       k0 < npairs; k0 += warps * 32) {
    size_t const kl     = k0 + lane;
    bool const have     = kl < npairs;
    uint32_t const q    = have ? pair_quad[kl] : 0u;
    uint32_t const hp   = have ? pair_poly[kl] : 0u;
    uint32_t const hlen = have ? qlen[q] : 0u;
    uint32_t const hoff = have ? qoff[q] : 0u;
    uint64_t const hwb  = have ? word_off[kl] : 0u;
    uint64_t const ho   = have ? out_off[kl] : 0u;
    uint32_t const nk   = npairs - k0 < 32 ? static_cast<uint32_t>(npairs - k0) : 32u;
    for (uint32_t j = 0; j < nk; ++j) {
      uint32_t const poly = __shfl_sync(0xFFFFFFFFu, hp, j);
      uint32_t const len  = __shfl_sync(0xFFFFFFFFu, hlen, j);
      uint32_t const off  = __shfl_sync(0xFFFFFFFFu, hoff, j);
      uint64_t const wb   = __shfl_sync(0xFFFFFFFFu, hwb, j);
      uint64_t o          = __shfl_sync(0xFFFFFFFFu, ho, j);
      uint32_t const nw   = (len + 31u) >> 5;
      for (uint32_t w0 = 0; w0 < nw; w0 += 32) {
        uint32_t const cnt  = nw - w0 < 32u ? nw - w0 : 32u;
        unsigned const mine = static_cast<uint32_t>(lane) < cnt ? bits[wb + w0 + lane] : 0u;
        for (uint32_t c = 0; c < cnt; ++c) {
          unsigned const w = __shfl_sync(0xFFFFFFFFu, mine, c);
          if (w == 0) continue;
          if (w & (1u << lane)) {
            uint64_t const d = o + __popc(w & lt);
            if (d < cap) {
              uint32_t const pos = off + ((w0 + c) << 5) + lane;
              out_poly[d]        = poly;
              out_point[d]       = id_map ? id_map[pos] : pos;
            }
          }
          o += __popc(w);
        }
      }
    }
  }
}

template <typename T>
void run(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t npairs,
         cspt_quadtree const* tree, uint32_t const* point_indices, size_t npi, T const* x,
         T const* y, uint32_t const* po, size_t npo, uint32_t const* ro, size_t nro,
         T const* vx, T const* vy, size_t nv, cspt_method method, Allocator const& alloc,
         uint32_t** out_poly, uint32_t** out_point, size_t* out_n, uint64_t* out_refined,
         HostRows const* host, T const* ordered, PolygonIndex<T>* prebuilt = nullptr,
         uint32_t const* id_map = nullptr)
{
  cudaStream_t const s = alloc.stream();
  PointSource<T> const src{point_indices, x, y, ordered};
  bool const filtered  = method == CSPT_METHOD_FILTERED && std::is_same<T, double>::value;
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
  Buffer<uint32_t> counts(alloc, npairs);
  // [0] refined candidates, [1] next pair, [2] pairs decided by the
  // edge-free test
  Buffer<unsigned long long> refined(alloc, 3);
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, 3 * sizeof(unsigned long long), s));
  unsigned const blk = 256;
  // filtered: groups of consecutive pairs sharing a quadrant, each pair's
  // group, and the leaf frames (float32 point offsets from the quadrant's
  // anchor), which need only the index's anchor grid
  Buffer<uint32_t> gstart, pgroup;
  Buffer<float2> u;
  Buffer<LeafFrame> frames;
  if (filtered) {
    gstart       = Buffer<uint32_t>(alloc, npairs + 1);
    pgroup       = Buffer<uint32_t>(alloc, npairs);
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
  }
  // The leaf frames (bound by HBM) run on a second stream while the index
  // writes its slab entries: they start once everything enqueued above,
  // the index's sizing pass and anchor grid included, is complete, and `join`
  // (destroyed before the index and the buffers above, also on an
  // exception) orders the rest of the call after them.  Nothing here waits
  // on the host.
  // (a prebuilt index, filled, may come with the call)
  std::unique_ptr<PolygonIndex<T>> own;
  if (!prebuilt)
    own.reset(new PolygonIndex<T>(po, npo, ro, nro, vx, vy, nv, filtered, alloc, false, filtered));
  PolygonIndex<T>& index  = prebuilt ? *prebuilt : *own;
  cudaStream_t const side = filtered ? side_stream() : nullptr;
  StreamJoin join(s, side);
  if constexpr (std::is_same<T, double>::value) {
    if (filtered) {
      stream_wait(side, s);
      KernelTimer timer("leaf_frames", side);
      leaf_frame_kernel<<<leaf_frame_grid(npairs), blk, 0, side>>>(
        gstart.data(), gstart.data() + npairs, pair_quad, qlen, qoff, src, npi, index.grid(),
        u.data(), frames.data());
      CSPT_CHECK_LAUNCH();
    }
  }
  if (!prebuilt) index.fill();
  join.join();
  // the bitmask's size: the one read-back before the evaluation, taken once
  // the index and the frames are queued, so the device stays busy meanwhile
  size_t const nwords = read_back(wo + npairs, s);
  Buffer<uint32_t> bits(alloc, nwords);
  // hit bitmask and per-pair counts of pairs [k0, k0 + n) (the pair
  // arrays are offset; word offsets and group ids stay absolute)
  auto evaluate = [&](size_t k0, size_t n) {
    KernelTimer timer("pip_bits", s);
    if constexpr (std::is_same<T, double>::value) {
      CSPT_CUDA_TRY(cudaMemsetAsync(refined.data() + 1, 0, sizeof(unsigned long long), s));
      if (filtered)
        pip_pair_kernel<true><<<pair_grid(pip_pair_kernel<true>, kPipBlock, n), kPipBlock, 0, s>>>(
          pair_poly + k0, pair_quad + k0, pgroup.data() + k0, n, qlen, qoff, src, npi, u.data(),
          frames.data(), index.view(), word_off.data() + k0, bits.data(), counts.data() + k0,
          refined.data(), refined.data() + 1, refined.data() + 2);
      else
        pip_pair_kernel<false>
          <<<pair_grid(pip_pair_kernel<false>, kPipBlock, n), kPipBlock, 0, s>>>(
            pair_poly + k0, pair_quad + k0, nullptr, n, qlen, qoff, src, npi, nullptr, nullptr,
            index.view(), word_off.data() + k0, bits.data(), counts.data() + k0, nullptr,
            refined.data() + 1, refined.data() + 2);
    } else {
      pip_pair_kernel_f32<<<grid_for(n * 32, blk, sm_grid(8u * 4u)), blk, 0, s>>>(
        pair_poly + k0, pair_quad + k0, n, qlen, qoff, src, npi, index.view(),
        word_off.data() + k0, bits.data(), counts.data() + k0);
    }
    CSPT_CHECK_LAUNCH();
  };
  // row offsets of pairs [k0, k0 + n) from their counts; returns the rows
  auto row_offsets = [&](size_t k0, size_t n, Buffer<uint64_t>& out_off) {
    out_off             = Buffer<uint64_t>(alloc, n + 1);
    uint64_t* oo        = out_off.data();
    uint32_t const* cnt = counts.data() + k0;
    scan_apply<uint64_t>([cnt] __device__(size_t k) { return static_cast<uint64_t>(cnt[k]); },
                         [oo] __device__(size_t k, uint64_t e, uint64_t) { oo[k] = e; }, n,
                         oo + n, alloc);
    return static_cast<size_t>(read_back(oo + n, s));
  };
  auto expand = [&](size_t k0, size_t n, Buffer<uint64_t> const& out_off, uint32_t* op,
                    uint32_t* oq, size_t m) {
    KernelTimer timer("pip_expand", s);
    pip_expand_kernel<<<grid_for(n, blk, sm_grid(8u * 4u)), blk, 0, s>>>(
      pair_poly + k0, pair_quad + k0, n, qlen, qoff, word_off.data() + k0, bits.data(),
      out_off.data(), op, oq, m, id_map);
    CSPT_CHECK_LAUNCH();
  };

  // the kernel's counters (read once the stream is idle)
  auto finish_counts = [&] {
    unsigned long long h[3] = {0, 0, 0};
    CSPT_CUDA_TRY(cudaMemcpyAsync(h, refined.data(), sizeof(h), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    if (out_refined) *out_refined = filtered ? h[0] : 0;
    last_edge_free_pairs() = filtered ? h[2] : 0;
  };
  if (!host) {
    evaluate(0, npairs);
    Buffer<uint64_t> out_off;
    size_t const m = row_offsets(0, npairs, out_off);
    finish_counts();
    *out_n = m;
    if (m == 0) return;
    Buffer<uint32_t> op(alloc, m), oq(alloc, m);
    expand(0, npairs, out_off, op.data(), oq.data(), m);
    *out_poly  = op.release();
    *out_point = oq.release();
    return;
  }

  // Host output: the pairs are evaluated in chunks, and each chunk's rows are
  // copied to the host on a second stream while the next chunk is evaluated.
  // The staged rows stay allocated until `copies` has joined.
  std::vector<Buffer<uint32_t>> staged;
  cudaStream_t const copy = side_stream();
  StreamJoin copies(s, copy);
  // Chunk sizes fall off linearly (weights chunks, chunks - 1, ..., 1), so
  // the copy of the last chunk, the only one nothing overlaps, is the
  // shortest.
  size_t const nchunks = std::max<size_t>(1, std::min<size_t>(kHostChunks, npairs >> 14));
  size_t const wsum    = nchunks * (nchunks + 1) / 2;
  auto const chunk_end = [&](size_t c) {  // pairs in chunks 0..c-1
    size_t const w = c * nchunks - c * (c - 1) / 2;  // sum of the first c weights
    return c == nchunks ? npairs : static_cast<size_t>(static_cast<double>(npairs) * w / wsum);
  };
  size_t rows = 0;
  for (size_t c = 0; c < nchunks; ++c) {
    size_t const k0 = chunk_end(c), n = chunk_end(c + 1) - k0;
    evaluate(k0, n);
    Buffer<uint64_t> out_off;
    size_t const m = row_offsets(k0, n, out_off);
    if (m > 0) {
      Buffer<uint32_t> op(alloc, m), oq(alloc, m);
      expand(k0, n, out_off, op.data(), oq.data(), m);
      if (rows + m <= host->capacity) {
        stream_wait(copy, s);
        CSPT_CUDA_TRY(cudaMemcpyAsync(host->polygon_index + rows, op.data(), m * 4,
                                      cudaMemcpyDeviceToHost, copy));
        CSPT_CUDA_TRY(cudaMemcpyAsync(host->point_index + rows, oq.data(), m * 4,
                                      cudaMemcpyDeviceToHost, copy));
      }
      staged.push_back(std::move(op));
      staged.push_back(std::move(oq));
    }
    rows += m;
  }
  copies.join();
  finish_counts();
  *out_n = rows;
  CSPT_EXPECTS(rows <= host->capacity,
               "the host buffers hold " + std::to_string(host->capacity) +
                 " rows; the result has " + std::to_string(rows));
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
    refined_  = Buffer<unsigned long long>(alloc, 3);  // refined, next pair, edge-free pairs
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
    unsigned const grd = grid_for(np_ * 32, blk, sm_grid(8u * 1024u / blk));
    CSPT_CUDA_TRY(cudaMemsetAsync(refined_.data(), 0, 3 * sizeof(unsigned long long), s));
    if (filtered_) {
      leaf_frame_kernel<<<grd, blk, 0, s>>>(gstart_.data(), gstart_.data() + np_, pq_, qlen_,
                                            qoff_, src(), npi_, ix_.grid, u_.data(),
                                            frames_.data());
      CSPT_CHECK_LAUNCH();
      if (ix_.slab_nfull)
        pip_pair_kernel<true, true><<<grid_ordered_, blk, 0, s>>>(
          pp_, pq_, pgroup_.data(), np_, qlen_, qoff_, src(), npi_, u_.data(), frames_.data(),
          ix_, word_off_.data(), bits_.data(), counts_.data(), refined_.data(),
          refined_.data() + 1, refined_.data() + 2);
      else
        pip_pair_kernel<true><<<grid_true_, blk, 0, s>>>(
          pp_, pq_, pgroup_.data(), np_, qlen_, qoff_, src(), npi_, u_.data(), frames_.data(),
          ix_, word_off_.data(), bits_.data(), counts_.data(), refined_.data(),
          refined_.data() + 1, refined_.data() + 2);
    } else {
      pip_pair_kernel<false><<<grid_false_, blk, 0, s>>>(
        pp_, pq_, nullptr, np_, qlen_, qoff_, src(), npi_, nullptr, nullptr, ix_,
        word_off_.data(), bits_.data(), counts_.data(), nullptr, refined_.data() + 1,
        refined_.data() + 2);
    }
    CSPT_CHECK_LAUNCH();
    scan_apply_prealloc<uint64_t>(CountsOf{counts_.data()}, Store64{out_off_.data()}, np_,
                                  out_off_.data() + np_, partials_.data(), s);
  }

  // writes the rows of the last evaluation to op/oq, up to cap entries
  void expand(cudaStream_t s, uint32_t* op, uint32_t* oq, uint64_t cap)
  {
    unsigned const blk = blk_;
    unsigned const grd = grid_for(np_, blk, sm_grid(8u * 1024u / blk));  // a warp per 32 pairs
    pip_expand_kernel<<<grd, blk, 0, s>>>(pp_, pq_, np_, qlen_, qoff_, word_off_.data(),
                                          bits_.data(), out_off_.data(), op, oq, cap, nullptr);
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
  PointSource<double> src() const { return PointSource<double>{pi_, x_, y_, nullptr}; }
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
                               uint64_t* out_refined, HostRows const* host, void const* ordered)
{
  if (dtype == CSPT_FLOAT64)
    run<double>(pair_poly, pair_quad, npairs, tree, point_indices, npi,
                static_cast<double const*>(x), static_cast<double const*>(y), po, npo, ro, nro,
                static_cast<double const*>(vx), static_cast<double const*>(vy), nv, method, alloc,
                out_poly, out_point, out_n, out_refined, host,
                static_cast<double const*>(ordered));
  else
    run<float>(pair_poly, pair_quad, npairs, tree, point_indices, npi,
               static_cast<float const*>(x), static_cast<float const*>(y), po, npo, ro, nro,
               static_cast<float const*>(vx), static_cast<float const*>(vy), nv, method, alloc,
               out_poly, out_point, out_n, out_refined, host, static_cast<float const*>(ordered));
}

// defined in the other kernel translation units
void quadtree_on_points_from_host(void const* host_x, void const* host_y, void* dev_x,
                                  void* dev_y, size_t n, cspt_dtype dtype, double x_min,
                                  double x_max, double y_min, double y_max, double scale,
                                  int max_depth, int32_t max_size, Allocator const& alloc,
                                  uint32_t** out_point_indices, cspt_quadtree* out_tree,
                                  void* ordered,
                                  std::function<void(cudaStream_t)> const* after_copies);
void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);
void join_quadtree_and_bounding_boxes(cspt_quadtree const* tree, void const* bminx,
                                      void const* bminy, void const* bmaxx, void const* bmaxy,
                                      size_t nb, cspt_dtype dtype, double x_min, double y_min,
                                      double scale, int max_depth, Allocator const& alloc,
                                      uint32_t** out_box, uint32_t** out_node, size_t* out_n);

namespace {

// The whole join from host columns to host rows on stream s.  The points go
// to the device in chunks, each chunk's Morton keys computed as it lands
// (quadtree_on_points from host); the polygons follow them on the link, and
// their boxes and index are built on a second stream while the quadtree is
// built; then the box join and the point-in-polygon test with its rows
// copied to the host chunk by chunk.  Rows carry input point ids.
template <typename T>
void join_host(T const* hx, T const* hy, size_t n, double x_min, double x_max, double y_min,
               double y_max, double scale, int max_depth, int32_t max_size, uint32_t const* hpo,
               size_t npo, uint32_t const* hro, size_t nro, T const* hvx, T const* hvy,
               size_t nv, cspt_method method, cspt_allocator const* mr, cudaStream_t s,
               HostRows const& out, size_t* out_n, uint64_t* out_refined)
{
  cspt_dtype const dtype = std::is_same<T, double>::value ? CSPT_FLOAT64 : CSPT_FLOAT32;
  bool const filtered    = method == CSPT_METHOD_FILTERED && std::is_same<T, double>::value;
  size_t const np        = npo - 1;
  Allocator const alloc(mr, s);
  cudaStream_t const ps = side_stream(1);
  Allocator const palloc(mr, ps);
  // polygon columns, boxes and index: allocated and used on ps, read on s
  // once s has waited for ps
  Buffer<uint32_t> dpo(palloc, npo), dro(palloc, nro);
  Buffer<T> dvx(palloc, nv), dvy(palloc, nv);
  Buffer<T> bminx(palloc, np), bminy(palloc, np), bmaxx(palloc, np), bmaxy(palloc, np);
  std::unique_ptr<PolygonIndex<T>> index;
  // (declared after the polygon buffers: on every exit ps first waits for
  // s, so the buffers are released on ps only after s's last use of them)
  StreamJoin ps_after_s(ps, s);
  Buffer<T> dx(alloc, n), dy(alloc, n), oxy(alloc, 2 * n);
  std::function<void(cudaStream_t)> const after_points = [&](cudaStream_t copy) {
    stream_wait(ps, copy);  // behind the points on the host link
    CSPT_CUDA_TRY(cudaMemcpyAsync(dpo.data(), hpo, npo * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, ps));
    CSPT_CUDA_TRY(cudaMemcpyAsync(dro.data(), hro, nro * sizeof(uint32_t),
                                  cudaMemcpyHostToDevice, ps));
    CSPT_CUDA_TRY(cudaMemcpyAsync(dvx.data(), hvx, nv * sizeof(T), cudaMemcpyHostToDevice, ps));
    CSPT_CUDA_TRY(cudaMemcpyAsync(dvy.data(), hvy, nv * sizeof(T), cudaMemcpyHostToDevice, ps));
    polygon_bounding_boxes(dpo.data(), npo, dro.data(), nro, dvx.data(), dvy.data(), nv, dtype,
                           0.0, bminx.data(), bminy.data(), bmaxx.data(), bmaxy.data(), palloc);
    index.reset(new PolygonIndex<T>(dpo.data(), npo, dro.data(), nro, dvx.data(), dvy.data(), nv,
                                    filtered, palloc, false, false));
  };
  uint32_t* pi_raw = nullptr;
  cspt_quadtree tree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
  quadtree_on_points_from_host(hx, hy, dx.data(), dy.data(), n, dtype, x_min, x_max, y_min,
                               y_max, scale, max_depth, max_size, alloc, &pi_raw, &tree,
                               oxy.data(), &after_points);
  Buffer<uint32_t> pidx = Buffer<uint32_t>::adopt(alloc, pi_raw, n);
  size_t const q        = tree.num_nodes;
  Buffer<uint32_t> tkey = Buffer<uint32_t>::adopt(alloc, const_cast<uint32_t*>(tree.key), q);
  Buffer<uint8_t> tlev  = Buffer<uint8_t>::adopt(alloc, const_cast<uint8_t*>(tree.level), q);
  Buffer<uint8_t> tint = Buffer<uint8_t>::adopt(alloc, const_cast<uint8_t*>(tree.is_internal_node), q);
  Buffer<uint32_t> tlen = Buffer<uint32_t>::adopt(alloc, const_cast<uint32_t*>(tree.length), q);
  Buffer<uint32_t> toff = Buffer<uint32_t>::adopt(alloc, const_cast<uint32_t*>(tree.offset), q);
  CSPT_EXPECTS(index != nullptr, "the polygons were not queued behind the points");
  stream_wait(s, ps);  // boxes and index
  uint32_t* pb_raw = nullptr;
  uint32_t* pq_raw = nullptr;
  size_t npairs    = 0;
  if (q > 0)
    join_quadtree_and_bounding_boxes(&tree, bminx.data(), bminy.data(), bmaxx.data(),
                                     bmaxy.data(), np, dtype, x_min, y_min, scale, max_depth,
                                     alloc, &pb_raw, &pq_raw, &npairs);
  Buffer<uint32_t> pair_poly = Buffer<uint32_t>::adopt(alloc, pb_raw, npairs);
  Buffer<uint32_t> pair_quad = Buffer<uint32_t>::adopt(alloc, pq_raw, npairs);
  *out_n = 0;
  if (npairs == 0) return;
  run<T>(pair_poly.data(), pair_quad.data(), npairs, &tree, pidx.data(), n, dx.data(), dy.data(),
         dpo.data(), npo, dro.data(), nro, dvx.data(), dvy.data(), nv, method, alloc, nullptr,
         nullptr, out_n, out_refined, &out, oxy.data(), index.get(), pidx.data());
}

}  // namespace

void point_in_polygon_join_host(void const* hx, void const* hy, size_t n, cspt_dtype dtype,
                                double x_min, double x_max, double y_min, double y_max,
                                double scale, int max_depth, int32_t max_size,
                                uint32_t const* hpo, size_t npo, uint32_t const* hro,
                                size_t nro, void const* hvx, void const* hvy, size_t nv,
                                cspt_method method, cspt_allocator const* mr, cudaStream_t s,
                                HostRows const& out, size_t* out_n, uint64_t* out_refined)
{
  if (dtype == CSPT_FLOAT64)
    join_host<double>(static_cast<double const*>(hx), static_cast<double const*>(hy), n, x_min,
                      x_max, y_min, y_max, scale, max_depth, max_size, hpo, npo, hro, nro,
                      static_cast<double const*>(hvx), static_cast<double const*>(hvy), nv,
                      method, mr, s, out, out_n, out_refined);
  else
    join_host<float>(static_cast<float const*>(hx), static_cast<float const*>(hy), n, x_min,
                     x_max, y_min, y_max, scale, max_depth, max_size, hpo, npo, hro, nro,
                     static_cast<float const*>(hvx), static_cast<float const*>(hvy), nv, method,
                     mr, s, out, out_n, out_refined);
}

}  // namespace cspt
