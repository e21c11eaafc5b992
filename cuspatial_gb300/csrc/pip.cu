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
    uint32_t const v  = ix.slab_edges[k];
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

// float32 filter: returns 0/1 when every edge of the slab is decided, else
// kUndecided.  Bound on |cross32 - (lhs64 - rhs64)|: 48 u32 M^2 for offsets of
// magnitude <= M (input rounding of the anchored coordinates, the
// differences, the products and the FMA), plus the float64 rounding and the
// 4-ULP collinear band (< 2^-49 M^2); 2^-18 M^2 = 64 u32 M^2 covers all of it,
// and 2^-120 covers float32 underflow.
__device__ int pip_filter32(double px, double py, PolygonIndexView<double> const& ix,
                            uint32_t poly)
{
  if (!(py >= ix.pminy[poly]) || !(py < ix.pmaxy[poly])) return 0;
  if (ix.exact_only[poly] || !isfinite(px)) return kUndecided;
  float const qx = static_cast<float>(px - ix.anchor_x[poly]);
  float const qy = static_cast<float>(py - ix.anchor_y[poly]);
  if (!isfinite(qx) || !isfinite(qy)) return kUndecided;
  uint32_t const vb = ix.vert_begin[poly], ve = ix.vert_end[poly];
  if (vb < ve && sorted_has<float>(ix.vert_x32, vb, ve, qx)) return kUndecided;
  float const m  = fmaxf(ix.max_offset[poly], fmaxf(fabsf(qx), fabsf(qy)));
  float const eb = __fmaf_rn(3.814697265625e-06f * m, m, 7.52316384526264e-37f);
  uint32_t const s  = ix.slab_base[poly] + point_slab<double>(py, ix, poly);
  uint32_t const e0 = ix.slab_start[s], e1 = ix.slab_start[s + 1];
  bool within       = false;
  for (uint32_t k = e0; k < e1; ++k) {
    float4 const e = ix.edge32[ix.slab_edges[k]];  // (ax, ay, bx, by)
    if (e.y == qy || e.w == qy) return kUndecided;
    bool const y1    = e.y > qy;
    bool const y0    = e.w > qy;
    float const rtpx = qx - e.x;
    float const rise = e.w - e.y;
    float const run  = e.z - e.x;
    float const rtp  = qy - e.y;
    float const cr   = __fmaf_rn(rtpx, rise, -(run * rtp));
    if (fabsf(cr) <= eb) {
      float const mn = fminf(e.x, e.z), mx = fmaxf(e.x, e.z);
      if (!(qx < mn || qx > mx)) return kUndecided;
      if (y1 != y0) return kUndecided;
    } else if (y1 != y0) {
      if ((cr < 0.0f) != y1) within = !within;
    }
  }
  return within ? 1 : 0;
}

template <typename T, bool Filtered>
__global__ void __launch_bounds__(256)
  pip_bits_kernel(uint32_t const* __restrict__ pair_poly, uint32_t const* __restrict__ pair_quad,
                  size_t npairs, uint32_t const* __restrict__ qlen,
                  uint32_t const* __restrict__ qoff, uint32_t const* __restrict__ point_indices,
                  size_t npi, T const* __restrict__ x, T const* __restrict__ y,
                  PolygonIndexView<T> ix, uint64_t const* __restrict__ word_off,
                  uint32_t* __restrict__ bits, uint32_t* __restrict__ counts,
                  unsigned long long* __restrict__ refined)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t nref      = 0;
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
        T const px = x[pi], py = y[pi];
        if constexpr (Filtered) {
          int const r = pip_filter32(px, py, ix, poly);
          if (r == kUndecided) {
            ++nref;
            hit = pip_exact<T>(px, py, ix, poly);
          } else {
            hit = r == 1;
          }
        } else {
          hit = pip_exact<T>(px, py, ix, poly);
        }
      }
      unsigned const w = __ballot_sync(0xFFFFFFFFu, hit);
      if (lane == 0) bits[wb + (c >> 5)] = w;
      cnt += __popc(w);
    }
    if (lane == 0) counts[k] = cnt;
  }
  if (Filtered && refined) {
    for (int off = 16; off > 0; off >>= 1) nref += __shfl_xor_sync(0xFFFFFFFFu, nref, off);
    if (lane == 0 && nref) atomicAdd(refined, static_cast<unsigned long long>(nref));
  }
}

__global__ void __launch_bounds__(256)
  pip_expand_kernel(uint32_t const* __restrict__ pair_poly, uint32_t const* __restrict__ pair_quad,
                    size_t npairs, uint32_t const* __restrict__ qlen,
                    uint32_t const* __restrict__ qoff, uint64_t const* __restrict__ word_off,
                    uint32_t const* __restrict__ bits, uint64_t const* __restrict__ out_off,
                    uint32_t* __restrict__ out_poly, uint32_t* __restrict__ out_point)
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
        out_poly[d]      = poly;
        out_point[d]     = off + c + lane;
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
  Buffer<unsigned long long> refined(alloc, 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, sizeof(unsigned long long), s));
  unsigned const blk = 256;
  unsigned const grd = grid_for(npairs * 32, blk, 152u * 8u * 4u);
  {
    KernelTimer timer("pip_bits", s);
    bool launched = false;
    if constexpr (std::is_same<T, double>::value) {
      if (filtered) {
        pip_bits_kernel<double, true><<<grd, blk, 0, s>>>(
          pair_poly, pair_quad, npairs, qlen, qoff, point_indices, npi, x, y, index.view(),
          word_off.data(), bits.data(), counts.data(), refined.data());
        launched = true;
      }
    }
    if (!launched) {
      pip_bits_kernel<T, false><<<grd, blk, 0, s>>>(pair_poly, pair_quad, npairs, qlen, qoff,
                                                     point_indices, npi, x, y, index.view(),
                                                     word_off.data(), bits.data(),
                                                     counts.data(), nullptr);
    }
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
                                          op.data(), oq.data());
    CSPT_CHECK_LAUNCH();
  }
  *out_poly  = op.release();
  *out_point = oq.release();
}

}  // namespace

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
