// Leaf frames shared by the point-in-polygon and nearest-linestring
// filters: the points of a quadrant as float32 offsets from a grid-rounded
// anchor (the quadrant's first point), plus their extent.
#pragma once

#include "common.cuh"
#include "f32_diff.cuh"

namespace cspt {
namespace {  // one copy per translation unit

__device__ inline float warp_max(float v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, off));
  return v;
}
__device__ inline float warp_min(float v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, off));
  return v;
}

// Leaf frames: for every group of consecutive pairs that share a quadrant,
// one warp rounds the quadrant's first point to the anchor grid and writes
// u = fl32(p - A_l) for each of its points (indexed by sorted position; one
// rounding of the exact difference), the largest |u| and the u-range.
// Non-finite points are flagged per leaf.
struct LeafFrame {
  double ax, ay;
  long long ix, iy;               // anchor in grid steps
  float m;                        // max |u| over finite points
  float uxmin, uxmax, uymin, uymax;
  uint32_t nonfinite;
};

__global__ void __launch_bounds__(256)
  leaf_frame_kernel(uint32_t const* __restrict__ group_start, uint32_t const* __restrict__ ngroups_p,
                    uint32_t const* __restrict__ pair_quad, uint32_t const* __restrict__ qlen,
                    uint32_t const* __restrict__ qoff, PointSource<double> const src,
                    size_t npi, double const* __restrict__ gridp, float2* __restrict__ u,
                    LeafFrame* __restrict__ frames)
{
  int const lane      = threadIdx.x & 31;
  size_t const nwarps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t const ng   = *ngroups_p;
  double const g      = *gridp;
  double const ginv   = 1.0 / g;  // g is a power of two: v * ginv == v / g while 1/g is finite
  bool const ginv_ok  = isfinite(ginv);
  for (size_t gi = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; gi < ng;
       gi += nwarps) {
    uint32_t const quad = pair_quad[group_start[gi]];
    uint32_t const len  = qlen[quad];
    uint64_t const off  = qoff[quad];
    double x0 = 0.0, y0 = 0.0;
    if (len > 0 && off < npi) src.load(off, x0, y0);
    double rx = rint(ginv_ok ? x0 * ginv : x0 / g), ry = rint(ginv_ok ? y0 * ginv : y0 / g);
    if (!(fabs(rx) < 4.0e18)) rx = 0.0;  // also NaN
    if (!(fabs(ry) < 4.0e18)) ry = 0.0;
    double const ax = rx * g, ay = ry * g;
    float m = 0.0f, xmn = INFINITY, xmx = -INFINITY, ymn = INFINITY, ymx = -INFINITY;
    bool bad = false;
    // four independent loads per lane per round (with points in quadtree
    // order one coalesced 16-byte load each; otherwise the index, then the
    // two gathers)
    for (uint32_t c0 = 0; c0 < len; c0 += 128) {
      uint32_t pi[4];
      bool ok[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        uint32_t const c   = c0 + t * 32 + lane;
        uint64_t const pos = off + c;
        ok[t]              = c < len && pos < npi;
        pi[t]              = (ok[t] && !src.xy) ? src.point_indices[pos] : 0u;
      }
      double px[4], py[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        px[t] = 0.0;
        py[t] = 0.0;
        if (!ok[t]) continue;
        if (src.xy) {
          double2 const v = reinterpret_cast<double2 const*>(src.xy)[off + c0 + t * 32 + lane];
          px[t]           = v.x;
          py[t]           = v.y;
        } else {
          px[t] = src.x[pi[t]];
          py[t] = src.y[pi[t]];
        }
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        if (!ok[t]) continue;
        // fl32(p - A), rounded once; on the integer pipe where the inputs
        // allow, else through the float64 subtraction
        float2 v;
        if (!f32_of_difference(px[t], ax, v.x)) v.x = static_cast<float>(px[t] - ax);
        if (!f32_of_difference(py[t], ay, v.y)) v.y = static_cast<float>(py[t] - ay);
        u[off + c0 + t * 32 + lane]   = v;
        if (isfinite(v.x) && isfinite(v.y)) {
          m   = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
          xmn = fminf(xmn, v.x);
          xmx = fmaxf(xmx, v.x);
          ymn = fminf(ymn, v.y);
          ymx = fmaxf(ymx, v.y);
        } else {
          bad = true;
        }
      }
    }
    m   = warp_max(m);
    xmn = warp_min(xmn);
    xmx = warp_max(xmx);
    ymn = warp_min(ymn);
    ymx = warp_max(ymx);
    bad = __any_sync(0xFFFFFFFFu, bad);
    if (lane == 0)
      frames[gi] = LeafFrame{ax,  ay,  static_cast<long long>(rx), static_cast<long long>(ry), m,
                             xmn, xmx, ymn, ymx, bad ? 1u : 0u};
  }
}

}  // namespace
}  // namespace cspt
