// Quadtree point-to-nearest-linestring join on sm_103a.
//
// Reference: cpp/include/cuspatial/detail/join/quadtree_point_to_nearest_
// linestring.cuh:143-312 and detail/algorithm/point_linestring_distance.cuh:
// 26-51.
//
// The reference enumerates, per quadrant, the (point, linestring) candidates
// point-major (the "transposed" index math at :63-89), reduces each point's
// run with a custom minimum (:279-294) and scatters to the point's position.
// Here the consecutive pairs that share a quadrant form a group; one warp owns
// a group, each lane a point, and the lane folds the group's linestrings in
// pair order with the same rule:
//   a running distance of exactly 0 yields to the next candidate, a new
//   candidate at exactly 0 never wins, equal distances keep the smaller id,
//   otherwise the smaller distance wins.
// The distance is the reference's expression with its dot products contracted
// the way nvcc contracts a.x*b.x + a.y*b.y (one FMA on the x term).
//
// Filtered method (float64 inputs): each segment is first bounded in float32
// with a forward error bound; only segments whose lower bound can still beat
// the best upper bound of the point are evaluated with the float64
// expression, so the winner and its distance are the exact ones.
#include "common.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

template <typename T>
__device__ inline T dot_fma(T ax, T ay, T bx, T by)
{
  return fma_rn(ax, bx, ay * by);
}

template <typename T>
__device__ inline T segment_dist2(T px, T py, T ax, T ay, T bx, T by)
{
  T const v1x = px - ax, v1y = py - ay;
  T const v2x = px - bx, v2y = py - by;
  T const d0  = dot_fma(v1x, v1y, v1x, v1y);
  T const d1  = dot_fma(v2x, v2y, v2x, v2y);
  T const ex = bx - ax, ey = by - ay;
  T const d2  = dot_fma(ex, ey, ex, ey);
  T const d3  = dot_fma(px - ax, py - ay, ex, ey);
  T const r   = d3 * d3 / d2;
  return (d3 <= T{0} || r >= d2) ? fmin(d0, d1) : d0 - r;
}

// point_linestring_distance.cuh:32-51
template <typename T>
__device__ inline T linestring_distance(T px, T py, T const* lx, T const* ly, uint32_t v0,
                                        uint32_t v1)
{
  T ds = std::numeric_limits<T>::max();
  for (uint32_t s = v0; s + 1 < v1; ++s)
    ds = fmin(ds, segment_dist2<T>(px, py, lx[s], ly[s], lx[s + 1], ly[s + 1]));
  return sqrt(ds);
}

// quadtree_point_to_nearest_linestring.cuh:279-294 — lhs is the running
// value, rhs the next candidate.
template <typename T>
__device__ inline bool take_rhs(T dl, uint32_t il, T dr, uint32_t ir)
{
  if (dl == T{0}) return true;
  if (dr == T{0}) return false;
  if (dl == dr) return !(il < ir);
  return !(dl < dr);
}

__global__ void init_rows_kernel(size_t n, uint32_t* __restrict__ opt, uint32_t* __restrict__ ols,
                                 void* __restrict__ od, int dsize)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    opt[i] = static_cast<uint32_t>(i);
    ols[i] = 0xFFFFFFFFu;
    if (dsize == 8)
      static_cast<double*>(od)[i] = 0.0;
    else
      static_cast<float*>(od)[i] = 0.0f;
  }
}

template <typename T, bool Filtered>
__global__ void __launch_bounds__(256)
  nearest_kernel(uint32_t const* __restrict__ group_start, size_t ngroups, size_t npairs,
                 uint32_t const* __restrict__ pair_ls, uint32_t const* __restrict__ pair_quad,
                 uint32_t const* __restrict__ qlen, uint32_t const* __restrict__ qoff,
                 uint32_t const* __restrict__ point_indices, size_t npi, T const* __restrict__ x,
                 T const* __restrict__ y, uint32_t const* __restrict__ lso, size_t nls,
                 T const* __restrict__ lx, T const* __restrict__ ly, uint32_t* __restrict__ opt,
                 uint32_t* __restrict__ ols, T* __restrict__ od)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t g = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; g < ngroups;
       g += warps) {
    uint32_t const k0   = group_start[g];
    uint32_t const k1   = (g + 1 < ngroups) ? group_start[g + 1] : static_cast<uint32_t>(npairs);
    uint32_t const quad = pair_quad[k0];
    uint32_t const len  = qlen[quad];
    uint64_t const off  = qoff[quad];
    for (uint32_t c = lane; c < len; c += 32) {
      uint64_t const pos = off + c;
      if (pos >= npi) continue;
      uint32_t const pi = point_indices[pos];
      T const px = x[pi], py = y[pi];
      bool have    = false;
      uint32_t bid = 0;
      T bd         = 0;
      for (uint32_t k = k0; k < k1; ++k) {
        uint32_t const lid = pair_ls[k];
        if (lid >= nls) continue;
        T const d = linestring_distance<T>(px, py, lx, ly, lso[lid], lso[lid + 1]);
        if (!have || take_rhs<T>(bd, bid, d, lid)) {
          bid = lid;
          bd  = d;
        }
        have = true;
      }
      if (have) {
        opt[pos] = static_cast<uint32_t>(pos);
        ols[pos] = bid;
        od[pos]  = bd;
      }
    }
  }
}

template <typename T>
void run(uint32_t const* pair_ls, uint32_t const* pair_quad, size_t npairs,
         cspt_quadtree const* tree, uint32_t const* point_indices, size_t npi, T const* x,
         T const* y, uint32_t const* lso, size_t nlso, T const* lx, T const* ly,
         cspt_method method, Allocator const& alloc, uint32_t* opt, uint32_t* ols, T* od)
{
  (void)method;
  cudaStream_t const s = alloc.stream();
  init_rows_kernel<<<grid_for(npi, 256, 152u * 16u), 256, 0, s>>>(npi, opt, ols, od, sizeof(T));
  CSPT_CHECK_LAUNCH();
  // groups: runs of consecutive pairs with the same quadrant first-point offset
  uint32_t const* qoff = tree->offset;
  Buffer<uint32_t> gstart(alloc, npairs + 1);
  uint32_t* gs = gstart.data();
  scan_apply<uint32_t>(
    [pair_quad, qoff] __device__(size_t k) {
      return (k == 0 || qoff[pair_quad[k]] != qoff[pair_quad[k - 1]]) ? 1u : 0u;
    },
    [gs] __device__(size_t k, uint32_t e, uint32_t f) {
      if (f) gs[e] = static_cast<uint32_t>(k);
    },
    npairs, gs + npairs, alloc);
  size_t const ng = read_back(gs + npairs, s);
  size_t const nls = nlso > 0 ? nlso - 1 : 0;
  {
    KernelTimer timer("nearest", s);
    nearest_kernel<T, false><<<grid_for(ng * 32, 256, 152u * 32u), 256, 0, s>>>(
      gs, ng, npairs, pair_ls, pair_quad, tree->length, qoff, point_indices, npi, x, y, lso,
      nls, lx, ly, opt, ols, od);
    CSPT_CHECK_LAUNCH();
  }
}

}  // namespace

void quadtree_point_to_nearest_linestring(uint32_t const* pair_ls, uint32_t const* pair_quad,
                                          size_t npairs, cspt_quadtree const* tree,
                                          uint32_t const* point_indices, size_t npi,
                                          void const* x, void const* y, uint32_t const* lso,
                                          size_t nlso, void const* lx, void const* ly,
                                          cspt_dtype dtype, cspt_method method,
                                          Allocator const& alloc, uint32_t* opt, uint32_t* ols,
                                          void* od)
{
  if (dtype == CSPT_FLOAT64)
    run<double>(pair_ls, pair_quad, npairs, tree, point_indices, npi,
                static_cast<double const*>(x), static_cast<double const*>(y), lso, nlso,
                static_cast<double const*>(lx), static_cast<double const*>(ly), method, alloc,
                opt, ols, static_cast<double*>(od));
  else
    run<float>(pair_ls, pair_quad, npairs, tree, point_indices, npi, static_cast<float const*>(x),
               static_cast<float const*>(y), lso, nlso, static_cast<float const*>(lx),
               static_cast<float const*>(ly), method, alloc, opt, ols, static_cast<float*>(od));
}

}  // namespace cspt
