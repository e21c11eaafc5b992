// Builds the polygon index described in polygon_index.cuh.  Every pass runs
// one warp per polygon with lanes striding over its vertices (coalesced).
#include "polygon_index.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

// A polygon's slab count: about two index entries per edge.  With S slabs an
// edge of height h appears in about h*S/H + 1 slabs, so S ~ V*H / sum(h),
// between 1 and min(V/2, 4096).
__device__ inline uint32_t choose_slabs(uint32_t nv, double height, double sum_rise)
{
  if (nv < 8 || !(height > 0.0) || !(sum_rise > 0.0)) return 1;
  double s = static_cast<double>(nv) * height / sum_rise;
  double const cap = fmin(static_cast<double>(nv) * 0.5, 4096.0);
  if (!(s <= cap)) s = cap;
  if (s < 1.0) s = 1.0;
  return static_cast<uint32_t>(s);
}

template <typename T>
__device__ inline uint32_t slab_of(T y, T ymin, T inv_h, uint32_t ns)
{
  T const f = (y - ymin) * inv_h;
  if (!(f > T{0})) return 0;  // also NaN
  if (f >= static_cast<T>(ns)) return ns - 1;
  uint32_t const j = static_cast<uint32_t>(f);
  return j < ns ? j : ns - 1;
}

template <typename T>
__device__ inline bool finite_t(T v)
{
  return isfinite(v);
}

// Ring r of polygon p containing vertex v (polygons have few rings).
__device__ inline uint32_t prev_in_ring(uint32_t const* ro, uint32_t r0, uint32_t r1, uint32_t v)
{
  for (uint32_t r = r0; r < r1; ++r) {
    uint32_t const b = ro[r], e = ro[r + 1];
    if (v >= b && v < e) return v == b ? e - 1 : v - 1;
  }
  return v;
}

template <typename T>
__global__ void poly_stats_kernel(uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                                  T const* __restrict__ vx, T const* __restrict__ vy, size_t np,
                                  T* pminx, T* pminy, T* pmaxx, T* pmaxy, T* ax, T* ay, T* invh,
                                  uint32_t* nslab, uint32_t* vert_count, float* maxoff,
                                  uint8_t* exact)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t p = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; p < np;
       p += warps) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    T mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    double sum_rise = 0.0;
    bool bad        = false;
    for (uint32_t v = vb + lane; v < ve; v += 32) {
      T const x = vx[v], y = vy[v];
      mnx       = fmin(mnx, x);
      mny       = fmin(mny, y);
      mxx       = fmax(mxx, x);
      mxy       = fmax(mxy, y);
      bad |= !finite_t(x) || !finite_t(y);
      uint32_t const pv = prev_in_ring(ro, r0, r1, v);
      sum_rise += fabs(static_cast<double>(vy[pv]) - static_cast<double>(y));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mnx = fmin(mnx, __shfl_xor_sync(0xFFFFFFFFu, mnx, off));
      mny = fmin(mny, __shfl_xor_sync(0xFFFFFFFFu, mny, off));
      mxx = fmax(mxx, __shfl_xor_sync(0xFFFFFFFFu, mxx, off));
      mxy = fmax(mxy, __shfl_xor_sync(0xFFFFFFFFu, mxy, off));
      sum_rise += __shfl_xor_sync(0xFFFFFFFFu, sum_rise, off);
    }
    bad = __any_sync(0xFFFFFFFFu, bad);
    if (lane == 0) {
      pminx[p]          = mnx;
      pminy[p]          = mny;
      pmaxx[p]          = mxx;
      pmaxy[p]          = mxy;
      T const cx        = ve > vb ? (mnx + mxx) * T{0.5} : T{0};
      T const cy        = ve > vb ? (mny + mxy) * T{0.5} : T{0};
      ax[p]             = cx;
      ay[p]             = cy;
      uint32_t const ns = choose_slabs(ve - vb, static_cast<double>(mxy) - mny, sum_rise);
      nslab[p]          = ns;
      T const h         = mxy - mny;
      invh[p]           = (ns > 1 && h > T{0}) ? static_cast<T>(ns) / h : T{0};
      vert_count[p]     = 0;
      maxoff[p]         = 0.0f;
      exact[p]          = bad ? 1 : 0;
    }
  }
}

// The anchor grid: 2^(e-22) where 2^e bounds every finite polygon coordinate.
template <typename T>
__global__ void __launch_bounds__(1024)
  grid_kernel(T const* __restrict__ pminx, T const* __restrict__ pminy,
              T const* __restrict__ pmaxx, T const* __restrict__ pmaxy, size_t np, T* grid)
{
  __shared__ T part[32];
  T m = 0;
  for (size_t p = threadIdx.x; p < np; p += blockDim.x) {
    T const v[4] = {pminx[p], pminy[p], pmaxx[p], pmaxy[p]};
    for (T a : v)
      if (isfinite(a)) m = fmax(m, fabs(a));
  }
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, off));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = part[threadIdx.x];
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, off));
    if (threadIdx.x == 0) {
      int e = 0;
      frexp(m > T{0} ? m : T{1}, &e);  // m < 2^e
      *grid = ldexp(T{1}, e - 22);
    }
  }
}

// Per edge: previous vertex, float32 offsets, degenerate/vertical flags and
// slab range.  fill == false counts entries; fill == true writes them.
template <typename T, bool Fill>
__global__ void poly_edges_kernel(uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                                  T const* __restrict__ vx, T const* __restrict__ vy, size_t np,
                                  T const* __restrict__ pminy, T const* __restrict__ ax,
                                  T const* __restrict__ ay, T const* __restrict__ invh,
                                  uint32_t const* __restrict__ nslab,
                                  uint32_t const* __restrict__ slab_base, uint32_t* slab_count,
                                  uint32_t const* __restrict__ slab_start,
                                  uint32_t* __restrict__ slab_edges, uint32_t* vert_count,
                                  uint32_t const* __restrict__ vert_begin, T* __restrict__ vert_x,
                                  float* maxoff, uint8_t* exact, uint32_t* __restrict__ prev_out,
                                  float4* __restrict__ edge32, bool build_float32,
                                  T const* __restrict__ pmaxy, T* anchor_x, T* anchor_y,
                                  T const* __restrict__ pminx, T const* __restrict__ pmaxx,
                                  T const* __restrict__ grid, float4* __restrict__ box32,
                                  long long* __restrict__ aix, long long* __restrict__ aiy,
                                  float* __restrict__ invh32)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t p = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; p < np;
       p += warps) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    uint32_t const ns = nslab[p];
    uint32_t const sb = slab_base[p];
    T const ymin = pminy[p], ih = invh[p];
    T cx = ax[p], cy = ay[p];
    if (!Fill) {
      // anchors: the box centre rounded to the grid
      T const g = *grid;
      if (ve > vb) {
        cx = rint((pminx[p] + pmaxx[p]) * T{0.5} / g) * g;
        cy = rint((ymin + pmaxy[p]) * T{0.5} / g) * g;
        if (!isfinite(cx)) cx = T{0};
        if (!isfinite(cy)) cy = T{0};
      }
      if (lane == 0) {
        anchor_x[p] = cx;
        anchor_y[p] = cy;
        aix[p]      = llrint(cx / g);
        aiy[p]      = llrint(cy / g);
        invh32[p]   = static_cast<float>(ih);
        box32[p]    = make_float4(static_cast<float>(pminx[p] - cx), static_cast<float>(ymin - cy),
                                  static_cast<float>(pmaxx[p] - cx),
                                  static_cast<float>(pmaxy[p] - cy));
      }
    }
    // a float32 slab lookup is within 1e-3 slab of the float64 one
    T const slab_margin = ih > T{0} ? T{1} / (ih * T{64}) : T{0};
    float local_max = 0.0f;
    bool tiny_skip  = false;
    for (uint32_t v = vb + lane; v < ve; v += 32) {
      uint32_t const pv = prev_in_ring(ro, r0, r1, v);
      T const axv = vx[v], ayv = vy[v], bxv = vx[pv], byv = vy[pv];
      T const run = bxv - axv, rise = byv - ayv;
      bool const skip = float_equal(run, T{0}) && float_equal(rise, T{0});
      if (!Fill) {
        prev_out[v] = pv;
        if (skip && (run != T{0} || rise != T{0})) tiny_skip = true;
        if (build_float32) {
          float4 e;
          e.x = static_cast<float>(axv - cx);
          e.y = static_cast<float>(ayv - cy);
          e.z = static_cast<float>(bxv - cx);
          e.w = static_cast<float>(byv - cy);
          edge32[v] = e;
          local_max = fmaxf(local_max, fmaxf(fmaxf(fabsf(e.x), fabsf(e.y)),
                                             fmaxf(fabsf(e.z), fabsf(e.w))));
        }
      }
      if (skip) continue;
      T const lo = ayv < byv ? ayv : byv;
      T const hi = ayv < byv ? byv : ayv;
      T const mu = (hi - lo) * T(1.4551915228366852e-11) + slab_margin;  // 2^-36 of the height
      uint32_t const j0 = slab_of<T>(lo - mu, ymin, ih, ns);
      uint32_t const j1 = slab_of<T>(hi + mu, ymin, ih, ns);
      for (uint32_t j = j0; j <= j1; ++j) {
        if (!Fill) {
          atomicAdd(&slab_count[sb + j], 1u);
        } else {
          uint32_t const k = atomicAdd(&slab_count[sb + j], 1u);
          slab_edges[slab_start[sb + j] + k] = v;
        }
      }
      if (run == T{0}) {
        uint32_t const k = atomicAdd(&vert_count[p], 1u);
        if (Fill) vert_x[vert_begin[p] + k] = axv;
      }
    }
    if (!Fill) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        local_max = fmaxf(local_max, __shfl_xor_sync(0xFFFFFFFFu, local_max, off));
      tiny_skip = __any_sync(0xFFFFFFFFu, tiny_skip);
      if (lane == 0) {
        maxoff[p] = local_max;
        if (tiny_skip) exact[p] = 1;
      }
    }
  }
}

// Sorts each polygon's vertical-x list (insertion sort; lists are short) and
// makes the float32 copy.
template <typename T>
__global__ void vert_sort_kernel(uint32_t const* __restrict__ vbeg,
                                 uint32_t const* __restrict__ vend, size_t np, T* vert_x,
                                 float* vert_x32, T const* __restrict__ ax)
{
  for (size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; p < np;
       p += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t const b = vbeg[p], e = vend[p];
    for (uint32_t i = b + 1; i < e; ++i) {
      T const v  = vert_x[i];
      uint32_t j = i;
      while (j > b && vert_x[j - 1] > v) {
        vert_x[j] = vert_x[j - 1];
        --j;
      }
      vert_x[j] = v;
    }
    if (vert_x32)
      for (uint32_t i = b; i < e; ++i) vert_x32[i] = static_cast<float>(vert_x[i] - ax[p]);
  }
}

__global__ void add_begin_kernel(uint32_t const* __restrict__ vbeg, uint32_t* __restrict__ vend,
                                 size_t np)
{
  for (size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; p < np;
       p += static_cast<size_t>(gridDim.x) * blockDim.x)
    vend[p] += vbeg[p];
}

}  // namespace

template <typename T>
PolygonIndex<T>::PolygonIndex(uint32_t const* po, size_t npo, uint32_t const* ro, size_t nro,
                              T const* vx, T const* vy, size_t nv, bool build_float32,
                              Allocator const& alloc)
{
  (void)nro;
  cudaStream_t const s = alloc.stream();
  KernelTimer timer("polygon_index", s);
  size_t const np      = npo > 0 ? npo - 1 : 0;
  pminx_  = Buffer<T>(alloc, np);
  pminy_  = Buffer<T>(alloc, np);
  pmaxx_  = Buffer<T>(alloc, np);
  pmaxy_  = Buffer<T>(alloc, np);
  ax_     = Buffer<T>(alloc, np);
  ay_     = Buffer<T>(alloc, np);
  invh_   = Buffer<T>(alloc, np);
  maxoff_ = Buffer<float>(alloc, np);
  nslab_  = Buffer<uint32_t>(alloc, np + 1);
  slab_base_ = Buffer<uint32_t>(alloc, np + 1);
  vbeg_   = Buffer<uint32_t>(alloc, np + 1);
  vend_   = Buffer<uint32_t>(alloc, np);
  exact_  = Buffer<uint8_t>(alloc, np);
  grid_   = Buffer<T>(alloc, 1);
  box32_  = Buffer<float4>(alloc, np);
  aix_    = Buffer<long long>(alloc, np);
  aiy_    = Buffer<long long>(alloc, np);
  invh32_ = Buffer<float>(alloc, np);
  prev_   = Buffer<uint32_t>(alloc, nv);
  if (build_float32) edge32_ = Buffer<float4>(alloc, nv);

  unsigned const blk = 256;
  unsigned const grd = grid_for(np * 32, blk, 152u * 32u);
  if (np > 0) {
    poly_stats_kernel<T><<<grd, blk, 0, s>>>(po, ro, vx, vy, np, pminx_.data(), pminy_.data(),
                                             pmaxx_.data(), pmaxy_.data(), ax_.data(),
                                             ay_.data(), invh_.data(), nslab_.data(),
                                             vend_.data(), maxoff_.data(), exact_.data());
    CSPT_CHECK_LAUNCH();
  }
  grid_kernel<T><<<1, 1024, 0, s>>>(pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
                                    np, grid_.data());
  CSPT_CHECK_LAUNCH();
  // slab bases
  Buffer<uint32_t> total(alloc, 1);
  exclusive_scan<uint32_t>(nslab_.data(), slab_base_.data(), np, total.data(), alloc);
  size_t const nslabs_total = read_back(total.data(), s);
  Buffer<uint32_t> slab_count(alloc, nslabs_total + 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(slab_count.data(), 0, (nslabs_total + 1) * sizeof(uint32_t), s));
  if (np > 0) {
    poly_edges_kernel<T, false><<<grd, blk, 0, s>>>(
      po, ro, vx, vy, np, pminy_.data(), ax_.data(), ay_.data(), invh_.data(), nslab_.data(),
      slab_base_.data(), slab_count.data(), nullptr, nullptr, vend_.data(), nullptr, nullptr,
      maxoff_.data(), exact_.data(), prev_.data(), edge32_.data(), build_float32, pmaxy_.data(),
      ax_.data(), ay_.data(), pminx_.data(), pmaxx_.data(), grid_.data(), box32_.data(),
      aix_.data(), aiy_.data(), invh32_.data());
    CSPT_CHECK_LAUNCH();
  }
  slab_start_ = Buffer<uint32_t>(alloc, nslabs_total + 1);
  exclusive_scan<uint32_t>(slab_count.data(), slab_start_.data(), nslabs_total,
                           slab_start_.data() + nslabs_total, alloc);
  size_t const nentries = read_back(slab_start_.data() + nslabs_total, s);
  exclusive_scan<uint32_t>(vend_.data(), vbeg_.data(), np, vbeg_.data() + np, alloc);
  size_t const nvert = read_back(vbeg_.data() + np, s);
  slab_edges_ = Buffer<uint32_t>(alloc, nentries);
  vert_x_     = Buffer<T>(alloc, nvert);
  if (build_float32) vert_x32_ = Buffer<float>(alloc, nvert);
  CSPT_CUDA_TRY(cudaMemsetAsync(slab_count.data(), 0, (nslabs_total + 1) * sizeof(uint32_t), s));
  CSPT_CUDA_TRY(cudaMemsetAsync(vend_.data(), 0, np * sizeof(uint32_t), s));
  if (np > 0) {
    poly_edges_kernel<T, true><<<grd, blk, 0, s>>>(
      po, ro, vx, vy, np, pminy_.data(), ax_.data(), ay_.data(), invh_.data(), nslab_.data(),
      slab_base_.data(), slab_count.data(), slab_start_.data(), slab_edges_.data(),
      vend_.data(), vbeg_.data(), vert_x_.data(), maxoff_.data(), exact_.data(), prev_.data(),
      edge32_.data(), build_float32, pmaxy_.data(), ax_.data(), ay_.data(), pminx_.data(),
      pmaxx_.data(), grid_.data(), box32_.data(), aix_.data(), aiy_.data(), invh32_.data());
    CSPT_CHECK_LAUNCH();
    // vend = vbeg + count
    add_begin_kernel<<<grid_for(np, 256, 152u * 16u), 256, 0, s>>>(vbeg_.data(), vend_.data(),
                                                                   np);
    CSPT_CHECK_LAUNCH();
    if (nvert > 0) {
      vert_sort_kernel<T><<<grid_for(np, 128, 152u * 16u), 128, 0, s>>>(
        vbeg_.data(), vend_.data(), np, vert_x_.data(), vert_x32_.data(), ax_.data());
      CSPT_CHECK_LAUNCH();
    }
  }
  v_ = PolygonIndexView<T>{po,
                           ro,
                           vx,
                           vy,
                           np,
                           pminx_.data(),
                           pminy_.data(),
                           pmaxx_.data(),
                           pmaxy_.data(),
                           ax_.data(),
                           ay_.data(),
                           grid_.data(),
                           aix_.data(),
                           aiy_.data(),
                           invh32_.data(),
                           invh_.data(),
                           maxoff_.data(),
                           box32_.data(),
                           nslab_.data(),
                           slab_base_.data(),
                           exact_.data(),
                           vbeg_.data(),
                           vend_.data(),
                           vert_x_.data(),
                           vert_x32_.data(),
                           slab_start_.data(),
                           slab_edges_.data(),
                           prev_.data(),
                           edge32_.data()};
}

template class PolygonIndex<float>;
template class PolygonIndex<double>;

}  // namespace cspt
