// Builds the polygon index described in polygon_index.cuh.
//
// Two passes, one 128-thread block per polygon, slab counters in shared
// memory (no global atomics):
//   count: vertex box, sum of edge heights, slab count, entries per polygon,
//          vertical edges, the "walk the reference loop" flag;
//   (scans of slab counts, entries and vertical counts over polygons)
//   fill:  grid-rounded anchors, float32 box and edges, slab offsets, slab
//          entries (vertex index and float32 edge), sorted vertical x.
#include "polygon_index.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

constexpr int kIdxBlock = 128;
constexpr int kMaxSlabs = 4096;

// About two index entries per edge: with S slabs an edge of height h appears
// in about h*S/H + 1 slabs, so S ~ V*H / sum(h), between 1 and min(V/2, 4096).
// Slab count: with s = density * V * height / sum|rise| slabs, a slab lists
// about (1 + 1/density) * sum|rise| / height edges (the edges crossing it plus
// those ending inside it) and the index holds (1 + density) entries per edge.
// Denser slabs shorten every candidate's edge walk at the cost of index
// memory and build time; measured on the 100k-polygon, 8-512-vertex star
// set, density 4 minimises build + float32 evaluation and density 8 the
// float64-only evaluation.
constexpr double kSlabDensityFloat32 = 4.0;
constexpr double kSlabDensityFloat64 = 8.0;
__device__ inline uint32_t choose_slabs(uint32_t nv, double height, double sum_rise,
                                        double density)
{
  if (nv < 8 || !(height > 0.0) || !(sum_rise > 0.0)) return 1;
  double s         = density * static_cast<double>(nv) * height / sum_rise;
  double const cap = fmin(static_cast<double>(nv) * 0.5 * density, static_cast<double>(kMaxSlabs));
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

// Previous vertex of v within its ring (polygons have few rings).
__device__ inline uint32_t prev_in_ring(uint32_t const* ro, uint32_t r0, uint32_t r1, uint32_t v)
{
  for (uint32_t r = r0; r < r1; ++r) {
    uint32_t const b = ro[r], e = ro[r + 1];
    if (v >= b && v < e) return v == b ? e - 1 : v - 1;
  }
  return v;
}

template <typename T>
__device__ inline T block_min(T v, T* sh)
{
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = sh[0];
  for (int w = 1; w < kIdxBlock / 32; ++w) r = fmin(r, sh[w]);
  __syncthreads();
  return r;
}
template <typename T>
__device__ inline T block_max(T v, T* sh)
{
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = sh[0];
  for (int w = 1; w < kIdxBlock / 32; ++w) r = fmax(r, sh[w]);
  __syncthreads();
  return r;
}
template <typename T>
__device__ inline T block_sum(T v, T* sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = sh[0];
  for (int w = 1; w < kIdxBlock / 32; ++w) r += sh[w];
  __syncthreads();
  return r;
}

// In-place exclusive scan of cnt[0..n) (n <= kMaxSlabs) by one block;
// returns the total.
__device__ inline uint32_t block_scan_counts(uint32_t* cnt, uint32_t n, uint32_t* sh)
{
  uint32_t const per = (n + kIdxBlock - 1) / kIdxBlock;
  uint32_t const b   = threadIdx.x * per;
  uint32_t const e   = min(n, b + per);
  uint32_t s         = 0;
  for (uint32_t i = b; i < e; ++i) s += cnt[i];
  uint32_t const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl       = s;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t const t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += t;
  }
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  uint32_t base = 0, total = 0;
  for (uint32_t w = 0; w < kIdxBlock / 32; ++w) {
    if (w < warp) base += sh[w];
    total += sh[w];
  }
  uint32_t run = base + incl - s;
  for (uint32_t i = b; i < e; ++i) {
    uint32_t const c = cnt[i];
    cnt[i]           = run;
    run += c;
  }
  __syncthreads();
  return total;
}

// A vertex's edge (prev -> v), packed in 32 bits: slab range j0..j1 (12 bits
// each), bit 24 degenerate (the reference skips it), bit 25 exactly vertical,
// bit 26 degenerate by ULP but not equal (walk the reference loop instead).
constexpr uint32_t kSpanSkip = 1u << 24, kSpanVertical = 1u << 25, kSpanTiny = 1u << 26;
__device__ inline uint32_t span_j0(uint32_t s) { return s & 0xFFFu; }
__device__ inline uint32_t span_j1(uint32_t s) { return (s >> 12) & 0xFFFu; }

// The slab coordinate (y - ymin) * inv_h is taken in float64 once per end
// point and rounded to float32 (2.5e-4 slab at most for 4096 slabs); the
// range is widened by 2^-36 of the edge height (on-edge band, see the header)
// plus 1/32 slab, which covers that rounding and the float32 slab lookup of
// the filter (below 1e-3 slab), so j0..j1 contains the float64 and float32
// slab of every point the edge can matter to.
template <typename T>
__device__ inline uint32_t edge_span(T const* vx, T const* vy, uint32_t v, uint32_t pv, T ymin,
                                     T ih, uint32_t ns)
{
  T const ax = vx[v], ay = vy[v], bx = vx[pv], by = vy[pv];
  T const run = bx - ax, rise = by - ay;
  bool const skip = float_equal(run, T{0}) && float_equal(rise, T{0});
  if (skip) return kSpanSkip | ((run != T{0} || rise != T{0}) ? kSpanTiny : 0u);
  float const fa = static_cast<float>((ay - ymin) * ih);
  float const fb = static_cast<float>((by - ymin) * ih);
  float const lo = fminf(fa, fb), hi = fmaxf(fa, fb);
  float const mg = (hi - lo) * 1.4551915228366852e-11f + 0.03125f;
  float const l  = lo - mg, h = hi + mg;
  float const top = static_cast<float>(ns);
  uint32_t const j0 = !(l > 0.0f) ? 0u : (l >= top ? ns - 1 : min(static_cast<uint32_t>(l), ns - 1));
  uint32_t const j1 = !(h > 0.0f) ? 0u : (h >= top ? ns - 1 : min(static_cast<uint32_t>(h), ns - 1));
  return j0 | (j1 << 12) | (run == T{0} ? kSpanVertical : 0u);
}

// Pass 1: per polygon box, slab count, entries, vertical edges, flags.
template <typename T>
__global__ void __launch_bounds__(kIdxBlock)
  index_count_kernel(uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                     T const* __restrict__ vx, T const* __restrict__ vy, size_t np, T* pminx,
                     T* pminy, T* pmaxx, T* pmaxy, T* invh, uint32_t* nslab, uint32_t* nentries,
                     uint32_t* nvert, uint8_t* exact, uint32_t* __restrict__ prev_out,
                     uint32_t* __restrict__ spans, double density)
{
  __shared__ uint32_t cnt[kMaxSlabs];
  __shared__ T shT[kIdxBlock / 32];
  __shared__ double shD[kIdxBlock / 32];
  __shared__ uint32_t shU[kIdxBlock / 32];
  for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    T mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    double sum_rise = 0.0;
    uint32_t bad    = 0;
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
      T const x = vx[v], y = vy[v];
      mnx       = fmin(mnx, x);
      mny       = fmin(mny, y);
      mxx       = fmax(mxx, x);
      mxy       = fmax(mxy, y);
      bad |= (isfinite(x) && isfinite(y)) ? 0u : 1u;
      uint32_t const pv = prev_in_ring(ro, r0, r1, v);
      sum_rise += fabs(static_cast<double>(vy[pv]) - static_cast<double>(y));
    }
    mnx      = block_min(mnx, shT);
    mny      = block_min(mny, shT);
    mxx      = block_max(mxx, shT);
    mxy      = block_max(mxy, shT);
    sum_rise = block_sum(sum_rise, shD);
    uint32_t const ns = choose_slabs(
      ve - vb, static_cast<double>(mxy) - static_cast<double>(mny), sum_rise, density);
    T const h  = mxy - mny;
    T const ih = (ns > 1 && h > T{0}) ? static_cast<T>(ns) / h : T{0};
    for (uint32_t j = threadIdx.x; j < ns; j += kIdxBlock) cnt[j] = 0;
    __syncthreads();
    uint32_t verts = 0;
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
      uint32_t const pv = prev_in_ring(ro, r0, r1, v);
      uint32_t const sp = edge_span<T>(vx, vy, v, pv, mny, ih, ns);
      prev_out[v]       = pv;
      spans[v]          = sp;
      bad |= (sp & kSpanTiny) ? 1u : 0u;
      if (sp & kSpanSkip) continue;
      verts += (sp & kSpanVertical) ? 1u : 0u;
      for (uint32_t j = span_j0(sp); j <= span_j1(sp); ++j) atomicAdd(&cnt[j], 1u);
    }
    __syncthreads();
    uint32_t local = 0;
    for (uint32_t j = threadIdx.x; j < ns; j += kIdxBlock) local += cnt[j];
    local = block_sum(local, shU);
    verts = block_sum(verts, shU);
    bad   = block_sum(bad, shU);
    if (threadIdx.x == 0) {
      pminx[p]    = mnx;
      pminy[p]    = mny;
      pmaxx[p]    = mxx;
      pmaxy[p]    = mxy;
      invh[p]     = ih;
      nslab[p]    = ns;
      nentries[p] = local;
      nvert[p]    = verts;
      exact[p]    = bad ? 1 : 0;
    }
    __syncthreads();
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

// Pass 2: anchors, float32 edges, slab offsets and entries, vertical x.
template <typename T>
__global__ void __launch_bounds__(kIdxBlock)
  index_fill_kernel(uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                    T const* __restrict__ vx, T const* __restrict__ vy, size_t np,
                    T const* __restrict__ pminx, T const* __restrict__ pminy,
                    T const* __restrict__ pmaxx, T const* __restrict__ pmaxy,
                    T const* __restrict__ invh, uint32_t const* __restrict__ nslab,
                    uint32_t const* __restrict__ slab_base, uint32_t const* __restrict__ entry_base,
                    uint32_t const* __restrict__ vert_base, T const* __restrict__ grid,
                    bool float32, T* anchor_x, T* anchor_y, long long* aix, long long* aiy,
                    float4* box32, float* invh32, float* maxoff, uint32_t const* __restrict__ prev,
                    uint32_t const* __restrict__ spans, float4* edge32, uint32_t* slab_start,
                    uint32_t* slab_edges, float4* slab_e32, T* vert_x, float* vert_x32)
{
  __shared__ uint32_t cur[kMaxSlabs];
  __shared__ uint32_t shU[kIdxBlock / 32];
  __shared__ float shF[kIdxBlock / 32];
  __shared__ uint32_t vcur;
  T const g = *grid;
  for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    uint32_t const ns = nslab[p];
    T const ymin = pminy[p], ih = invh[p];
    T cx = T{0}, cy = T{0};
    if (ve > vb) {
      cx = rint((pminx[p] + pmaxx[p]) * T{0.5} / g) * g;
      cy = rint((ymin + pmaxy[p]) * T{0.5} / g) * g;
      if (!isfinite(cx)) cx = T{0};
      if (!isfinite(cy)) cy = T{0};
    }
    if (threadIdx.x == 0) {
      anchor_x[p] = cx;
      anchor_y[p] = cy;
      aix[p]      = llrint(cx / g);
      aiy[p]      = llrint(cy / g);
      box32[p]    = make_float4(static_cast<float>(pminx[p] - cx), static_cast<float>(ymin - cy),
                                static_cast<float>(pmaxx[p] - cx), static_cast<float>(pmaxy[p] - cy));
      invh32[p]   = static_cast<float>(ih);
      vcur        = 0;
    }
    for (uint32_t j = threadIdx.x; j < ns; j += kIdxBlock) cur[j] = 0;
    __syncthreads();
    // slab sizes again, then their offsets
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
      uint32_t const sp = spans[v];
      if (sp & kSpanSkip) continue;
      for (uint32_t j = span_j0(sp); j <= span_j1(sp); ++j) atomicAdd(&cur[j], 1u);
    }
    __syncthreads();
    uint32_t const total = block_scan_counts(cur, ns, shU);
    uint32_t const eb    = entry_base[p];
    uint32_t const sb    = slab_base[p];
    for (uint32_t j = threadIdx.x; j <= ns; j += kIdxBlock)
      slab_start[sb + j] = eb + (j < ns ? cur[j] : total);
    __syncthreads();
    float local_max      = 0.0f;
    uint32_t const vbase = vert_base[p];
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
      uint32_t const sp = spans[v];
      uint32_t const pv = prev[v];
      float4 ef{};
      if (float32) {
        ef.x      = static_cast<float>(vx[v] - cx);
        ef.y      = static_cast<float>(vy[v] - cy);
        ef.z      = static_cast<float>(vx[pv] - cx);
        ef.w      = static_cast<float>(vy[pv] - cy);
        edge32[v] = ef;
        local_max = fmaxf(local_max, fmaxf(fmaxf(fabsf(ef.x), fabsf(ef.y)),
                                           fmaxf(fabsf(ef.z), fabsf(ef.w))));
      }
      if (sp & kSpanSkip) continue;
      for (uint32_t j = span_j0(sp); j <= span_j1(sp); ++j) {
        uint32_t const k = eb + atomicAdd(&cur[j], 1u);
        slab_edges[k]    = v;
        if (float32) slab_e32[k] = ef;
      }
      if (sp & kSpanVertical) {
        uint32_t const k  = atomicAdd(&vcur, 1u);
        vert_x[vbase + k] = vx[v];
      }
    }
    local_max = block_max(local_max, shF);
    __syncthreads();
    if (threadIdx.x == 0) {
      maxoff[p] = local_max;
      // sort the (short) vertical-x list
      uint32_t const n = vcur;
      for (uint32_t i = 1; i < n; ++i) {
        T const key = vert_x[vbase + i];
        uint32_t j  = i;
        while (j > 0 && vert_x[vbase + j - 1] > key) {
          vert_x[vbase + j] = vert_x[vbase + j - 1];
          --j;
        }
        vert_x[vbase + j] = key;
      }
      if (float32)
        for (uint32_t i = 0; i < n; ++i)
          vert_x32[vbase + i] = static_cast<float>(vert_x[vbase + i] - cx);
    }
    __syncthreads();
  }
}

__global__ void copy_totals_kernel(uint32_t const* a, uint32_t const* b, uint32_t const* c,
                                   uint32_t* out)
{
  out[0] = *a;
  out[1] = *b;
  out[2] = *c;
}

// 64-bit sums of the per-polygon slab and entry counts: the 32-bit scans
// above are only valid below 2^32
__global__ void wide_totals_kernel(uint32_t const* __restrict__ nslab,
                                   uint32_t const* __restrict__ nent, size_t np,
                                   unsigned long long* out)
{
  unsigned long long a = 0, b = 0;
  for (size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; p < np;
       p += static_cast<size_t>(gridDim.x) * blockDim.x) {
    a += nslab[p];
    b += nent[p];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
    b += __shfl_xor_sync(0xFFFFFFFFu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, a);
    atomicAdd(out + 1, b);
  }
}

__global__ void vert_end_kernel(uint32_t const* __restrict__ vbeg,
                                uint32_t const* __restrict__ nvert, size_t np,
                                uint32_t* __restrict__ vend)
{
  for (size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; p < np;
       p += static_cast<size_t>(gridDim.x) * blockDim.x)
    vend[p] = vbeg[p] + nvert[p];
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
  size_t const np = npo > 0 ? npo - 1 : 0;
  pminx_     = Buffer<T>(alloc, np);
  pminy_     = Buffer<T>(alloc, np);
  pmaxx_     = Buffer<T>(alloc, np);
  pmaxy_     = Buffer<T>(alloc, np);
  ax_        = Buffer<T>(alloc, np);
  ay_        = Buffer<T>(alloc, np);
  invh_      = Buffer<T>(alloc, np);
  grid_      = Buffer<T>(alloc, 1);
  maxoff_    = Buffer<float>(alloc, np);
  invh32_    = Buffer<float>(alloc, np);
  box32_     = Buffer<float4>(alloc, np);
  aix_       = Buffer<long long>(alloc, np);
  aiy_       = Buffer<long long>(alloc, np);
  nslab_     = Buffer<uint32_t>(alloc, np + 1);
  slab_base_ = Buffer<uint32_t>(alloc, np + 1);
  vbeg_      = Buffer<uint32_t>(alloc, np + 1);
  vend_      = Buffer<uint32_t>(alloc, np + 1);
  exact_     = Buffer<uint8_t>(alloc, np);
  prev_      = Buffer<uint32_t>(alloc, nv);
  if (build_float32) edge32_ = Buffer<float4>(alloc, nv);
  Buffer<uint32_t> nent(alloc, np + 1), ebase(alloc, np + 1), nvert(alloc, np + 1);
  Buffer<uint32_t> totals(alloc, 3);
  Buffer<uint32_t> spans(alloc, nv);

  unsigned const grd = static_cast<unsigned>(np < 152u * 64u ? (np ? np : 1) : 152u * 64u);
  if (np > 0) {
    index_count_kernel<T><<<grd, kIdxBlock, 0, s>>>(
      po, ro, vx, vy, np, pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
      invh_.data(), nslab_.data(), nent.data(), nvert.data(), exact_.data(), prev_.data(),
      spans.data(), build_float32 ? kSlabDensityFloat32 : kSlabDensityFloat64);
    CSPT_CHECK_LAUNCH();
  }
  grid_kernel<T><<<1, 1024, 0, s>>>(pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
                                    np, grid_.data());
  CSPT_CHECK_LAUNCH();
  exclusive_scan<uint32_t>(nslab_.data(), slab_base_.data(), np, slab_base_.data() + np, alloc);
  exclusive_scan<uint32_t>(nent.data(), ebase.data(), np, ebase.data() + np, alloc);
  exclusive_scan<uint32_t>(nvert.data(), vbeg_.data(), np, vbeg_.data() + np, alloc);
  copy_totals_kernel<<<1, 1, 0, s>>>(slab_base_.data() + np, ebase.data() + np,
                                     vbeg_.data() + np, totals.data());
  CSPT_CHECK_LAUNCH();
  Buffer<unsigned long long> wide(alloc, 2);
  CSPT_CUDA_TRY(cudaMemsetAsync(wide.data(), 0, 2 * sizeof(unsigned long long), s));
  if (np > 0) {
    wide_totals_kernel<<<grid_for(np, 256, 152u * 4u), 256, 0, s>>>(nslab_.data(), nent.data(),
                                                                     np, wide.data());
    CSPT_CHECK_LAUNCH();
  }
  uint32_t tot[3];
  unsigned long long wtot[2];
  CSPT_CUDA_TRY(cudaMemcpyAsync(tot, totals.data(), sizeof(tot), cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaMemcpyAsync(wtot, wide.data(), sizeof(wtot), cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaStreamSynchronize(s));
  CSPT_EXPECTS(wtot[0] < (1ull << 32) && wtot[1] < (1ull << 32),
               "polygon set too large for the slab index (2^32 slab entries)");
  size_t const nslabs_total = tot[0], nentries = tot[1], nvertical = tot[2];
  slab_start_ = Buffer<uint32_t>(alloc, nslabs_total + 1);
  slab_edges_ = Buffer<uint32_t>(alloc, nentries);
  if (build_float32) slab_e32_ = Buffer<float4>(alloc, nentries);
  vert_x_ = Buffer<T>(alloc, nvertical);
  if (build_float32) vert_x32_ = Buffer<float>(alloc, nvertical);
  if (nslabs_total == 0)
    CSPT_CUDA_TRY(cudaMemsetAsync(slab_start_.data(), 0, sizeof(uint32_t), s));
  if (np > 0) {
    index_fill_kernel<T><<<grd, kIdxBlock, 0, s>>>(
      po, ro, vx, vy, np, pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
      invh_.data(), nslab_.data(), slab_base_.data(), ebase.data(), vbeg_.data(), grid_.data(),
      build_float32, ax_.data(), ay_.data(), aix_.data(), aiy_.data(), box32_.data(),
      invh32_.data(), maxoff_.data(), prev_.data(), spans.data(), edge32_.data(),
      slab_start_.data(),
      slab_edges_.data(), slab_e32_.data(), vert_x_.data(), vert_x32_.data());
    CSPT_CHECK_LAUNCH();
    vert_end_kernel<<<grid_for(np, 256, 152u * 16u), 256, 0, s>>>(vbeg_.data(), nvert.data(),
                                                                  np, vend_.data());
    CSPT_CHECK_LAUNCH();
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
                           slab_e32_.data(),
                           prev_.data(),
                           edge32_.data()};
}

template class PolygonIndex<float>;
template class PolygonIndex<double>;

}  // namespace cspt
