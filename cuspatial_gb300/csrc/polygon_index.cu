// Builds the polygon index described in polygon_index.cuh.
//
// Two passes, one 128-thread block per polygon, slab counters in shared
// memory (no global atomics):
//   count: vertex box, sum of edge heights, slab count, entries per polygon,
//          vertical edges, the "walk the reference loop" flag;
//   (scans of slab counts, entries and vertical counts over polygons)
//   fill:  grid-rounded anchors, float32 box and edges, slab offsets, slab
//          entries (vertex index and float32 edge), sorted vertical x.
#include <cmath>

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
// memory and build time.  Measured on the 100k-polygon, 8-512-vertex star
// set (build + evaluation): density 2 for the one-shot float32 index, whose
// pair kernel classifies a quadrant's slab entries once (1: 12.90 ms,
// 2: 12.51, 3: 12.71, 4: 13.29); 4 for the ordered index, whose per-point
// windows gain from shorter slabs; 8 for the float64-only evaluation.
#ifndef CSPT_SLAB_DENSITY32
#define CSPT_SLAB_DENSITY32 2.0
#endif
constexpr double kSlabDensityFloat32 = CSPT_SLAB_DENSITY32;
constexpr double kSlabDensityOrdered = 4.0;
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

// The slab coordinate (y - ymin) * inv_h is taken in float64 once per
// vertex and rounded to float32 (2.5e-4 slab at most for 4096 slabs); an
// edge's range is widened by 2^-36 of its height (on-edge band, see the
// header) plus 1/32 slab, which covers that rounding and the float32 slab
// lookup of the filter (below 1e-3 slab), so j0..j1 contains the float64 and
// float32 slab of every point the edge can matter to.
//
// Degenerate and vertical edges are found on the bit patterns: for finite
// coordinates the reference's float_equal(b - a, 0) holds exactly when
// a == b, except where both coordinates lie below 2^-1019, where distinct
// neighbours can be within 4 ULP of each other; such edges are flagged
// (kSpanTiny) and their polygon is walked with the reference loop.
template <typename T>
__device__ inline bool same_value(T a, T b)
{
  return a == b;
}
template <>
__device__ inline bool same_value<double>(double a, double b)
{
  unsigned long long const x = __double_as_longlong(a), y = __double_as_longlong(b);
  return x == y || ((x | y) << 1) == 0ull;  // equal bits, or +0 and -0
}
// exponent field <= 3: |a| < 2^-1019 (double), 2^-123 (float)
__device__ inline bool below_tiny(float a) { return ((__float_as_uint(a) >> 23) & 0xFFu) <= 3u; }
__device__ inline bool below_tiny(double a)
{
  return ((static_cast<unsigned long long>(__double_as_longlong(a)) >> 52) & 0x7FFull) <= 3ull;
}

template <typename T>
__device__ inline uint32_t edge_span(T ax, T ay, T bx, T by, float fa, float fb, uint32_t ns)
{
  bool const ex = same_value(ax, bx), ey = same_value(ay, by);
  bool const nx = ex || (below_tiny(ax) && below_tiny(bx));
  bool const ny = ey || (below_tiny(ay) && below_tiny(by));
  if (ex && ey) return kSpanSkip;
  if (nx && ny) return kSpanSkip | kSpanTiny;
  float const lo = fminf(fa, fb), hi = fmaxf(fa, fb);
  float const mg = (hi - lo) * 1.4551915228366852e-11f + 0.03125f;
  float const l  = lo - mg, h = hi + mg;
  float const top = static_cast<float>(ns);
  uint32_t const j0 = !(l > 0.0f) ? 0u : (l >= top ? ns - 1 : min(static_cast<uint32_t>(l), ns - 1));
  uint32_t const j1 = !(h > 0.0f) ? 0u : (h >= top ? ns - 1 : min(static_cast<uint32_t>(h), ns - 1));
  return j0 | (j1 << 12) | (ex ? kSpanVertical : 0u);
}

// A double cut to float32 on the integer pipe (mantissa truncated; below
// float32's normal range -> 0, beyond it or non-finite -> infinity), for the
// slab-count heuristic only: any slab count gives a valid index.
__device__ inline float truncated_f32(double v)
{
  unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(v));
  uint32_t const sign        = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  int const e                = static_cast<int>((b >> 52) & 0x7FFull) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
  return __uint_as_float(sign | (static_cast<uint32_t>(e) << 23) |
                         static_cast<uint32_t>((b >> 29) & 0x7FFFFFull));
}

// Order-preserving integer image of a non-NaN double (min/max on the
// integer pipe; float64 comparisons run at a small fraction of that rate).
__device__ inline long long order_key(double v)
{
  long long const b = __double_as_longlong(v);
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
__device__ inline double from_order_key(long long k)
{
  return __longlong_as_double(k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL));
}
__device__ inline bool is_nan_bits(double v)
{
  unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(v));
  return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}
__device__ inline bool is_finite_bits(double v)
{
  unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(v));
  return (b & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

__device__ inline long long block_min_ll(long long v, long long* sh)
{
  for (int o = 16; o > 0; o >>= 1) {
    long long const t = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v                 = t < v ? t : v;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  long long r = sh[0];
  for (int w = 1; w < kIdxBlock / 32; ++w) r = sh[w] < r ? sh[w] : r;
  __syncthreads();
  return r;
}
__device__ inline long long block_max_ll(long long v, long long* sh)
{
  for (int o = 16; o > 0; o >>= 1) {
    long long const t = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v                 = t > v ? t : v;
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  long long r = sh[0];
  for (int w = 1; w < kIdxBlock / 32; ++w) r = sh[w] > r ? sh[w] : r;
  __syncthreads();
  return r;
}

// Pass 1: per polygon box, slab count, entries, vertical edges, flags.
// Per-polygon quantities are computed once (thread 0) and shared; each
// vertex's slab coordinate is computed once (yslab) and read by both edges
// that end at it.
template <typename T>
__global__ void __launch_bounds__(kIdxBlock)
  index_count_kernel(uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                     T const* __restrict__ vx, T const* __restrict__ vy, size_t np, T* pminx,
                     T* pminy, T* pmaxx, T* pmaxy, T* invh, uint32_t* nslab, uint32_t* nentries,
                     uint32_t* nvert, uint8_t* exact, uint32_t* __restrict__ prev_out,
                     uint32_t* __restrict__ spans, float* __restrict__ yslab, double density)
{
  __shared__ uint32_t cnt[kMaxSlabs];
  __shared__ T shT[kIdxBlock / 32];
  __shared__ long long shL[kIdxBlock / 32];
  __shared__ double shD[kIdxBlock / 32];
  __shared__ float shF[kIdxBlock / 32];
  __shared__ uint32_t shU[kIdxBlock / 32];
  __shared__ T s_ymin, s_ih;
  __shared__ uint32_t s_ns;
  for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    T mnx, mny, mxx, mxy;
    double sum_rise = 0.0;
    uint32_t bad    = 0;
    if constexpr (std::is_same<T, double>::value) {
      // the edges' rises for the slab count summed in float32 from
      // truncated vertices: the float64 pipe is this pass's bound
      float rise = 0.0f;
      long long kx0 = order_key(INFINITY), ky0 = order_key(INFINITY);
      long long kx1 = order_key(-INFINITY), ky1 = order_key(-INFINITY);
      for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
        double const x = vx[v], y = vy[v];
        bad |= (is_finite_bits(x) && is_finite_bits(y)) ? 0u : 1u;
        if (!is_nan_bits(x)) {
          long long const k = order_key(x);
          kx0               = k < kx0 ? k : kx0;
          kx1               = k > kx1 ? k : kx1;
        }
        if (!is_nan_bits(y)) {
          long long const k = order_key(y);
          ky0               = k < ky0 ? k : ky0;
          ky1               = k > ky1 ? k : ky1;
        }
        uint32_t const pv = prev_in_ring(ro, r0, r1, v);
        prev_out[v]       = pv;
        rise += fabsf(truncated_f32(vy[pv]) - truncated_f32(y));
      }
      mnx      = from_order_key(block_min_ll(kx0, shL));
      mny      = from_order_key(block_min_ll(ky0, shL));
      mxx      = from_order_key(block_max_ll(kx1, shL));
      mxy      = from_order_key(block_max_ll(ky1, shL));
      sum_rise = static_cast<double>(block_sum(rise, shF));
    } else {
      mnx = INFINITY;
      mny = INFINITY;
      mxx = -INFINITY;
      mxy = -INFINITY;
      for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
        T const x = vx[v], y = vy[v];
        mnx       = fmin(mnx, x);
        mny       = fmin(mny, y);
        mxx       = fmax(mxx, x);
        mxy       = fmax(mxy, y);
        bad |= (isfinite(x) && isfinite(y)) ? 0u : 1u;
        uint32_t const pv = prev_in_ring(ro, r0, r1, v);
        prev_out[v]       = pv;
        sum_rise += fabs(static_cast<double>(vy[pv]) - static_cast<double>(y));
      }
      mnx      = block_min(mnx, shT);
      mny      = block_min(mny, shT);
      mxx      = block_max(mxx, shT);
      mxy      = block_max(mxy, shT);
      sum_rise = block_sum(sum_rise, shD);
    }
    if (threadIdx.x == 0) {
      uint32_t const ns = choose_slabs(
        ve - vb, static_cast<double>(mxy) - static_cast<double>(mny), sum_rise, density);
      T const h = mxy - mny;
      s_ns      = ns;
      s_ih      = (ns > 1 && h > T{0}) ? static_cast<T>(ns) / h : T{0};
      s_ymin    = mny;
    }
    __syncthreads();
    uint32_t const ns = s_ns;
    T const ih = s_ih, ymin = s_ymin;
    for (uint32_t j = threadIdx.x; j < ns; j += kIdxBlock) cnt[j] = 0;
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock)
      yslab[v] = static_cast<float>((vy[v] - ymin) * ih);
    __syncthreads();  // counters cleared, yslab of every vertex visible
    uint32_t verts = 0;
    for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock) {
      uint32_t const pv = prev_out[v];
      uint32_t const sp = edge_span<T>(vx[v], vy[v], vx[pv], vy[pv], yslab[v], yslab[pv], ns);
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
// The largest magnitude is taken on the bit patterns (sign cleared,
// non-finite skipped), which order as the magnitudes: integer work only, so
// the FP64 pipe of the one SM this runs on stays out of the loop.
template <typename T>
__global__ void __launch_bounds__(1024)
  grid_kernel(T const* __restrict__ pminx, T const* __restrict__ pminy,
              T const* __restrict__ pmaxx, T const* __restrict__ pmaxy, size_t np, T* grid)
{
  using U             = typename uint_of<T>::type;
  constexpr U kMag    = ~(U{1} << (8 * sizeof(U) - 1));
  constexpr U kExpAll = sizeof(T) == 8 ? U(0x7FF0000000000000ull) : U(0x7F800000u);
  __shared__ U part[32];
  U m = 0;
  for (size_t p = threadIdx.x; p < np; p += blockDim.x) {
    T const v[4] = {pminx[p], pminy[p], pmaxx[p], pmaxy[p]};
    for (T a : v) {
      U b;
      memcpy(&b, &a, sizeof(T));
      b &= kMag;
      if ((b & kExpAll) != kExpAll && b > m) m = b;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    U const o = __shfl_xor_sync(0xFFFFFFFFu, m, off);
    m         = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : U{0};
    for (int off = 16; off > 0; off >>= 1) {
      U const o = __shfl_xor_sync(0xFFFFFFFFu, m, off);
      m         = o > m ? o : m;
    }
    if (threadIdx.x == 0) {
      T mv;
      memcpy(&mv, &m, sizeof(T));
      int e = 0;
      frexp(mv > T{0} ? mv : T{1}, &e);  // mv < 2^e
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
                    uint32_t* slab_edges, float4* slab_e32, T* vert_x, float* vert_x32,
                    float2* __restrict__ vxy32, float const* __restrict__ yslab)
{
  __shared__ uint32_t cur[kMaxSlabs];
  __shared__ uint32_t shU[kIdxBlock / 32];
  __shared__ float shF[kIdxBlock / 32];
  __shared__ uint32_t vcur;
  __shared__ T s_cx, s_cy;
  T const g    = *grid;
  T const ginv = T{1} / g;  // g is a power of two: v * ginv == v / g while 1/g is finite
  bool const gi = isfinite(ginv);
  for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
    uint32_t const r0 = po[p], r1 = po[p + 1];
    uint32_t const vb = ro[r0], ve = ro[r1];
    uint32_t const ns = nslab[p];
    if (threadIdx.x == 0) {
      T const ymin = pminy[p];
      T cx = T{0}, cy = T{0};
      if (ve > vb) {
        T const mx = (pminx[p] + pmaxx[p]) * T{0.5}, my = (ymin + pmaxy[p]) * T{0.5};
        cx = rint(gi ? mx * ginv : mx / g) * g;
        cy = rint(gi ? my * ginv : my / g) * g;
        if (!isfinite(cx)) cx = T{0};
        if (!isfinite(cy)) cy = T{0};
      }
      s_cx        = cx;
      s_cy        = cy;
      anchor_x[p] = cx;
      anchor_y[p] = cy;
      aix[p]      = llrint(gi ? cx * ginv : cx / g);
      aiy[p]      = llrint(gi ? cy * ginv : cy / g);
      box32[p]    = make_float4(static_cast<float>(pminx[p] - cx), static_cast<float>(ymin - cy),
                                static_cast<float>(pmaxx[p] - cx), static_cast<float>(pmaxy[p] - cy));
      invh32[p]   = static_cast<float>(invh[p]);
      vcur        = 0;
    }
    for (uint32_t j = threadIdx.x; j < ns; j += kIdxBlock) cur[j] = 0;
    __syncthreads();
    T const cx = s_cx, cy = s_cy;
    // each vertex's float32 offset once (both of its edges read it)
    if (float32)
      for (uint32_t v = vb + threadIdx.x; v < ve; v += kIdxBlock)
        vxy32[v] = make_float2(static_cast<float>(vx[v] - cx), static_cast<float>(vy[v] - cy));
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
        float2 const a = vxy32[v], b = vxy32[pv];
        ef             = make_float4(a.x, a.y, b.x, b.y);
        edge32[v]      = ef;
        local_max = fmaxf(local_max, fmaxf(fmaxf(fabsf(ef.x), fabsf(ef.y)),
                                           fmaxf(fabsf(ef.z), fabsf(ef.w))));
      }
      if (sp & kSpanSkip) continue;
      float const fa = yslab[v], fb = yslab[pv];
      float const flo = fminf(fa, fb), fhi = fmaxf(fa, fb);
      for (uint32_t j = span_j0(sp); j <= span_j1(sp); ++j) {
        uint32_t const k = eb + atomicAdd(&cur[j], 1u);
        // bit 31: the edge crosses the whole slab (ends more than 1/16 slab
        // beyond it), used by the float32 ordering pass
        bool const crossing = flo < static_cast<float>(j) - 0.0625f &&
                              fhi > static_cast<float>(j) + 1.0625f;
        slab_edges[k]       = v | (crossing ? kEntryCrossing : 0u);
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

// Pass 3 (float32 index): within each slab, the edges that cross the whole
// slab (both ends more than 1/16 slab beyond it) come first, sorted left to
// right by their x at the slab's middle; the edges ending inside the slab
// follow.  Per slab and x-bin (kSlabBins bins across the polygon box) a
// record gives the window [lo, hi) of crossing edges to test: the crossing
// edges before lo end more than 1/16 bin left of the bin (certainly left of
// any point of the bin), those from hi on start more than 1/16 bin right of
// it (certainly right: each one toggles, so their count's parity is stored).
// The runs are found on the sorted order itself, so the records are valid
// whatever the order; the sort only makes the windows short.  Slabs with more
// than kSortSlab entries get an empty crossing set (every edge is tested).
constexpr int kSortSlab = 64;


// One warp per slab; lane l holds entries l and l + 32 (kSortSlab = 64).
__global__ void __launch_bounds__(kIdxBlock)
  slab_order_kernel(size_t np, uint32_t const* __restrict__ nslab,
                    uint32_t const* __restrict__ slab_base, uint32_t const* __restrict__ slab_start,
                    uint8_t const* __restrict__ exact, float4 const* __restrict__ box32,
                    uint32_t const* __restrict__ in_edges, float4 const* __restrict__ in_e32,
                    uint32_t* __restrict__ out_edges, float4* __restrict__ out_e32,
                    uint32_t* __restrict__ nfull_out, uint32_t* __restrict__ bins_out,
                    float* __restrict__ inv_bin_w)
{
  constexpr int kWarps = kIdxBlock / 32;
  __shared__ float2 sx[kWarps][kSortSlab];  // (x_min, x_max) of the crossing entries by rank
  int const lane = threadIdx.x & 31;
  int const warp = threadIdx.x >> 5;
  for (size_t p = blockIdx.x; p < np; p += gridDim.x) {
    uint32_t const ns = nslab[p], sb = slab_base[p];
    float4 const bx   = box32[p];
    float const width = bx.z - bx.x;
    bool const binned = !exact[p] && width > 0.0f && isfinite(width);
    float const invw  = binned ? static_cast<float>(kSlabBins) / width : 0.0f;
    float const w     = binned ? width / static_cast<float>(kSlabBins) : 0.0f;
    float const hstep = (bx.w - bx.y) / static_cast<float>(ns);
    if (threadIdx.x == 0) inv_bin_w[p] = invw;
    for (uint32_t j = warp; j < ns; j += kWarps) {
      uint32_t const sidx = sb + j;
      uint32_t const e0 = slab_start[sidx], e1 = slab_start[sidx + 1];
      uint32_t const n  = e1 - e0;
      if (!binned || n > static_cast<uint32_t>(kSortSlab) || n < 2) {
        // every entry is tested: copy, no crossing set
        for (uint32_t k = lane; k < n; k += 32) {
          out_edges[e0 + k] = in_edges[e0 + k];
          out_e32[e0 + k]   = in_e32[e0 + k];
        }
        if (lane < kSlabBins) bins_out[static_cast<size_t>(sidx) * kSlabBins + lane] = 0u;
        if (lane == 0) nfull_out[sidx] = 0;
        continue;
      }
      int const halves = n > 32u ? 2 : 1;
      float const ymid = bx.y + (static_cast<float>(j) + 0.5f) * hstep;
      uint32_t ev[2] = {0u, 0u};
      float4 ee[2];
      bool cross[2] = {false, false};
      float key[2]  = {0.0f, 0.0f};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t const k = lane + 32u * h;
        ee[h]            = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (h < halves && k < n) {
          ev[h]          = in_edges[e0 + k];
          ee[h]          = in_e32[e0 + k];
          cross[h]       = (ev[h] & kEntryCrossing) != 0u;
          float const t  = (ymid - ee[h].y) / (ee[h].w - ee[h].y);
          float const tc = t > 0.0f ? (t < 1.0f ? t : 1.0f) : 0.0f;
          float const km = ee[h].x + tc * (ee[h].z - ee[h].x);
          key[h]         = km == km ? km : 0.0f;  // ranks need a total order
        }
      }
      unsigned const c0 = __ballot_sync(0xFFFFFFFFu, cross[0]);
      unsigned const c1 = __ballot_sync(0xFFFFFFFFu, cross[1]);
      uint32_t const nf = __popc(c0) + __popc(c1);
      // crossing entries ranked by (key, entry index); the other entries
      // follow them in their original order
      unsigned const valid0 = n >= 32u ? 0xFFFFFFFFu : ((1u << n) - 1u);
      unsigned const valid1 = n >= 64u ? 0xFFFFFFFFu : (n > 32u ? ((1u << (n - 32u)) - 1u) : 0u);
      unsigned const part0  = valid0 & ~c0, part1 = valid1 & ~c1;
      unsigned const lt     = (1u << lane) - 1u;
      uint32_t rank[2]      = {nf + __popc(part0 & lt), nf + __popc(part0) + __popc(part1 & lt)};
      if (nf) {
        for (int h = 0; h < halves; ++h) {
          uint32_t const k = lane + 32u * h;
          uint32_t r       = 0;
          for (int src = 0; src < static_cast<int>(n); ++src) {
            int const sl      = src & 31, sh = src >> 5;
            float const okey  = __shfl_sync(0xFFFFFFFFu, sh ? key[1] : key[0], sl);
            bool const ocross = ((sh ? c1 : c0) >> sl) & 1u;
            r += (ocross &&
                  (okey < key[h] || (okey == key[h] && static_cast<uint32_t>(src) < k)))
                   ? 1u
                   : 0u;
          }
          if (cross[h]) {
            rank[h]             = r;
            sx[warp][r]         = make_float2(fminf(ee[h].x, ee[h].z), fmaxf(ee[h].x, ee[h].z));
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t const k = lane + 32u * h;
        if (h < halves && k < n) {
          out_edges[e0 + rank[h]] = ev[h];
          out_e32[e0 + rank[h]]   = ee[h];
        }
      }
      if (lane == 0) nfull_out[sidx] = nf;
      if (nf == 0) {
        if (lane < kSlabBins) bins_out[static_cast<size_t>(sidx) * kSlabBins + lane] = 0u;
        continue;
      }
      __syncwarp();
      // sorted crossing entries: lane i holds ranks i and i + 32
      float2 const s0 = lane < static_cast<int>(nf) ? sx[warp][lane] : make_float2(0.0f, 0.0f);
      float2 const s1 =
        lane + 32 < static_cast<int>(nf) ? sx[warp][lane + 32] : make_float2(0.0f, 0.0f);
      unsigned const in0 = nf >= 32u ? 0xFFFFFFFFu : ((1u << nf) - 1u);
      unsigned const in1 = nf >= 64u ? 0xFFFFFFFFu : (nf > 32u ? ((1u << (nf - 32u)) - 1u) : 0u);
      uint32_t rec = 0;
      for (int b = 0; b < kSlabBins; ++b) {
        float const blo = bx.x + static_cast<float>(b) * w - 0.0625f * w;
        float const bhi = bx.x + static_cast<float>(b + 1) * w + 0.0625f * w;
        // leading run of certainly-left entries, trailing run of certainly-right ones
        unsigned const l0 = __ballot_sync(0xFFFFFFFFu, s0.y < blo) & in0;
        unsigned const l1 = __ballot_sync(0xFFFFFFFFu, s1.y < blo) & in1;
        unsigned const r0 = __ballot_sync(0xFFFFFFFFu, s0.x > bhi) & in0;
        unsigned const r1 = __ballot_sync(0xFFFFFFFFu, s1.x > bhi) & in1;
        // lo: length of the run of ones from rank 0 (never past nf: bits
        // from nf on are zero unless nf = 64)
        unsigned long long const ll = (static_cast<unsigned long long>(l1) << 32) | l0;
        uint32_t const lo          = ~ll ? static_cast<uint32_t>(__ffsll(~ll) - 1) : 64u;
        // hi: one past the last rank that is not certainly right
        unsigned long long const rr = (static_cast<unsigned long long>(r1) << 32) | r0;
        unsigned long long const valid =
          nf >= 64u ? ~0ull : ((1ull << nf) - 1ull);
        unsigned long long const notr = ~rr & valid;  // entries that are not certainly right
        uint32_t hi = notr ? 64u - static_cast<uint32_t>(__clzll(notr)) : 0u;
        if (hi < lo) hi = lo;
        if (lane == b) rec = lo | (hi << 15) | (((nf - hi) & 1u) << 30);
      }
      if (lane < kSlabBins) bins_out[static_cast<size_t>(sidx) * kSlabBins + lane] = rec;
      __syncwarp();
    }
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
struct PolygonIndex<T>::Sizing {
  uint32_t const *po, *ro;
  T const *vx, *vy;
  size_t np, nslabs_total, nentries, nvertical;
  bool build_float32, order_slabs;
  unsigned grd;
  Buffer<uint32_t> ebase, nvert, spans;
  Buffer<float> yslab;
  Allocator const* alloc;  // the caller's: the index's buffers keep pointing to it
};

template <typename T>
PolygonIndex<T>::PolygonIndex(uint32_t const* po, size_t npo, uint32_t const* ro, size_t nro,
                              T const* vx, T const* vy, size_t nv, bool build_float32,
                              Allocator const& alloc, bool order_slabs, bool defer_fill)
{
  (void)nro;
  cudaStream_t const s = alloc.stream();
  KernelTimer timer("polygon_index", s);
  size_t const np = npo > 0 ? npo - 1 : 0;
  CSPT_EXPECTS(nv < (size_t{1} << 31), "the polygon index takes fewer than 2^31 vertices");
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
  Buffer<uint32_t> spans(alloc, nv);
  Buffer<float> yslab(alloc, nv);

  double const density = build_float32 ? (order_slabs ? kSlabDensityOrdered : kSlabDensityFloat32)
                                       : kSlabDensityFloat64;
  unsigned const grd = static_cast<unsigned>(np < sm_grid(64u) ? (np ? np : 1) : sm_grid(64u));
  if (np > 0) {
    index_count_kernel<T><<<grd, kIdxBlock, 0, s>>>(
      po, ro, vx, vy, np, pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
      invh_.data(), nslab_.data(), nent.data(), nvert.data(), exact_.data(), prev_.data(),
      spans.data(), yslab.data(), density);
    CSPT_CHECK_LAUNCH();
  }
  grid_kernel<T><<<1, 1024, 0, s>>>(pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
                                    np, grid_.data());
  CSPT_CHECK_LAUNCH();
  exclusive_scan<uint32_t>(nslab_.data(), slab_base_.data(), np, slab_base_.data() + np, alloc);
  exclusive_scan<uint32_t>(nent.data(), ebase.data(), np, ebase.data() + np, alloc);
  exclusive_scan<uint32_t>(nvert.data(), vbeg_.data(), np, vbeg_.data() + np, alloc);
  // Sizes of the slab arrays.  A polygon of V vertices gets
  // ns <= max(1, density V / 2) slabs, and its edges' slab spans add up to
  // at most (density + 1.07) V entries: with ns = s <= density V H / sum|rise|
  // slabs of height H / ns, an edge of rise r spans at most
  // r ns / H (1 + 2^-35) + 1 + 1/16 slabs (its range widened by 2^-36 of
  // itself plus 1/32 slab at each end, float32 slab coordinates within
  // 2^-12 slab), and the sum over edges of r ns / H is at most density V
  // (with one slab every edge spans one).  So (density + 2) entries per
  // vertex, 1 + density / 2 slabs per polygon and one vertical edge per
  // vertex bound the arrays without reading the counts back: no host
  // synchronisation.  Only where those bounds reach 2^32 (the 32-bit
  // offsets' limit) are the exact totals read back and checked.
  size_t const slab_bound  = np + static_cast<size_t>(std::ceil(density * 0.5 * nv)) + 1;
  size_t const entry_bound = static_cast<size_t>(std::ceil((density + 2.0) * nv)) + 1;
  size_t nslabs_total = slab_bound, nentries = entry_bound, nvertical = nv;
  if (slab_bound >= (size_t{1} << 32) || entry_bound >= (size_t{1} << 32)) {
    Buffer<uint32_t> totals(alloc, 3);
    copy_totals_kernel<<<1, 1, 0, s>>>(slab_base_.data() + np, ebase.data() + np,
                                       vbeg_.data() + np, totals.data());
    CSPT_CHECK_LAUNCH();
    Buffer<unsigned long long> wide(alloc, 2);
    CSPT_CUDA_TRY(cudaMemsetAsync(wide.data(), 0, 2 * sizeof(unsigned long long), s));
    if (np > 0) {
      wide_totals_kernel<<<grid_for(np, 256, sm_grid(4u)), 256, 0, s>>>(nslab_.data(),
                                                                       nent.data(), np,
                                                                       wide.data());
      CSPT_CHECK_LAUNCH();
    }
    uint32_t tot[3];
    unsigned long long wtot[2];
    CSPT_CUDA_TRY(cudaMemcpyAsync(tot, totals.data(), sizeof(tot), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(wtot, wide.data(), sizeof(wtot), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    CSPT_EXPECTS(wtot[0] < (1ull << 32) && wtot[1] < (1ull << 32),
                 "polygon set too large for the slab index (2^32 slab entries)");
    nslabs_total = tot[0];
    nentries     = tot[1];
    nvertical    = tot[2];
  }
  sizing_.reset(new Sizing{po, ro, vx, vy, np, nslabs_total, nentries, nvertical, build_float32,
                           order_slabs, grd, std::move(ebase), std::move(nvert), std::move(spans),
                           std::move(yslab), &alloc});
  if (!defer_fill) fill();
}

template <typename T>
PolygonIndex<T>::~PolygonIndex() = default;

template <typename T>
void PolygonIndex<T>::fill()
{
  if (!sizing_) return;
  std::unique_ptr<Sizing> const z = std::move(sizing_);
  Allocator const& alloc = *z->alloc;
  cudaStream_t const s   = alloc.stream();
  KernelTimer timer("polygon_index", s);
  uint32_t const *po = z->po, *ro = z->ro;
  T const *vx = z->vx, *vy = z->vy;
  size_t const np = z->np, nslabs_total = z->nslabs_total, nentries = z->nentries,
               nvertical = z->nvertical;
  size_t const nv          = prev_.size();
  bool const build_float32 = z->build_float32;
  unsigned const grd       = z->grd;
  slab_start_ = Buffer<uint32_t>(alloc, nslabs_total + 1);
  slab_edges_ = Buffer<uint32_t>(alloc, nentries);
  if (build_float32) slab_e32_ = Buffer<float4>(alloc, nentries);
  vert_x_ = Buffer<T>(alloc, nvertical);
  if (build_float32) vert_x32_ = Buffer<float>(alloc, nvertical);
  if (np == 0) CSPT_CUDA_TRY(cudaMemsetAsync(slab_start_.data(), 0, sizeof(uint32_t), s));
  Buffer<float2> vxy32(alloc, build_float32 ? nv : 0);
  if (np > 0) {
    index_fill_kernel<T><<<grd, kIdxBlock, 0, s>>>(
      po, ro, vx, vy, np, pminx_.data(), pminy_.data(), pmaxx_.data(), pmaxy_.data(),
      invh_.data(), nslab_.data(), slab_base_.data(), z->ebase.data(), vbeg_.data(), grid_.data(),
      build_float32, ax_.data(), ay_.data(), aix_.data(), aiy_.data(), box32_.data(),
      invh32_.data(), maxoff_.data(), prev_.data(), z->spans.data(), edge32_.data(),
      slab_start_.data(),
      slab_edges_.data(), slab_e32_.data(), vert_x_.data(), vert_x32_.data(), vxy32.data(),
      z->yslab.data());
    CSPT_CHECK_LAUNCH();
    vert_end_kernel<<<grid_for(np, 256, sm_grid(16u)), 256, 0, s>>>(vbeg_.data(), z->nvert.data(),
                                                                  np, vend_.data());
    CSPT_CHECK_LAUNCH();
  }
  vxy32.reset();
  bool const ordered = build_float32 && z->order_slabs;
  slab_nfull_ = Buffer<uint32_t>(alloc, ordered ? nslabs_total : 0);
  slab_bins_  = Buffer<uint32_t>(alloc, ordered ? nslabs_total * kSlabBins : 0);
  invw32_     = Buffer<float>(alloc, ordered ? np : 0);
  if (ordered && np > 0) {
    Buffer<uint32_t> edges2(alloc, nentries);
    Buffer<float4> e32b(alloc, nentries);
    slab_order_kernel<<<grd, kIdxBlock, 0, s>>>(
      np, nslab_.data(), slab_base_.data(), slab_start_.data(), exact_.data(), box32_.data(),
      slab_edges_.data(), slab_e32_.data(), edges2.data(),
      e32b.data(), slab_nfull_.data(), slab_bins_.data(), invw32_.data());
    CSPT_CHECK_LAUNCH();
    slab_edges_ = std::move(edges2);
    slab_e32_   = std::move(e32b);
  }
  z->yslab.reset();
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
                           edge32_.data(),
                           slab_nfull_.data(),
                           slab_bins_.data(),
                           invw32_.data()};
}

template class PolygonIndex<float>;
template class PolygonIndex<double>;

}  // namespace cspt
