// Unindexed point-in-polygon on sm_103a: every point against every polygon
// (at most 31, one result bit each), and the pairwise form (point i against
// polygon i).
//
// Reference: cpp/src/point_in_polygon/point_in_polygon.cu:36-150 (column API
// and validation), cpp/include/cuspatial/detail/point_in_polygon.cuh:41-140
// (pip_functor and the pairwise transform) and detail/algorithm/
// is_point_in_polygon.cuh:45-100 (the per-pair test).
//
// Bitmask form: the polygons go into the slab index (polygon_index.cuh), which
// limits each test to the edges of the point's slab; each lane holds one
// polygon's index fields in registers and the lanes of a warp cover
// (point, polygon) combinations.  With float64 input and the filtered method
// each point is placed once on the index's anchor grid (bit arithmetic, no
// float64 instruction) and the float32 filter decides each polygon, as in the
// quadtree join.
//
// Pairwise form: every polygon is used once, so no index is built; a group
// of G lanes (1, 4, 8 or 32, from the mean polygon size) walks the polygon's
// edges in parallel and combines the edge results (on-edge OR, crossing
// parity XOR), which equals the reference's sequential walk wherever its
// skipped vertices are exact repeats (polygon_index.cuh, points 1 and 2);
// polygons where that can fail (non-finite or sub-2^-1019 coordinates) are
// walked sequentially by the group's first lane.  With float64 input and the
// filtered method each vertex is moved into the point's frame in float32
// (one float64 subtraction per coordinate) and an edge falls back to the
// reference's float64 expression only where the error bound below cannot
// decide it.
#include "common.cuh"
#include "pip_test.cuh"
#include "polygon_index.cuh"

namespace cspt {
namespace {

constexpr unsigned kPointsBlock = 256;

// Places v on the power-of-two grid 2^k, from its bit pattern: q = v / 2^k
// truncated toward zero, u = fl32(v - q 2^k).  False where the split is not
// representable (non-finite or subnormal v, |v - q 2^k| below 2^-120, q
// beyond 2^62); the caller then uses the exact test.
__device__ inline bool grid_split(double v, int k, long long& q, float& u)
{
  unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(v));
  int const e                = static_cast<int>((b >> 52) & 0x7FFull);
  unsigned long long m       = b & ((1ull << 52) - 1ull);
  bool const neg             = (b >> 63) != 0ull;
  if (e == 0x7FF) return false;
  if (e == 0) {
    q = 0;
    u = 0.0f;
    return m == 0ull;  // +-0 only
  }
  m |= 1ull << 52;
  int const e2 = e - 1075;  // v = +-m 2^e2
  if (e2 < -120) return false;
  unsigned long long qq = 0, low = 0;
  if (e2 >= k) {
    if (e2 - k > 9) return false;
    qq = m << (e2 - k);
  } else {
    int const sh = k - e2;
    if (sh >= 64) {
      low = m;
    } else {
      qq  = m >> sh;
      low = m & ((1ull << sh) - 1ull);
    }
  }
  // low < 2^(k - e2): |u| < 2^k, and scaling by 2^e2 (>= 2^-120) is exact
  float const f = low ? __ull2float_rn(low) * __int_as_float((e2 + 127) << 23) : 0.0f;
  q             = neg ? -static_cast<long long>(qq) : static_cast<long long>(qq);
  u             = neg ? -f : f;
  return true;
}

// Bitmask form (pip_functor, detail/point_in_polygon.cuh:41-66): bit p of
// out[i] = point i inside polygon p.  With at most 31 polygons every lane
// keeps one polygon's index fields in registers for the whole kernel: with
// P = 2^lp >= the polygon count, lane = (slot s, polygon p) with
// p = lane % P and s = lane / P, so a warp tests 32 / P points at a time
// against all polygons; a ballot then holds each point's mask in P bits.
// Points are read (and masks written) 32 at a time, one per lane, and passed
// to the testing lanes by shuffles.
template <typename T, bool Filtered>
__global__ void __launch_bounds__(kPointsBlock)
  points_pip_kernel(T const* __restrict__ x, T const* __restrict__ y, size_t n,
                    PolygonIndexView<T> ix, uint32_t lp, int32_t* __restrict__ out,
                    unsigned long long* __restrict__ refined)
{
  int const lane       = threadIdx.x & 31;
  uint32_t const P     = 1u << lp;
  uint32_t const S     = 32u >> lp;
  uint32_t const p     = static_cast<uint32_t>(lane) & (P - 1u);
  uint32_t const slot  = static_cast<uint32_t>(lane) >> lp;
  unsigned const pbits = P == 32u ? 0xFFFFFFFFu : ((1u << P) - 1u);
  bool const has_poly  = p < ix.num_polygons;
  uint32_t nref        = 0;
  // the lane's polygon
  float4 box    = make_float4(0.f, 0.f, 0.f, 0.f);
  float mp = 0.0f, invh = 0.0f, gf = 0.0f;
  uint32_t ns = 1, slab0 = 0, vb = 0, ve = 0;
  long long aix = 0, aiy = 0;
  bool exact_poly = true, gok = false;
  int gk          = 0;
  if constexpr (Filtered) {
    double const g = *ix.grid;
    gf             = static_cast<float>(g);
    gok            = gf >= 1.17549435e-38f && gf < 1.0e30f;  // normal float grid step
    gk = static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(g)) >> 52) &
                          0x7FFull) -
         1023;
    if (has_poly) {
      box        = ix.box32[p];
      mp         = ix.max_offset[p];
      invh       = ix.inv_slab_h32[p];
      ns         = ix.num_slabs[p];
      slab0      = ix.slab_base[p];
      vb         = ix.vert_begin[p];
      ve         = ix.vert_end[p];
      aix        = ix.anchor_ix[p];
      aiy        = ix.anchor_iy[p];
      exact_poly = ix.exact_only[p] != 0;
    }
  }
  size_t const warp   = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5;
  size_t const nwarps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t base = warp * 32; base < n; base += nwarps * 32) {
    size_t const i = base + static_cast<size_t>(lane);
    T px = T{0}, py = T{0};
    if (i < n) {
      px = x[i];
      py = y[i];
    }
    long long qx = 0, qy = 0;
    float ux = 0.0f, uy = 0.0f;
    bool framed = false;
    if constexpr (Filtered)
      framed = gok && grid_split(px, gk, qx, ux) && grid_split(py, gk, qy, uy);
    int32_t mine = 0;
    for (uint32_t b = 0; b < P; ++b) {
      int const src  = static_cast<int>(b * S + slot);  // lane holding the tested point
      T const tx     = __shfl_sync(0xFFFFFFFFu, px, src);
      T const ty     = __shfl_sync(0xFFFFFFFFu, py, src);
      bool const live = has_poly && base + static_cast<size_t>(src) < n;
      bool hit        = false;
      if constexpr (Filtered) {
        long long const tqx = __shfl_sync(0xFFFFFFFFu, qx, src);
        long long const tqy = __shfl_sync(0xFFFFFFFFu, qy, src);
        float const tux     = __shfl_sync(0xFFFFFFFFu, ux, src);
        float const tuy     = __shfl_sync(0xFFFFFFFFu, uy, src);
        bool const tfr      = __shfl_sync(0xFFFFFFFFu, static_cast<int>(framed), src) != 0;
        if (live) {
          long long const dix = aix - tqx;
          long long const diy = aiy - tqy;
          bool const exact    = !tfr || exact_poly || dix <= -16777216LL || dix >= 16777216LL ||
                             diy <= -16777216LL || diy >= 16777216LL;
          if (exact) {
            ++nref;
            hit = pip_exact<double>(tx, ty, ix, p);
          } else {
            // anchor offset in grid steps: exact in float32 below 2^24 steps
            float const dx = static_cast<float>(static_cast<int>(dix)) * gf;
            float const dy = static_cast<float>(static_cast<int>(diy)) * gf;
            hit            = filtered_test<false>(
              ix, p, tux - dx, tuy - dy, mp, fmaxf(fabsf(tux), fabsf(tuy)), box, invh, 0.0f, ns,
              slab0, vb, ve,
              [&](double& ox, double& oy) {
                ox = tx;
                oy = ty;
              },
              nref);
          }
        }
      } else {
        if (live) hit = pip_exact<T>(tx, ty, ix, p);
      }
      unsigned const bal = __ballot_sync(0xFFFFFFFFu, hit);
      uint32_t const own = static_cast<uint32_t>(lane) - b * S;  // this lane's point slot
      if (own < S) mine = static_cast<int32_t>((bal >> (own * P)) & pbits);
    }
    if (i < n) out[i] = mine;
  }
  if (Filtered && refined) {
    for (int o = 16; o > 0; o >>= 1) nref += __shfl_xor_sync(0xFFFFFFFFu, nref, o);
    if (lane == 0 && nref) atomicAdd(refined, static_cast<unsigned long long>(nref));
  }
}

__device__ inline bool same_bits(double a, double b)
{
  unsigned long long const u = __double_as_longlong(a), v = __double_as_longlong(b);
  return u == v || ((u | v) << 1) == 0ull;  // equal bits, or +0 and -0
}
__device__ inline bool same_bits(float a, float b) { return a == b; }
// exponent field <= 3: |a| < 2^-1019 (double), 2^-123 (float)
__device__ inline bool tiny_bits(double a)
{
  return ((static_cast<unsigned long long>(__double_as_longlong(a)) >> 52) & 0x7FFull) <= 3ull;
}
__device__ inline bool tiny_bits(float a) { return ((__float_as_uint(a) >> 23) & 0xFFu) <= 3u; }

template <int G, typename V>
__device__ inline V group_up(unsigned gmask, V v)
{
  if constexpr (G == 1)
    return v;
  else
    return __shfl_up_sync(gmask, v, 1, G);
}
template <int G, typename V>
__device__ inline V group_last(unsigned gmask, V v)
{
  if constexpr (G == 1)
    return v;
  else
    return __shfl_sync(gmask, v, G - 1, G);
}

// Pairwise form: a group of G lanes per (point i, polygon i).  Lane g takes
// the vertices v0 + c + g of each ring; the edge ending at vertex v starts at
// v - 1 (the ring's last vertex for v0), passed from the neighbouring lane.
//
// Filtered (float64 input): a = fl32(v_a - p), b = fl32(v_b - p) with one
// rounding each (|error| <= u32 M, M = max |a|, |b|).  The reference compares
// lhs = (px - ax)(by - ay) with rhs = (bx - ax)(py - ay), whose difference is
// a_y b_x - a_x b_y; cr = fma(a_y, b_x, -a_x b_y) is within 7 u32 M^2 of it,
// the float64 roundings of lhs and rhs add 12 u64 M^2 and the 4-ULP collinear
// band 2^-49 M^2, all below eb = 2^-17 M^2 (+ 2^-120 for float32 underflow).
// The y-flags (ay > py) are the signs of a_y and b_y, exact unless zero; the
// x-range (min(ax, bx) <= px <= max(ax, bx)) is excluded when a_x and b_x
// have the same non-zero sign.  Anything else goes to the float64 edge test.
template <typename T, int G, bool Filtered>
__global__ void __launch_bounds__(kPointsBlock)
  pairwise_pip_kernel(T const* __restrict__ x, T const* __restrict__ y, size_t n,
                      uint32_t const* __restrict__ po, uint32_t const* __restrict__ ro,
                      T const* __restrict__ vx, T const* __restrict__ vy,
                      uint8_t* __restrict__ out, unsigned long long* __restrict__ refined)
{
  static_assert(G == 1 || G == 4 || G == 8 || G == 32, "group width");
  int const lane       = threadIdx.x & 31;
  int const g          = lane & (G - 1);
  unsigned const gmask = G == 32 ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  size_t const per_warp = 32 / G;
  size_t const warp     = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5;
  size_t const nwarps   = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t nref         = 0;
  for (size_t base = warp * per_warp; base < n; base += nwarps * per_warp) {
    size_t const i = base + static_cast<size_t>(lane / G);
    if (i >= n) continue;  // uniform over the group
    T const px    = x[i];
    T const py    = y[i];
    bool on       = false;
    bool within   = false;
    bool literal  = !(isfinite(px) && isfinite(py));
    uint32_t const r0 = po[i], r1 = po[i + 1];
    for (uint32_t r = r0; r < r1 && !literal; ++r) {
      uint32_t const v0 = ro[r], v1 = ro[r + 1];
      if (v1 <= v0) continue;
      // the edge into v0 starts at the ring's last vertex
      T cx = T{0}, cy = T{0};
      float cfx = 0.0f, cfy = 0.0f;
      if (g == 0) {
        cx = vx[v1 - 1];
        cy = vy[v1 - 1];
        if constexpr (Filtered) {
          cfx = static_cast<float>(cx - px);
          cfy = static_cast<float>(cy - py);
        }
      }
      for (uint32_t c = v0; c < v1; c += G) {
        uint32_t const v = c + static_cast<uint32_t>(g);
        bool const own   = v < v1;
        T const ax       = own ? vx[v] : T{0};
        T const ay       = own ? vy[v] : T{0};
        float fax = 0.0f, fay = 0.0f;
        if constexpr (Filtered) {
          fax = static_cast<float>(ax - px);
          fay = static_cast<float>(ay - py);
        }
        T bx = group_up<G>(gmask, ax), by = group_up<G>(gmask, ay);
        float fbx = group_up<G>(gmask, fax), fby = group_up<G>(gmask, fay);
        if (g == 0) {
          bx  = cx;
          by  = cy;
          fbx = cfx;
          fby = cfy;
        }
        // the next chunk's first edge starts at this chunk's last vertex
        cx  = group_last<G>(gmask, ax);
        cy  = group_last<G>(gmask, ay);
        cfx = group_last<G>(gmask, fax);
        cfy = group_last<G>(gmask, fay);
        if (!own) continue;
        bool const ex = same_bits(ax, bx), ey = same_bits(ay, by);
        if (!(isfinite(ax) && isfinite(ay)) ||
            ((ex || (tiny_bits(ax) && tiny_bits(bx))) &&
             (ey || (tiny_bits(ay) && tiny_bits(by))) && !(ex && ey))) {
          literal = true;  // the reference's skip rule needs the sequential walk
          continue;
        }
        if (ex && ey) continue;  // repeated vertex: skipped, b kept
        int ee = -1;
        if constexpr (Filtered) {
          float const m = fmaxf(fmaxf(fabsf(fax), fabsf(fay)), fmaxf(fabsf(fbx), fabsf(fby)));
          if (m < 1.152921504606847e18f) {  // 2^60: M^2 finite
            float const eb  = __fmaf_rn(7.62939453125e-06f * m, m, 7.52316384526264e-37f);
            float const cr  = __fmaf_rn(fay, fbx, -(fax * fby));
            bool const y1   = fay > 0.0f;
            bool const y0   = fby > 0.0f;
            bool const xout = (fax > 0.0f && fbx > 0.0f) || (fax < 0.0f && fbx < 0.0f);
            bool const undecided =
              fay == 0.0f || fby == 0.0f || (fabsf(cr) <= eb && (y1 != y0 || !xout));
            if (!undecided) ee = (y1 != y0 && ((cr < 0.0f) != y1)) ? 1 : 0;
          }
          if (ee < 0) ++nref;
        }
        if (ee < 0) ee = exact_edge<T>(px, py, ax, ay, bx, by);
        if (ee == 2) on = true;
        if (ee == 1) within = !within;
      }
      if constexpr (G > 1) literal = __any_sync(gmask, literal);
    }
    if constexpr (G > 1) {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) {
        on     = on | static_cast<bool>(__shfl_xor_sync(gmask, static_cast<int>(on), o, G));
        within = within != static_cast<bool>(__shfl_xor_sync(gmask, static_cast<int>(within), o, G));
        literal =
          literal | static_cast<bool>(__shfl_xor_sync(gmask, static_cast<int>(literal), o, G));
      }
    }
    if (g == 0) {
      bool hit = !on && within;
      if (literal) {
        PolygonIndexView<T> v{};
        v.poly_offsets = po;
        v.ring_offsets = ro;
        v.vx           = vx;
        v.vy           = vy;
        hit            = ring_walk<T>(px, py, v, static_cast<uint32_t>(i));
      }
      out[i] = hit ? 1 : 0;
    }
  }
  if (Filtered && refined) {
    for (int o = 16; o > 0; o >>= 1) nref += __shfl_xor_sync(0xFFFFFFFFu, nref, o);
    if (lane == 0 && nref) atomicAdd(refined, static_cast<unsigned long long>(nref));
  }
}

unsigned points_grid(size_t n)
{
  return grid_for(n, kPointsBlock, static_cast<unsigned>(num_sms()) * 8u);
}

// log2 of the lanes per point: the smallest power of two >= the polygons
uint32_t lanes_log2(size_t npoly)
{
  uint32_t lp = 0;
  while ((size_t{1} << lp) < npoly) ++lp;
  return lp;
}

template <typename T>
void bitmask(T const* x, T const* y, size_t n, uint32_t const* po, size_t npo, uint32_t const* ro,
             size_t nro, T const* vx, T const* vy, size_t nv, bool filtered, Allocator const& alloc,
             int32_t* out, uint64_t* out_refined)
{
  cudaStream_t const s = alloc.stream();
  PolygonIndex<T> index(po, npo, ro, nro, vx, vy, nv, filtered, alloc);
  uint32_t const lp = lanes_log2(npo - 1);
  Buffer<unsigned long long> refined(alloc, 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, sizeof(unsigned long long), s));
  {
    KernelTimer timer("points_pip", s);
    if (filtered) {
      if constexpr (std::is_same<T, double>::value) {
        points_pip_kernel<double, true><<<points_grid(n), kPointsBlock, 0, s>>>(
          x, y, n, index.view(), lp, out, refined.data());
      }
    } else {
      points_pip_kernel<T, false>
        <<<points_grid(n), kPointsBlock, 0, s>>>(x, y, n, index.view(), lp, out, nullptr);
    }
    CSPT_CHECK_LAUNCH();
  }
  *out_refined = filtered ? read_back(reinterpret_cast<uint64_t*>(refined.data()), s) : 0;
}

template <typename T, int G>
void launch_pairwise(T const* x, T const* y, size_t n, uint32_t const* po, uint32_t const* ro,
                     T const* vx, T const* vy, bool filtered, uint8_t* out,
                     unsigned long long* refined, cudaStream_t s)
{
  size_t const threads = n * G;
  unsigned const grd   = grid_for(threads, kPointsBlock, static_cast<unsigned>(num_sms()) * 8u);
  if (filtered) {
    if constexpr (std::is_same<T, double>::value)
      pairwise_pip_kernel<double, G, true>
        <<<grd, kPointsBlock, 0, s>>>(x, y, n, po, ro, vx, vy, out, refined);
  } else {
    pairwise_pip_kernel<T, G, false>
      <<<grd, kPointsBlock, 0, s>>>(x, y, n, po, ro, vx, vy, out, nullptr);
  }
  CSPT_CHECK_LAUNCH();
}

template <typename T>
void pairwise(T const* x, T const* y, size_t n, uint32_t const* po, uint32_t const* ro,
              T const* vx, T const* vy, size_t nv, bool filtered, Allocator const& alloc,
              uint8_t* out, uint64_t* out_refined)
{
  cudaStream_t const s = alloc.stream();
  Buffer<unsigned long long> refined(alloc, 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, sizeof(unsigned long long), s));
  // lanes per polygon from the mean vertex count
  double const mean = static_cast<double>(nv) / static_cast<double>(n);
  {
    KernelTimer timer("pairwise_pip", s);
    if (mean < 12.0)
      launch_pairwise<T, 1>(x, y, n, po, ro, vx, vy, filtered, out, refined.data(), s);
    else if (mean < 48.0)
      launch_pairwise<T, 4>(x, y, n, po, ro, vx, vy, filtered, out, refined.data(), s);
    else if (mean < 160.0)
      launch_pairwise<T, 8>(x, y, n, po, ro, vx, vy, filtered, out, refined.data(), s);
    else
      launch_pairwise<T, 32>(x, y, n, po, ro, vx, vy, filtered, out, refined.data(), s);
  }
  *out_refined = filtered ? read_back(reinterpret_cast<uint64_t*>(refined.data()), s) : 0;
}

}  // namespace

void point_in_polygon(void const* x, void const* y, size_t n, uint32_t const* po, size_t npo,
                      uint32_t const* ro, size_t nro, void const* vx, void const* vy, size_t nv,
                      cspt_dtype dtype, cspt_method method, Allocator const& alloc, int32_t* out,
                      uint64_t* out_refined)
{
  bool const filtered = method == CSPT_METHOD_FILTERED && dtype == CSPT_FLOAT64;
  if (dtype == CSPT_FLOAT64)
    bitmask<double>(static_cast<double const*>(x), static_cast<double const*>(y), n, po, npo, ro,
                    nro, static_cast<double const*>(vx), static_cast<double const*>(vy), nv,
                    filtered, alloc, out, out_refined);
  else
    bitmask<float>(static_cast<float const*>(x), static_cast<float const*>(y), n, po, npo, ro,
                   nro, static_cast<float const*>(vx), static_cast<float const*>(vy), nv, false,
                   alloc, out, out_refined);
}

void pairwise_point_in_polygon(void const* x, void const* y, size_t n, uint32_t const* po,
                               uint32_t const* ro, void const* vx, void const* vy, size_t nv,
                               cspt_dtype dtype, cspt_method method, Allocator const& alloc,
                               uint8_t* out, uint64_t* out_refined)
{
  bool const filtered = method == CSPT_METHOD_FILTERED && dtype == CSPT_FLOAT64;
  if (dtype == CSPT_FLOAT64)
    pairwise<double>(static_cast<double const*>(x), static_cast<double const*>(y), n, po, ro,
                     static_cast<double const*>(vx), static_cast<double const*>(vy), nv,
                     filtered, alloc, out, out_refined);
  else
    pairwise<float>(static_cast<float const*>(x), static_cast<float const*>(y), n, po, ro,
                    static_cast<float const*>(vx), static_cast<float const*>(vy), nv, false,
                    alloc, out, out_refined);
}

}  // namespace cspt
