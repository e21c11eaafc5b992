// Pairwise (multi)point - (multi)linestring distance and nearest points on
// sm_103a.
//
// Reference: cpp/include/cuspatial/detail/kernel/pairwise_distance.cuh:94-131
// with detail/distance/point_linestring_distance.cuh:37-60 (distance: per
// segment the smallest squared distance over the multipoint, its square
// root, the smallest over the segments), detail/point_linestring_nearest_
// points.cuh:55-110 (nearest points: the first strictly smaller squared
// distance over (point, part, segment) in order) and detail/utility/
// linestring.cuh:56-75 (the squared distance and nearest point of one
// segment); column APIs cpp/src/distance/point_linestring_distance.cu:80-110
// and cpp/src/nearest_points/point_linestring_nearest_points.cu:210-245.
//
// Layout: a group of G lanes (1, 4, 8 or 32, from the mean vertex count of a
// pair) per pair; lane g takes the segments v0+c+g of each part.  Both
// results are the minimum of per-(point, segment) values, so lanes keep a
// running best (value, then position in the reference's iteration order)
// and the group reduces it; the square root of the smallest squared
// distance equals the reference's smallest square root (the rounded square
// root is monotone).
//
// Filtered (float64 input): pass 1 estimates every squared distance in
// float32 in the point's frame (a = fl32(v - p)) with an error bound
// e = 2^-18 M^2 + 2^-120, M the segment's largest offset: moving the ends by
// u32 M changes the distance by at most u32 M, the float32 evaluation adds
// well under 32 u32 M^2 and the reference's float64 rounding under
// 2^-48 M^2.  U = the smallest estimate + e; pass 2 evaluates in float64,
// with the reference's expression, every (point, segment) whose estimate - e
// is at most U.  The float64 minimum and every tie with it are among those,
// so the result is the reference's.  Pairs with a non-finite coordinate or
// M >= 2^62 take the float64 path for every segment.
#include <limits>

#include "common.cuh"

namespace cspt {
namespace {

constexpr unsigned kPlBlock = 256;

// linestring.cuh:56-75 with the reference build's contractions: each dot
// product x1*x2 + y1*y2 as fma(x1, x2, y1*y2), a + t*ab as fma(t, ab, a).
template <typename T>
__device__ inline T segment_nearest(T cx, T cy, T ax, T ay, T bx, T by, T& nx, T& ny)
{
  T const abx = bx - ax, aby = by - ay;
  T const acx = cx - ax, acy = cy - ay;
  T const l2  = fma_rn(abx, abx, aby * aby);
  if (float_equal(l2, T{0})) {
    nx = ax;
    ny = ay;
    return fma_rn(acx, acx, acy * acy);
  }
  T const r   = fma_rn(acx, abx, acy * aby);
  T const bcx = cx - bx, bcy = cy - by;
  if (r <= T{0} || r >= l2) {
    T const dac = fma_rn(acx, acx, acy * acy);
    T const dbc = fma_rn(bcx, bcx, bcy * bcy);
    if (dac < dbc) {
      nx = ax;
      ny = ay;
      return dac;
    }
    nx = bx;
    ny = by;
    return dbc;
  }
  T const t   = r / l2;
  T const px  = fma_rn(t, abx, ax);
  T const py  = fma_rn(t, aby, ay);
  T const pcx = cx - px, pcy = cy - py;
  nx          = px;
  ny          = py;
  return fma_rn(pcx, pcx, pcy * pcy);
}

// float32 estimate of the squared distance from the origin to segment ab
// (the point's frame), the same branches as segment_nearest.
__device__ inline float segment_estimate(float ax, float ay, float bx, float by)
{
  float const abx = bx - ax, aby = by - ay;
  float const l2  = __fmaf_rn(abx, abx, aby * aby);
  float const da  = __fmaf_rn(ax, ax, ay * ay);
  if (!(l2 > 0.0f)) return da;
  float const r = -__fmaf_rn(ax, abx, ay * aby);
  if (r <= 0.0f || r >= l2) return fminf(da, __fmaf_rn(bx, bx, by * by));
  float const t  = __fdiv_rn(r, l2);
  float const px = __fmaf_rn(t, abx, ax), py = __fmaf_rn(t, aby, ay);
  return __fmaf_rn(px, px, py * py);
}

struct Best {
  double d;               // squared distance (T's value)
  unsigned long long k;   // (point, vertex) in the reference's order
  uint32_t part, seg, pt;
  double nx, ny;
};

template <typename T>
__device__ inline void offer(Best& b, T d, unsigned long long k, uint32_t pt, uint32_t part,
                             uint32_t seg, T nx, T ny)
{
  // point_linestring_nearest_points.cuh:91: strictly below the running
  // value, which starts at T's largest finite value
  if (!(d < std::numeric_limits<T>::max())) return;
  double const dd = static_cast<double>(d);
  if (dd < b.d || (dd == b.d && k < b.k)) {
    b.d    = dd;
    b.k    = k;
    b.pt   = pt;
    b.part = part;
    b.seg  = seg;
    b.nx   = static_cast<double>(nx);
    b.ny   = static_cast<double>(ny);
  }
}

template <int G>
__device__ inline void group_best(unsigned gmask, Best& b)
{
  if constexpr (G > 1) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      Best c;
      c.d    = __shfl_xor_sync(gmask, b.d, o, G);
      c.k    = __shfl_xor_sync(gmask, b.k, o, G);
      c.pt   = __shfl_xor_sync(gmask, b.pt, o, G);
      c.part = __shfl_xor_sync(gmask, b.part, o, G);
      c.seg  = __shfl_xor_sync(gmask, b.seg, o, G);
      c.nx   = __shfl_xor_sync(gmask, b.nx, o, G);
      c.ny   = __shfl_xor_sync(gmask, b.ny, o, G);
      if (c.d < b.d || (c.d == b.d && c.k < b.k)) b = c;
    }
  }
}

template <int G, typename V>
__device__ inline V group_min(unsigned gmask, V v)
{
  if constexpr (G > 1) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(gmask, v, o, G));
  }
  return v;
}

template <int G>
__device__ inline bool group_any(unsigned gmask, bool v)
{
  if constexpr (G > 1) return __any_sync(gmask, v);
  return v;
}

// Array sizes for the bounds checks: an offset that points outside its
// array records (what << 56 | index) in err and the pair is skipped.
struct Sizes {
  size_t points, part_offsets, vertices, point_geometry_offsets, linestring_geometry_offsets;
};
constexpr unsigned long long kBadPointOffset = 1, kBadVertex = 3, kBadGeometry = 4;
__device__ inline void flag(unsigned long long* err, unsigned long long what, size_t idx)
{
  atomicCAS(err, 0ull, (what << 56) | (static_cast<unsigned long long>(idx) & ((1ull << 56) - 1)));
}

// One pair per group of G lanes.  pgo / lgo null: one point / one
// linestring per pair.  Outputs may be null (distance only, or nearest
// points only).
template <typename T, int G, bool Filtered>
__global__ void __launch_bounds__(kPlBlock)
  pairwise_point_linestring_kernel(size_t n, uint32_t const* __restrict__ pgo,
                                   T const* __restrict__ x, T const* __restrict__ y,
                                   uint32_t const* __restrict__ lgo,
                                   uint32_t const* __restrict__ lpo, T const* __restrict__ lx,
                                   T const* __restrict__ ly, T* __restrict__ out_dist,
                                   int32_t* __restrict__ out_pt, int32_t* __restrict__ out_ls,
                                   int32_t* __restrict__ out_seg, T* __restrict__ out_xy,
                                   unsigned long long* __restrict__ refined, Sizes sz,
                                   unsigned long long* __restrict__ err)
{
  static_assert(G == 1 || G == 4 || G == 8 || G == 32, "group width");
  int const lane        = threadIdx.x & 31;
  uint32_t const g      = static_cast<uint32_t>(lane & (G - 1));
  unsigned const gmask  = G == 32 ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  size_t const per_warp = 32 / G;
  size_t const warp     = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5;
  size_t const nwarps   = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  T const big           = std::numeric_limits<T>::max();
  uint32_t nref         = 0;
  for (size_t base = warp * per_warp; base < n; base += nwarps * per_warp) {
    size_t const i = base + static_cast<size_t>(lane / G);
    if (i >= n) continue;  // uniform over the group
    if ((pgo && i + 1 >= sz.point_geometry_offsets) ||
        (lgo && i + 1 >= sz.linestring_geometry_offsets)) {
      if (g == 0) flag(err, kBadGeometry, i);
      continue;
    }
    uint32_t const p0 = pgo ? pgo[i] : static_cast<uint32_t>(i);
    uint32_t const p1 = pgo ? pgo[i + 1] : static_cast<uint32_t>(i + 1);
    // parts beyond the last part offset do not exist: the reference's
    // distance kernel walks vertices and maps each to its part and geometry
    // (pairwise_distance.cuh:115-121), so geometry offsets that name more
    // parts than there are select only the existing ones
    uint32_t const nparts = static_cast<uint32_t>(sz.part_offsets - 1);
    uint32_t const l1 = min(lgo ? lgo[i + 1] : static_cast<uint32_t>(i + 1), nparts);
    uint32_t const l0 = min(lgo ? lgo[i] : static_cast<uint32_t>(i), l1);
    // every index below stays inside its array, or the pair is skipped
    bool ok = p0 <= p1 && p1 <= sz.points;
    if (!ok) {
      if (g == 0) flag(err, kBadPointOffset, i);
      continue;
    }
    for (uint32_t part = l0; part < l1 && ok; ++part)
      ok = lpo[part] <= lpo[part + 1] && lpo[part + 1] <= sz.vertices;
    if (!ok) {
      if (g == 0) flag(err, kBadVertex, i);
      continue;
    }
    Best best{static_cast<double>(big), ~0ull, 0u, 0u, 0u, 0.0, 0.0};
    T dmin   = big;  // fmin over every squared distance (NaN ignored)
    bool seg_any = false;
    for (uint32_t part = l0; part < l1; ++part) seg_any |= lpo[part + 1] > lpo[part] + 1u;

    // pass 1 (filtered): the bound U
    bool exact = !Filtered;
    float U    = INFINITY;
    if constexpr (Filtered) {
      bool bad = false;
      for (uint32_t pp = p0; pp < p1; ++pp) {
        double const px = x[pp], py = y[pp];
        bad |= !(isfinite(px) && isfinite(py));
        for (uint32_t part = l0; part < l1; ++part) {
          uint32_t const s0 = lpo[part], s1 = lpo[part + 1];
          for (uint32_t v = s0 + g; v + 1 < s1; v += G) {
            double const ax = lx[v], ay = ly[v], bx = lx[v + 1], by = ly[v + 1];
            float const fax = static_cast<float>(ax - px), fay = static_cast<float>(ay - py);
            float const fbx = static_cast<float>(bx - px), fby = static_cast<float>(by - py);
            float const m =
              fmaxf(fmaxf(fabsf(fax), fabsf(fay)), fmaxf(fabsf(fbx), fabsf(fby)));
            if (!(m < 4.611686018427388e18f)) {  // 2^62, also NaN
              bad = true;
              continue;
            }
            float const e = __fmaf_rn(3.814697265625e-06f * m, m, 7.52316384526264e-37f);
            U             = fminf(U, segment_estimate(fax, fay, fbx, fby) + e);
          }
        }
      }
      exact = group_any<G>(gmask, bad);
      U     = group_min<G>(gmask, U);
    }
    // pass 2: the reference's expression where it can matter
    for (uint32_t pp = p0; pp < p1; ++pp) {
      T const px = x[pp], py = y[pp];
      for (uint32_t part = l0; part < l1; ++part) {
        uint32_t const s0 = lpo[part], s1 = lpo[part + 1];
        for (uint32_t v = s0 + g; v + 1 < s1; v += G) {
          T const ax = lx[v], ay = ly[v], bx = lx[v + 1], by = ly[v + 1];
          if constexpr (Filtered) {
            if (!exact) {
              float const fax = static_cast<float>(ax - px), fay = static_cast<float>(ay - py);
              float const fbx = static_cast<float>(bx - px), fby = static_cast<float>(by - py);
              float const m =
                fmaxf(fmaxf(fabsf(fax), fabsf(fay)), fmaxf(fabsf(fbx), fabsf(fby)));
              float const e = __fmaf_rn(3.814697265625e-06f * m, m, 7.52316384526264e-37f);
              if (segment_estimate(fax, fay, fbx, fby) - e > U) continue;
              ++nref;
            }
          }
          T nx, ny;
          T const d = segment_nearest<T>(px, py, ax, ay, bx, by, nx, ny);
          dmin      = fmin(dmin, d);
          offer<T>(best, d, (static_cast<unsigned long long>(pp - p0) << 32) | v, pp - p0,
                   part - l0, v - s0, nx, ny);
        }
      }
    }
    group_best<G>(gmask, best);
    dmin = group_min<G>(gmask, dmin);
    if (g == 0) {
      if (out_dist) out_dist[i] = seg_any ? sqrt(dmin) : big;
      if (out_seg) {
        if (out_pt) out_pt[i] = static_cast<int32_t>(best.pt);
        if (out_ls) out_ls[i] = static_cast<int32_t>(best.part);
        out_seg[i]        = static_cast<int32_t>(best.seg);
        out_xy[2 * i]     = static_cast<T>(best.nx);
        out_xy[2 * i + 1] = static_cast<T>(best.ny);
      }
    }
  }
  if (Filtered && refined) {
    for (int o = 16; o > 0; o >>= 1) nref += __shfl_xor_sync(0xFFFFFFFFu, nref, o);
    if (lane == 0 && nref) atomicAdd(refined, static_cast<unsigned long long>(nref));
  }
}

template <typename T, int G>
void launch(size_t n, uint32_t const* pgo, T const* x, T const* y, uint32_t const* lgo,
            uint32_t const* lpo, T const* lx, T const* ly, bool filtered, T* od, int32_t* opt,
            int32_t* ols, int32_t* oseg, T* oxy, unsigned long long* refined, Sizes sz,
            unsigned long long* err, cudaStream_t s)
{
  unsigned const grd = grid_for(n * G, kPlBlock, static_cast<unsigned>(num_sms()) * 8u);
  if (filtered) {
    if constexpr (std::is_same<T, double>::value)
      pairwise_point_linestring_kernel<double, G, true><<<grd, kPlBlock, 0, s>>>(
        n, pgo, x, y, lgo, lpo, lx, ly, od, opt, ols, oseg, oxy, refined, sz, err);
  } else {
    pairwise_point_linestring_kernel<T, G, false><<<grd, kPlBlock, 0, s>>>(
      n, pgo, x, y, lgo, lpo, lx, ly, od, opt, ols, oseg, oxy, nullptr, sz, err);
  }
  CSPT_CHECK_LAUNCH();
}

template <typename T>
void run(size_t n, uint32_t const* pgo, T const* x, T const* y, size_t np, uint32_t const* lgo,
         uint32_t const* lpo, T const* lx, T const* ly, size_t nv, Sizes sz, bool filtered,
         Allocator const& alloc, T* od, int32_t* opt, int32_t* ols, int32_t* oseg, T* oxy,
         uint64_t* out_refined)
{
  cudaStream_t const s = alloc.stream();
  Buffer<unsigned long long> refined(alloc, 2);  // [0] refined, [1] bounds error
  CSPT_CUDA_TRY(cudaMemsetAsync(refined.data(), 0, 2 * sizeof(unsigned long long), s));
  unsigned long long* err = refined.data() + 1;
  // lanes per pair from the mean work of a pair (points x vertices)
  double const mean = static_cast<double>(nv) * static_cast<double>(np ? np : 1) /
                      (static_cast<double>(n) * static_cast<double>(n));
  {
    KernelTimer timer("pairwise_point_linestring", s);
    if (mean < 12.0)
      launch<T, 1>(n, pgo, x, y, lgo, lpo, lx, ly, filtered, od, opt, ols, oseg, oxy,
                   refined.data(), sz, err, s);
    else if (mean < 48.0)
      launch<T, 4>(n, pgo, x, y, lgo, lpo, lx, ly, filtered, od, opt, ols, oseg, oxy,
                   refined.data(), sz, err, s);
    else if (mean < 160.0)
      launch<T, 8>(n, pgo, x, y, lgo, lpo, lx, ly, filtered, od, opt, ols, oseg, oxy,
                   refined.data(), sz, err, s);
    else
      launch<T, 32>(n, pgo, x, y, lgo, lpo, lx, ly, filtered, od, opt, ols, oseg, oxy,
                    refined.data(), sz, err, s);
  }
  unsigned long long h[2];
  CSPT_CUDA_TRY(cudaMemcpyAsync(h, refined.data(), sizeof h, cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[1]) {
    static char const* const what[] = {"", "point geometry offsets", "",
                                       "linestring part offsets", "geometry offsets"};
    unsigned const w = static_cast<unsigned>(h[1] >> 56);
    throw Error{CSPT_INVALID_ARGUMENT,
                std::string("offsets out of range (") + (w < 5 ? what[w] : "?") + ") at pair " +
                  std::to_string(h[1] & ((1ull << 56) - 1))};
  }
  *out_refined = filtered ? h[0] : 0;
}

}  // namespace

void pairwise_point_linestring(size_t n, uint32_t const* pgo, size_t npgo, void const* x,
                               void const* y, size_t np, uint32_t const* lgo, size_t nlgo,
                               uint32_t const* lpo, size_t nlpo, void const* lx, void const* ly,
                               size_t nv, cspt_dtype dtype, cspt_method method,
                               Allocator const& alloc, void* od, int32_t* opt, int32_t* ols,
                               int32_t* oseg, void* oxy, uint64_t* out_refined)
{
  bool const filtered = method == CSPT_METHOD_FILTERED && dtype == CSPT_FLOAT64;
  Sizes const sz{np, nlpo, nv, npgo, nlgo};
  if (dtype == CSPT_FLOAT64)
    run<double>(n, pgo, static_cast<double const*>(x), static_cast<double const*>(y), np, lgo,
                lpo, static_cast<double const*>(lx), static_cast<double const*>(ly), nv, sz,
                filtered, alloc, static_cast<double*>(od), opt, ols, oseg,
                static_cast<double*>(oxy), out_refined);
  else
    run<float>(n, pgo, static_cast<float const*>(x), static_cast<float const*>(y), np, lgo, lpo,
               static_cast<float const*>(lx), static_cast<float const*>(ly), nv, sz, false, alloc,
               static_cast<float*>(od), opt, ols, oseg, static_cast<float*>(oxy), out_refined);
}

}  // namespace cspt
