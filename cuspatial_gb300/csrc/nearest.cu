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
#include <memory>

#include "common.cuh"
#include "leaf_frame.cuh"
#include "scan.cuh"

namespace cspt {

uint64_t& last_fallbacks()
{
  static thread_local uint64_t n = 0;
  return n;
}
uint64_t& last_group_scans()
{
  static thread_local uint64_t n = 0;
  return n;
}
uint64_t& last_f64_segments()
{
  static thread_local uint64_t n = 0;
  return n;
}

namespace {

template <typename T>
__device__ inline T dot_fma(T ax, T ay, T bx, T by)
{
  return fma_rn(ax, bx, ay * by);
}

// (the quotient r is only formed where the result depends on it: when
// d3 <= 0 the reference's expression yields fmin(d0, d1) whatever r is)
template <typename T>
__device__ inline T segment_dist2(T px, T py, T ax, T ay, T bx, T by)
{
  T const v1x = px - ax, v1y = py - ay;
  T const v2x = px - bx, v2y = py - by;
  T const d0  = dot_fma(v1x, v1y, v1x, v1y);
  T const d1  = dot_fma(v2x, v2y, v2x, v2y);
  T const ex = bx - ax, ey = by - ay;
  T const d3  = dot_fma(px - ax, py - ay, ex, ey);
  if (d3 <= T{0}) return fmin(d0, d1);
  T const d2 = dot_fma(ex, ey, ex, ey);
  T const r  = d3 * d3 / d2;
  return r >= d2 ? fmin(d0, d1) : d0 - r;
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
                 PointSource<T> const src, size_t npi, uint32_t const* __restrict__ lso, size_t nls,
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
      T px, py;
      src.load(pos, px, py);
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

// ---------------------------------------------------------------------------
// float32 filter (float64 inputs)
// ---------------------------------------------------------------------------
constexpr int kSegChunk = 8;  // segments per pruning box

// Per linestring, what the segment listing needs in one 64-byte record.
struct __align__(16) LsRec {
  long long aix, aiy;  // anchor in grid steps
  float4 box;          // box of its float32 segments, anchor frame
  float maxoff;        // largest |float32 offset|
  uint32_t v0, nseg;   // first vertex, segments
  uint32_t cb;         // first chunk
  uint32_t exact;      // non-finite coordinates: exact path only
  uint32_t pad[3];
};
static_assert(sizeof(LsRec) == 64, "one 64-byte record per linestring");

struct LinestringIndexView {
  long long const* aix;  // anchors in grid steps
  long long const* aiy;
  float const* maxoff;   // largest |float32 offset| of the linestring
  uint32_t const* chunk_base;
  float4 const* chunk_box;  // (minx, miny, maxx, maxy) of 8 segments, anchor frame
  float4 const* seg32;      // per segment start vertex: (ax, ay, bx, by), anchor frame
  uint8_t const* exact;     // non-finite coordinates: exact path only
  LsRec const* rec;
};

// per linestring: box, anchor, float32 segments, chunk boxes (one warp each)
__global__ void __launch_bounds__(256)
  ls_box_kernel(uint32_t const* __restrict__ lso, size_t nls, double const* __restrict__ lx,
                double const* __restrict__ ly, double4_16a* __restrict__ box, uint8_t* exact,
                uint32_t* nchunks)
{
  int const lane      = threadIdx.x & 31;
  size_t const nwarps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t l = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; l < nls;
       l += nwarps) {
    uint32_t const v0 = lso[l], v1 = lso[l + 1];
    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    bool bad = false;
    for (uint32_t v = v0 + lane; v < v1; v += 32) {
      double const x = lx[v], y = ly[v];
      bad |= !(isfinite(x) && isfinite(y));
      mnx = fmin(mnx, x);
      mny = fmin(mny, y);
      mxx = fmax(mxx, x);
      mxy = fmax(mxy, y);
    }
    for (int o = 16; o > 0; o >>= 1) {
      mnx = fmin(mnx, __shfl_xor_sync(0xFFFFFFFFu, mnx, o));
      mny = fmin(mny, __shfl_xor_sync(0xFFFFFFFFu, mny, o));
      mxx = fmax(mxx, __shfl_xor_sync(0xFFFFFFFFu, mxx, o));
      mxy = fmax(mxy, __shfl_xor_sync(0xFFFFFFFFu, mxy, o));
    }
    bad = __any_sync(0xFFFFFFFFu, bad);
    if (lane == 0) {
      box[l]         = make_double4_16a(mnx, mny, mxx, mxy);
      exact[l]       = bad ? 1 : 0;
      uint32_t const ns = v1 > v0 + 1 ? v1 - v0 - 1 : 0;
      nchunks[l]     = (ns + kSegChunk - 1) / kSegChunk;
    }
  }
}

__global__ void __launch_bounds__(1024) ls_grid_kernel(double4_16a const* __restrict__ box, size_t nls,
                                                       double* grid)
{
  __shared__ double part[32];
  double m = 0;
  for (size_t l = threadIdx.x; l < nls; l += blockDim.x) {
    double4_16a const b = box[l];
    double const v[4] = {b.x, b.y, b.z, b.w};
    for (double a : v)
      if (isfinite(a)) m = fmax(m, fabs(a));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = part[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if (threadIdx.x == 0) {
      int e = 0;
      frexp(m > 0.0 ? m : 1.0, &e);
      *grid = ldexp(1.0, e - 22);
    }
  }
}

__global__ void __launch_bounds__(256)
  ls_fill_kernel(uint32_t const* __restrict__ lso, size_t nls, double const* __restrict__ lx,
                 double const* __restrict__ ly, double4_16a const* __restrict__ box,
                 double const* __restrict__ gridp, uint32_t const* __restrict__ chunk_base,
                 uint8_t const* __restrict__ exact, long long* aix, long long* aiy,
                 float* maxoff, float4* chunk_box, float4* seg32, LsRec* rec)
{
  int const lane      = threadIdx.x & 31;
  size_t const nwarps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  double const g      = *gridp;
  for (size_t l = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; l < nls;
       l += nwarps) {
    uint32_t const v0 = lso[l], v1 = lso[l + 1];
    double4_16a const b   = box[l];
    double rx = v1 > v0 ? rint((b.x + b.z) * 0.5 / g) : 0.0;
    double ry = v1 > v0 ? rint((b.y + b.w) * 0.5 / g) : 0.0;
    if (!(fabs(rx) < 4.0e18)) rx = 0.0;
    if (!(fabs(ry) < 4.0e18)) ry = 0.0;
    double const cx = rx * g, cy = ry * g;
    uint32_t const nseg = v1 > v0 + 1 ? v1 - v0 - 1 : 0;
    uint32_t const nch  = (nseg + kSegChunk - 1) / kSegChunk;
    uint32_t const cb   = chunk_base[l];
    float m             = 0.0f;
    float4 lbx          = make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
    // lane per chunk
    for (uint32_t c = lane; c < nch; c += 32) {
      float4 cbx = make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
      uint32_t const s0 = v0 + c * kSegChunk;
      uint32_t const s1 = min(s0 + kSegChunk, v0 + nseg);
      for (uint32_t sg = s0; sg < s1; ++sg) {
        float4 e;
        e.x       = static_cast<float>(lx[sg] - cx);
        e.y       = static_cast<float>(ly[sg] - cy);
        e.z       = static_cast<float>(lx[sg + 1] - cx);
        e.w       = static_cast<float>(ly[sg + 1] - cy);
        seg32[sg] = e;
        cbx.x     = fminf(cbx.x, fminf(e.x, e.z));
        cbx.y     = fminf(cbx.y, fminf(e.y, e.w));
        cbx.z     = fmaxf(cbx.z, fmaxf(e.x, e.z));
        cbx.w     = fmaxf(cbx.w, fmaxf(e.y, e.w));
        m = fmaxf(m, fmaxf(fmaxf(fabsf(e.x), fabsf(e.y)), fmaxf(fabsf(e.z), fabsf(e.w))));
      }
      chunk_box[cb + c] = cbx;
      lbx = make_float4(fminf(lbx.x, cbx.x), fminf(lbx.y, cbx.y), fmaxf(lbx.z, cbx.z),
                        fmaxf(lbx.w, cbx.w));
    }
    m     = warp_max(m);
    lbx.x = warp_min(lbx.x);
    lbx.y = warp_min(lbx.y);
    lbx.z = warp_max(lbx.z);
    lbx.w = warp_max(lbx.w);
    if (lane == 0) {
      aix[l]    = static_cast<long long>(rx);
      aiy[l]    = static_cast<long long>(ry);
      maxoff[l] = m;
      LsRec r{};
      r.aix    = static_cast<long long>(rx);
      r.aiy    = static_cast<long long>(ry);
      r.box    = lbx;
      r.maxoff = m;
      r.v0     = v0;
      r.nseg   = nseg;
      r.cb     = cb;
      r.exact  = exact[l];
      rec[l]   = r;
    }
  }
}

// float32 estimate of the reference's squared segment distance and a bound on
// |estimate - float64 value|.  With d = 2 u32 M bounding each coordinate's
// mapping error (point in the leaf frame, segment in the linestring frame,
// M the largest offset), s = |v1|, t = |e|:
//   d0, d1: 4 d s + 4 u32 s^2 (and with w = |v2| <= s + t),
//   d2: 4 d t + 4 u32 t^2, d3: 2 d (s + t) + 4 u32 s t,
//   d0 - d3^2/d2 adds r (dd3/d3 * 2 + dd2/d2), i.e. up to 4 d s^2 / t;
// the branch choice near a projection end changes the value by the square
// of those errors only (the two branches meet there).  The bound below takes
// four times their sum plus 2^-40 of the magnitudes for the float64
// rounding; t -> 0 makes it infinite, which sends the segment to float64.
__device__ inline void seg_estimate(float qx, float qy, float4 e, float dm, float& est,
                                    float& err)
{
  float const v1x = qx - e.x, v1y = qy - e.y;
  float const v2x = qx - e.z, v2y = qy - e.w;
  float const ex = e.z - e.x, ey = e.w - e.y;
  float const d0 = __fmaf_rn(v1x, v1x, v1y * v1y);
  float const d1 = __fmaf_rn(v2x, v2x, v2y * v2y);
  float const d2 = __fmaf_rn(ex, ex, ey * ey);
  float const d3 = __fmaf_rn(v1x, ex, v1y * ey);
  float const r  = d3 * d3 / d2;
  est            = (d3 <= 0.0f || r >= d2) ? fminf(d0, d1) : d0 - r;
  float const sv = sqrtf(d0), tv = sqrtf(d2);
  float const u32 = 5.960464477539063e-08f;
  err = 4.0f * (dm * (8.0f * sv + 4.0f * tv + 4.0f * d0 / tv) +
                u32 * (12.0f * d0 + 8.0f * sv * tv + 4.0f * d2)) +
        9.094947017729282e-13f * (d0 + d2) + 7.52316384526264e-37f;
  if (!(err < INFINITY)) err = INFINITY;
}

// squared distance from q to a box widened by tol, shrunk by 2^-30 relative
__device__ inline float box_lb(float qx, float qy, float4 b, float tol)
{
  float const dx = fmaxf(fmaxf(b.x - tol - qx, 0.0f), qx - b.z - tol);
  float const dy = fmaxf(fmaxf(b.y - tol - qy, 0.0f), qy - b.w - tol);
  return __fmaf_rn(dx, dx, dy * dy) * 0.9999999990686774f;
}

// squared distance between two boxes, each side widened by tol, shrunk by
// 2^-30 relative: a lower bound of box_lb for every point of box a
__device__ inline float boxbox_lb(float4 a, float4 b, float tol)
{
  float const dx = fmaxf(fmaxf(b.x - tol - a.z, 0.0f), a.x - b.z - tol);
  float const dy = fmaxf(fmaxf(b.y - tol - a.w, 0.0f), a.y - b.w - tol);
  return __fmaf_rn(dx, dx, dy * dy) * 0.9999999990686774f;
}

// Arguments of the filtered nearest-linestring kernel.
struct NearestArgs {
  uint32_t const* group_start;
  uint32_t const* ngroups_p;
  size_t npairs;
  uint32_t const* pair_ls;
  uint32_t const* pair_quad;
  uint32_t const* qlen;
  uint32_t const* qoff;
  PointSource<double> src;
  size_t npi;
  uint32_t const* lso;
  size_t nls;
  double const* lx;
  double const* ly;
  float2 const* u;
  LeafFrame const* frames;
  LinestringIndexView li;
  float gf;
  uint32_t* opt;
  uint32_t* ols;
  double* od;
  unsigned long long* stats;  // [0] points folded over every candidate, [1] groups scanned whole
  unsigned long long* next_group;
};

// The reference's fold over every candidate of the group, in float64 (the
// literal per-point loop of the reference).
__device__ inline void fold_all(NearestArgs const& a, uint32_t k0, uint32_t k1, double px,
                                double py, bool& have, uint32_t& bid, double& bd)
{
  have = false;
  for (uint32_t k = k0; k < k1; ++k) {
    uint32_t const lid = a.pair_ls[k];
    if (lid >= a.nls) continue;
    double const d = linestring_distance<double>(px, py, a.lx, a.ly, a.lso[lid], a.lso[lid + 1]);
    if (!have || take_rhs<double>(bd, bid, d, lid)) {
      bid = lid;
      bd  = d;
    }
    have = true;
  }
}

// One point against every candidate linestring of its group, chunk by chunk:
// pass 1 bounds the running minimum U with float32 estimates and chunk
// pruning, pass 2 evaluates in float64 only the segments whose estimate can
// reach U, then the fold; a point whose candidates reach only zero distances
// (or none) takes fold_all.  Used for groups the listing below cannot take.
__device__ inline void nearest_point_scan(NearestArgs const& a, uint32_t k0, uint32_t k1,
                                          LeafFrame const& lf, uint64_t pos, bool gok,
                                          uint32_t& nfb)
{
  LinestringIndexView const& li = a.li;
  float const gf  = a.gf;
  float2 const uv = a.u[pos];
  bool full       = lf.nonfinite || !gok;
  float U         = INFINITY;
  for (uint32_t k = k0; k < k1 && !full; ++k) {
    uint32_t const lid = a.pair_ls[k];
    if (lid >= a.nls) continue;
    long long const dix = li.aix[lid] - lf.ix, diy = li.aiy[lid] - lf.iy;
    if (li.exact[lid] || dix <= -16777216LL || dix >= 16777216LL || diy <= -16777216LL ||
        diy >= 16777216LL) {
      full = true;
      break;
    }
    float const qx  = uv.x - static_cast<float>(static_cast<int>(dix)) * gf;
    float const qy  = uv.y - static_cast<float>(static_cast<int>(diy)) * gf;
    float const m   = fmaxf(fmaxf(li.maxoff[lid], lf.m), fmaxf(fabsf(qx), fabsf(qy)));
    float const dm  = 1.1920928955078125e-07f * m;  // 2 u32 M
    float const tol = 4.76837158203125e-07f * m;
    uint32_t const v0 = a.lso[lid], v1 = a.lso[lid + 1];
    uint32_t const nseg = v1 > v0 + 1 ? v1 - v0 - 1 : 0;
    uint32_t const cb   = li.chunk_base[lid];
    for (uint32_t ch = 0; ch * kSegChunk < nseg; ++ch) {
      if (box_lb(qx, qy, li.chunk_box[cb + ch], tol) > U) continue;
      uint32_t const s0 = v0 + ch * kSegChunk, s1 = min(s0 + kSegChunk, v0 + nseg);
      for (uint32_t sg = s0; sg < s1; ++sg) {
        float est, err;
        seg_estimate(qx, qy, li.seg32[sg], dm, est, err);
        U = fminf(U, est + err);
      }
    }
  }
  double px = 0.0, py = 0.0;
  a.src.load(pos, px, py);
  bool have = false, skipped = false, nonzero = false;
  uint32_t bid = 0;
  double bd    = 0.0;
  if (!full) {
    // pass 2: float64 on every segment that can reach U (widened so that
    // distances left out are larger even after the square root)
    float const Uw = U * 1.0000000009313226f + 7.52316384526264e-37f;
    for (uint32_t k = k0; k < k1; ++k) {
      uint32_t const lid = a.pair_ls[k];
      if (lid >= a.nls) continue;
      long long const dix = li.aix[lid] - lf.ix, diy = li.aiy[lid] - lf.iy;
      float const qx  = uv.x - static_cast<float>(static_cast<int>(dix)) * gf;
      float const qy  = uv.y - static_cast<float>(static_cast<int>(diy)) * gf;
      float const m   = fmaxf(fmaxf(li.maxoff[lid], lf.m), fmaxf(fabsf(qx), fabsf(qy)));
      float const dm  = 1.1920928955078125e-07f * m;
      float const tol = 4.76837158203125e-07f * m;
      uint32_t const v0 = a.lso[lid], v1 = a.lso[lid + 1];
      uint32_t const nseg = v1 > v0 + 1 ? v1 - v0 - 1 : 0;
      uint32_t const cb   = li.chunk_base[lid];
      double dmin         = std::numeric_limits<double>::max();
      bool evaluated      = false;
      for (uint32_t ch = 0; ch * kSegChunk < nseg; ++ch) {
        if (box_lb(qx, qy, li.chunk_box[cb + ch], tol) > Uw) continue;
        uint32_t const s0 = v0 + ch * kSegChunk, s1 = min(s0 + kSegChunk, v0 + nseg);
        for (uint32_t sg = s0; sg < s1; ++sg) {
          float est, err;
          seg_estimate(qx, qy, li.seg32[sg], dm, est, err);
          if (est - err > Uw) continue;
          dmin = fmin(dmin, segment_dist2<double>(px, py, a.lx[sg], a.ly[sg], a.lx[sg + 1],
                                                  a.ly[sg + 1]));
          evaluated = true;
        }
      }
      if (!evaluated || !(dmin <= static_cast<double>(Uw))) {
        skipped = true;  // farther than the best: cannot win
        continue;
      }
      double const d = sqrt(dmin);
      if (!have || take_rhs<double>(bd, bid, d, lid)) {
        bid = lid;
        bd  = d;
      }
      have = true;
      nonzero |= d != 0.0;
    }
    // only zero distances among the candidates while others were left out:
    // the winner is the nearest non-zero one, find it exactly
    if (!have || (!nonzero && skipped)) full = true;
  }
  if (full) {
    ++nfb;
    fold_all(a, k0, k1, px, py, have, bid, bd);
  }
  if (have) {
    a.opt[pos] = static_cast<uint32_t>(pos);
    a.ols[pos] = bid;
    a.od[pos]  = bd;
  }
}

// The group's segment list (per warp, in shared memory): the candidate
// segments whose box lies within a radius of the leaf's point box, each in
// the leaf's float32 frame, with its global start vertex and its
// linestring, in no particular order.
constexpr int kNearWarps    = 4;    // warps per block
constexpr uint32_t kNearCap = 384;  // listed segments per warp
static_assert(kNearCap <= 65536, "candidate slots hold 16-bit list positions");
// float64 candidates per point evaluated in lockstep rounds (more are taken
// one lane at a time)
constexpr uint32_t kNearCand = 4;
struct NearList {
  float4 e[kNearCap];
  uint32_t seg[kNearCap];
  uint32_t lid[kNearCap];
};
constexpr uint32_t kListOverflow = 0xFFFFFFFEu;  // more than kNearCap segments
constexpr uint32_t kListFrame    = 0xFFFFFFFFu;  // a linestring outside the float32 frames

// Lists the segments of the group's linestrings whose box is within squared
// distance r2 of the leaf's point box (box-to-box lower bound with the
// filter's margin tol, computed in each linestring's frame; the leaf box
// maps into that frame monotonically, so it holds every point's mapped
// offset and the bound is below each point's own box_lb).  Three filters,
// each on every lane: 32 candidate linestrings at a time, each lane loading
// one linestring's 64-byte record and testing its whole box; the chunks of
// the linestrings that pass, flattened over the lanes (a lane finds its
// chunk's linestring by a binary search over the lanes' running chunk
// counts); four near chunks at a time, eight lanes per chunk, one segment
// each.  Listed segments are stored in the leaf frame, rounded once from the
// float64 vertices; mg receives the largest magnitude of the leaf frame (its
// points' and the listed segments' offsets), which bounds their errors.
// Returns the count, kListOverflow or kListFrame.
__device__ uint32_t list_segments(NearestArgs const& a, NearList& L, uint32_t k0, uint32_t k1,
                                  LeafFrame const& lf, float r2, float& mg)
{
  LinestringIndexView const& li = a.li;
  constexpr unsigned kAll       = 0xFFFFFFFFu;
  int const lane                = threadIdx.x & 31;
  unsigned const lt             = (1u << lane) - 1u;
  uint32_t n                    = 0;
  float m                       = lf.m;
  for (uint32_t kb = k0; kb < k1; kb += 32) {
    // this lane's linestring: its frame relative to the leaf and whether its
    // whole box is near the leaf box
    uint32_t const k = kb + static_cast<uint32_t>(lane);
    uint32_t lid     = 0;
    bool valid       = k < k1;
    if (valid) {
      lid   = a.pair_ls[k];
      valid = lid < a.nls;
    }
    LsRec r{};
    if (valid) r = li.rec[lid];
    bool bad = false;
    float4 lb{};
    float tol    = 0.0f;
    uint32_t nch = 0;
    if (valid) {
      long long const dix = r.aix - lf.ix, diy = r.aiy - lf.iy;
      bad = r.exact || dix <= -16777216LL || dix >= 16777216LL || diy <= -16777216LL ||
            diy >= 16777216LL;
      if (!bad) {
        float const sx = static_cast<float>(static_cast<int>(dix)) * a.gf;
        float const sy = static_cast<float>(static_cast<int>(diy)) * a.gf;
        lb             = make_float4(lf.uxmin - sx, lf.uymin - sy, lf.uxmax - sx, lf.uymax - sy);
        float const mk = fmaxf(fmaxf(r.maxoff, lf.m), fmaxf(fmaxf(fabsf(lb.x), fabsf(lb.y)),
                                                            fmaxf(fabsf(lb.z), fabsf(lb.w))));
        tol            = 4.76837158203125e-07f * mk;
        if (boxbox_lb(lb, r.box, tol) <= r2) nch = (r.nseg + kSegChunk - 1) / kSegChunk;
      }
    }
    if (__any_sync(kAll, bad)) return kListFrame;
    // running chunk counts over the lanes
    uint32_t incl = nch;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t const t = __shfl_up_sync(kAll, incl, o);
      if (lane >= o) incl += t;
    }
    uint32_t const total = __shfl_sync(kAll, incl, 31);
    for (uint32_t c0 = 0; c0 < total; c0 += 32) {
      uint32_t const c = c0 + static_cast<uint32_t>(lane);
      // the chunk's linestring: the first lane whose running count exceeds c
      int ow = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        uint32_t const v = __shfl_sync(kAll, incl, ow + step - 1);
        if (v <= c) ow += step;
      }
      ow = ow < 31 ? ow : 31;
      float4 const olb     = make_float4(__shfl_sync(kAll, lb.x, ow), __shfl_sync(kAll, lb.y, ow),
                                         __shfl_sync(kAll, lb.z, ow), __shfl_sync(kAll, lb.w, ow));
      float const otol     = __shfl_sync(kAll, tol, ow);
      uint32_t const olid  = __shfl_sync(kAll, lid, ow);
      uint32_t const ov0   = __shfl_sync(kAll, r.v0, ow);
      uint32_t const onseg = __shfl_sync(kAll, r.nseg, ow);
      uint32_t const ocb   = __shfl_sync(kAll, r.cb, ow);
      uint32_t const oinc  = __shfl_sync(kAll, incl, ow);
      uint32_t const onch  = __shfl_sync(kAll, nch, ow);
      uint32_t const ch    = c - (oinc - onch);  // the chunk within its linestring
      bool const near      = c < total && boxbox_lb(olb, li.chunk_box[ocb + ch], otol) <= r2;
      unsigned cm          = __ballot_sync(kAll, near);
      while (cm) {
        // lane l expands the (l / 8)-th remaining near chunk, segment l % 8;
        // that chunk's linestring fields are held by lane src
        unsigned mm = cm;
        for (int t = 0; t < (lane >> 3); ++t) mm &= mm - 1u;
        int const src       = mm ? __ffs(mm) - 1 : 0;
        float4 const slb    = make_float4(__shfl_sync(kAll, olb.x, src), __shfl_sync(kAll, olb.y, src),
                                          __shfl_sync(kAll, olb.z, src), __shfl_sync(kAll, olb.w, src));
        float const stol    = __shfl_sync(kAll, otol, src);
        uint32_t const slid = __shfl_sync(kAll, olid, src);
        uint32_t const sv0  = __shfl_sync(kAll, ov0, src);
        uint32_t const snsg = __shfl_sync(kAll, onseg, src);
        uint32_t const sch  = __shfl_sync(kAll, ch, src);
        uint32_t const sg   = sv0 + sch * kSegChunk + static_cast<uint32_t>(lane & 7);
        bool keep           = false;
        if (mm && sg < sv0 + snsg) {
          float4 const e   = li.seg32[sg];
          float4 const sbx = make_float4(fminf(e.x, e.z), fminf(e.y, e.w), fmaxf(e.x, e.z),
                                         fmaxf(e.y, e.w));
          keep             = boxbox_lb(slb, sbx, stol) <= r2;
        }
        unsigned const km = __ballot_sync(kAll, keep);
        if (n + __popc(km) > kNearCap) return kListOverflow;
        if (keep) {
          // the segment in the leaf frame, rounded once from the float64
          // vertices: its error is a float32 rounding of a leaf-local value,
          // not of the linestring-frame offset (which grows with the
          // linestring's extent), so the estimates' bound stays tight
          uint32_t const slot = n + __popc(km & lt);
          float4 const el     = make_float4(static_cast<float>(a.lx[sg] - lf.ax),
                                            static_cast<float>(a.ly[sg] - lf.ay),
                                            static_cast<float>(a.lx[sg + 1] - lf.ax),
                                            static_cast<float>(a.ly[sg + 1] - lf.ay));
          L.e[slot]   = el;
          L.seg[slot] = sg;
          L.lid[slot] = slid;
          m = fmaxf(m, fmaxf(fmaxf(fabsf(el.x), fabsf(el.y)), fmaxf(fabsf(el.z), fabsf(el.w))));
        }
        n += __popc(km);
        for (int t = 0; t < 4 && cm; ++t) cm &= cm - 1u;
      }
    }
  }
  __syncwarp();
  mg = warp_max(m);
  return n;
}

// An upper bound, valid for every point of the leaf, of the squared
// float64 distance to its nearest candidate segment: the smallest, over the
// candidate chunks, of the largest squared distance from the leaf box to the
// chunk's first vertex (a segment's distance is at most its start vertex's),
// each coordinate widened by the margin tol (above the mapping errors) and
// the result by 2^-20 (above the float32 rounding).  Infinite when a
// linestring lies outside the float32 frames or there is no segment.
__device__ float group_upper(NearestArgs const& a, uint32_t k0, uint32_t k1, LeafFrame const& lf)
{
  LinestringIndexView const& li = a.li;
  int const lane = threadIdx.x & 31;
  float ub       = INFINITY;
  bool frame_ok  = true;
  for (uint32_t k = k0; k < k1; ++k) {
    uint32_t const lid = a.pair_ls[k];
    if (lid >= a.nls) continue;
    long long const dix = li.aix[lid] - lf.ix, diy = li.aiy[lid] - lf.iy;
    if (li.exact[lid] || dix <= -16777216LL || dix >= 16777216LL || diy <= -16777216LL ||
        diy >= 16777216LL) {
      frame_ok = false;
      break;
    }
    float const sx  = static_cast<float>(static_cast<int>(dix)) * a.gf;
    float const sy  = static_cast<float>(static_cast<int>(diy)) * a.gf;
    float4 const lb = make_float4(lf.uxmin - sx, lf.uymin - sy, lf.uxmax - sx, lf.uymax - sy);
    float const mk  = fmaxf(fmaxf(li.maxoff[lid], lf.m),
                            fmaxf(fmaxf(fabsf(lb.x), fabsf(lb.y)), fmaxf(fabsf(lb.z), fabsf(lb.w))));
    float const tol = 4.76837158203125e-07f * mk;
    uint32_t const v0 = a.lso[lid], v1 = a.lso[lid + 1];
    uint32_t const nseg = v1 > v0 + 1 ? v1 - v0 - 1 : 0;
    for (uint32_t ch = lane; ch * kSegChunk < nseg; ch += 32) {
      float4 const e = li.seg32[v0 + ch * kSegChunk];
      float const dx = fmaxf(fabsf(e.x - lb.x), fabsf(e.x - lb.z)) + tol;
      float const dy = fmaxf(fabsf(e.y - lb.y), fabsf(e.y - lb.w)) + tol;
      ub             = fminf(ub, __fmaf_rn(dx, dx, dy * dy) * 1.0000009536743164f);
    }
  }
  ub = warp_min(ub);
  return frame_ok ? ub : INFINITY;
}

// Smallest float32 upper bound (estimate + error) of the squared distance
// from point offset (qx, qy) to the listed segments.  A segment whose box is
// farther than the running bound (box_lb, a lower bound of its distance) is
// passed over without its estimate.
__device__ inline float list_upper(NearList const& L, uint32_t n, float qx, float qy, float dm,
                                   float tol)
{
  float U = INFINITY;
  for (uint32_t t = 0; t < n; ++t) {
    float4 const e  = L.e[t];
    float4 const sb = make_float4(fminf(e.x, e.z), fminf(e.y, e.w), fmaxf(e.x, e.z),
                                  fmaxf(e.y, e.w));
    if (box_lb(qx, qy, sb, tol) > U) continue;
    float est, err;
    seg_estimate(qx, qy, e, dm, est, err);
    U = fminf(U, est + err);
  }
  return U;
}

// Whether listed segment t can reach the bound Uw from point offset
// (qx, qy): its box and then its float32 estimate (minus the estimate's
// error) are within Uw.
__device__ inline bool seg_can_reach(NearList const& L, uint32_t t, float qx, float qy, float dm,
                                     float tol, float Uw)
{
  float4 const e  = L.e[t];
  float4 const sb = make_float4(fminf(e.x, e.z), fminf(e.y, e.w), fmaxf(e.x, e.z), fmaxf(e.y, e.w));
  if (box_lb(qx, qy, sb, tol) > Uw) return false;
  float est, err;
  seg_estimate(qx, qy, e, dm, est, err);
  return !(est - err > Uw);
}

// One warp per group of pairs sharing a quadrant (handed out from a device
// counter), one lane per point.
//   1. list the segments whose box meets the leaf's point box (radius 0);
//   2. each point's float32 upper bound U over that list; r2 = the largest U
//      of the group's points: every point's nearest segment lies within r2
//      of the leaf box;
//   3. list the segments within r2 of the leaf box: a segment left out has
//      a float64 distance above r2 >= U for every point, so it can neither
//      win nor tie;
//   4. per point: U over the list, then float64 (the reference's expression)
//      on every listed segment whose estimate can reach U; the winner is the
//      smallest (distance, linestring id) among them, which is the
//      reference's fold (:279-294) whenever no distance is exactly 0.  A
//      point that reaches a zero distance (the reference then passes over
//      that linestring, whose other segments may be unlisted) or none is
//      folded over every candidate.
// A group whose list overflows, or that meets a linestring outside the
// float32 frames, a non-finite point or an unusable grid, is scanned whole
// per point (nearest_point_scan).
__global__ void __launch_bounds__(kNearWarps * 32, 6)
  nearest_filtered_kernel(NearestArgs const a)
{
  __shared__ NearList s_list[kNearWarps];
  __shared__ uint16_t s_cand[kNearWarps][kNearCand][32];
  int const lane    = threadIdx.x & 31;
  NearList& L       = s_list[threadIdx.x >> 5];
  uint32_t const ng = *a.ngroups_p;
  bool const gok    = a.gf >= 1.17549435e-38f && a.gf < 1.0e30f;
  uint32_t nfb = 0, nscan = 0, nf64 = 0;
  for (;;) {
    unsigned long long gg = 0;
    if (lane == 0) gg = atomicAdd(a.next_group, 1ull);
    uint64_t const gi = __shfl_sync(0xFFFFFFFFu, gg, 0);
    if (gi >= ng) break;
    uint32_t const k0   = a.group_start[gi];
    uint32_t const k1   = gi + 1 < ng ? a.group_start[gi + 1] : static_cast<uint32_t>(a.npairs);
    uint32_t const quad = a.pair_quad[k0];
    uint32_t const len  = a.qlen[quad];
    uint64_t const off  = a.qoff[quad];
    LeafFrame const lf  = a.frames[gi];
    bool listed         = !lf.nonfinite && gok;
    float mg            = 0.0f;
    uint32_t n          = 0;
    if (listed) {
      n = list_segments(a, L, k0, k1, lf, 0.0f, mg);
      listed = n != kListOverflow && n != kListFrame;
      if (listed && n == 0) {
        // no segment meets the leaf box: a radius from the chunks' vertices
        float const r2 = group_upper(a, k0, k1, lf);
        listed         = r2 < INFINITY;
        if (listed) {
          n      = list_segments(a, L, k0, k1, lf, r2, mg);
          listed = n != kListOverflow && n != kListFrame && n > 0;
        }
      }
    }
    if (listed) {
      float const dm  = 1.1920928955078125e-07f * mg;
      float const tol = 4.76837158203125e-07f * mg;
      float r2        = 0.0f;
      for (uint32_t c = lane; c < len; c += 32) {
        uint64_t const pos = off + c;
        if (pos >= a.npi) continue;
        float2 const uv = a.u[pos];
        r2              = fmaxf(r2, list_upper(L, n, uv.x, uv.y, dm, tol));
      }
      r2 = warp_max(r2);
      __syncwarp();  // every lane is done with the first list
      listed = r2 < INFINITY;
      if (listed) {
        n      = list_segments(a, L, k0, k1, lf, r2 * 1.0000009536743164f, mg);
        listed = n != kListOverflow && n != kListFrame && n > 0;
      }
    }
    if (!listed) {
      __syncwarp();
      ++nscan;
      for (uint32_t c = lane; c < len; c += 32) {
        uint64_t const pos = off + c;
        if (pos < a.npi) nearest_point_scan(a, k0, k1, lf, pos, gok, nfb);
      }
      __syncwarp();
      continue;
    }
    float const dm  = 1.1920928955078125e-07f * mg;
    float const tol = 4.76837158203125e-07f * mg;
    uint16_t(&cand)[kNearCand][32] = s_cand[threadIdx.x >> 5];
    for (uint32_t c0 = 0; c0 < len; c0 += 32) {
      uint64_t const pos = off + c0 + static_cast<uint32_t>(lane);
      bool const act     = c0 + static_cast<uint32_t>(lane) < len && pos < a.npi;
      // this point's candidates: the listed segments whose estimate can
      // reach U (the smallest upper bound over the list), the first
      // kNearCand of them kept in list order
      float2 const uv = act ? a.u[pos] : make_float2(0.0f, 0.0f);
      float Uw        = 0.0f;
      uint32_t nc     = 0;
      if (act) {
        float const U = list_upper(L, n, uv.x, uv.y, dm, tol);
        Uw            = U * 1.0000000009313226f + 7.52316384526264e-37f;
        for (uint32_t t = 0; t < n; ++t) {
          if (!seg_can_reach(L, t, uv.x, uv.y, dm, tol, Uw)) continue;
          if (nc < kNearCand) cand[nc][lane] = static_cast<uint16_t>(t);
          ++nc;
        }
      }
      double px = 0.0, py = 0.0;
      if (act) a.src.load(pos, px, py);
      // The float64 distance of every candidate; per segment, since a
      // linestring's distance is the smallest of its segments' (square
      // roots are monotone) and the reference's winner is the smallest
      // non-zero (distance, id): the fold needs no order.  The lanes take
      // their r-th candidates together, so each float64 instruction serves
      // every lane that has one.  A segment at distance exactly 0 makes its
      // linestring's distance 0, which the reference passes over; such a
      // point is folded over every candidate instead.
      bool have = false, zero = false;
      uint32_t bid = 0;
      double bd    = 0.0;
      double bd2   = 0.0;  // smallest squared distance so far (its root is bd)
      auto fold_seg = [&](uint32_t t) {
        uint32_t const sg = L.seg[t];
        ++nf64;
        double const d2 =
          segment_dist2<double>(px, py, a.lx[sg], a.ly[sg], a.lx[sg + 1], a.ly[sg + 1]);
        if (!(d2 <= static_cast<double>(Uw))) return;
        if (d2 == 0.0) {
          zero = true;
          return;
        }
        // a squared distance more than 2^-48 above the smallest so far has a
        // larger (rounded) square root: it can neither win nor tie, so its
        // root is not needed
        if (have && d2 > bd2 * 1.0000000000000036) return;
        double const d     = sqrt(d2);
        uint32_t const lid = L.lid[t];
        if (!have || d < bd || (d == bd && lid < bid)) {
          bd  = d;
          bid = lid;
        }
        bd2  = have ? fmin(bd2, d2) : d2;
        have = true;
      };
      uint32_t const mine   = nc < kNearCand ? nc : kNearCand;
      uint32_t const rounds = __reduce_max_sync(0xFFFFFFFFu, mine);
      __syncwarp();  // every lane's candidates are stored
      for (uint32_t r = 0; r < rounds; ++r)
        if (r < mine && !zero) fold_seg(cand[r][lane]);
      if (nc > kNearCand && !zero) {
        // more candidates than kept: the rest in list order, this lane alone
        uint32_t seen = 0;
        for (uint32_t t = 0; t < n && !zero; ++t) {
          if (!seg_can_reach(L, t, uv.x, uv.y, dm, tol, Uw)) continue;
          if (seen++ < kNearCand) continue;
          fold_seg(t);
        }
      }
      __syncwarp();  // the candidate slots are reused by the next chunk
      if (act) {
        if (!have || zero) {
          ++nfb;
          fold_all(a, k0, k1, px, py, have, bid, bd);
        }
        if (have) {
          a.opt[pos] = static_cast<uint32_t>(pos);
          a.ols[pos] = bid;
          a.od[pos]  = bd;
        }
      }
    }
    __syncwarp();  // the next group rewrites this warp's list
  }
  if (a.stats) {
    for (int o = 16; o > 0; o >>= 1) {
      nfb += __shfl_xor_sync(0xFFFFFFFFu, nfb, o);
      nf64 += __shfl_xor_sync(0xFFFFFFFFu, nf64, o);
    }
    if (lane == 0 && nfb) atomicAdd(a.stats, static_cast<unsigned long long>(nfb));
    if (lane == 0 && nscan) atomicAdd(a.stats + 1, static_cast<unsigned long long>(nscan));
    if (lane == 0 && nf64) atomicAdd(a.stats + 3, static_cast<unsigned long long>(nf64));
  }
}

template <typename T>
void run(uint32_t const* pair_ls, uint32_t const* pair_quad, size_t npairs,
         cspt_quadtree const* tree, uint32_t const* point_indices, size_t npi, T const* x,
         T const* y, uint32_t const* lso, size_t nlso, T const* lx, T const* ly,
         cspt_method method, Allocator const& alloc, uint32_t* opt, uint32_t* ols, T* od,
         T const* ordered)
{
  cudaStream_t const s = alloc.stream();
  PointSource<T> const src{point_indices, x, y, ordered};
  init_rows_kernel<<<grid_for(npi, 256, sm_grid(16u)), 256, 0, s>>>(npi, opt, ols, od, sizeof(T));
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
  size_t const nls = nlso > 0 ? nlso - 1 : 0;
  if constexpr (std::is_same<T, double>::value) {
    if (method == CSPT_METHOD_FILTERED) {
      // linestring index
      std::unique_ptr<KernelTimer> index_timer(new KernelTimer("nearest_index", s));
      Buffer<double4_16a> box(alloc, nls);
      Buffer<uint8_t> lexact(alloc, nls);
      Buffer<uint32_t> nch(alloc, nls + 1), cbase(alloc, nls + 1);
      Buffer<double> grid(alloc, 1);
      unsigned const lgrd = grid_for(nls * 32, 256, sm_grid(32u));
      ls_box_kernel<<<lgrd, 256, 0, s>>>(lso, nls, lx, ly, box.data(), lexact.data(), nch.data());
      CSPT_CHECK_LAUNCH();
      ls_grid_kernel<<<1, 1024, 0, s>>>(box.data(), nls, grid.data());
      CSPT_CHECK_LAUNCH();
      exclusive_scan<uint32_t>(nch.data(), cbase.data(), nls, cbase.data() + nls, alloc);
      size_t const nv = nls ? read_back(lso + nls, s) : 0;
      Buffer<long long> aix(alloc, nls), aiy(alloc, nls);
      Buffer<float> maxoff(alloc, nls);
      Buffer<float4> cbox(alloc, nv / kSegChunk + nls + 1), seg32(alloc, nv);
      Buffer<LsRec> lrec(alloc, nls);
      ls_fill_kernel<<<lgrd, 256, 0, s>>>(lso, nls, lx, ly, box.data(), grid.data(),
                                          cbase.data(), lexact.data(), aix.data(), aiy.data(),
                                          maxoff.data(), cbox.data(), seg32.data(), lrec.data());
      CSPT_CHECK_LAUNCH();
      double const g = read_back(grid.data(), s);
      index_timer.reset();
      // leaf frames of the groups
      Buffer<float2> u(alloc, npi);
      Buffer<LeafFrame> frames(alloc, npairs);
      std::unique_ptr<KernelTimer> frames_timer(new KernelTimer("leaf_frames", s));
      leaf_frame_kernel<<<grid_for(npairs * 32, 256, sm_grid(32u)), 256, 0, s>>>(
        gs, gs + npairs, pair_quad, tree->length, qoff, src, npi, grid.data(), u.data(),
        frames.data());
      CSPT_CHECK_LAUNCH();
      frames_timer.reset();
      LinestringIndexView liv{aix.data(),  aiy.data(),   maxoff.data(), cbase.data(),
                              cbox.data(), seg32.data(), lexact.data(), lrec.data()};
      // points folded whole, groups scanned, next group, float64 segment distances
      Buffer<unsigned long long> fb(alloc, 4);
      CSPT_CUDA_TRY(cudaMemsetAsync(fb.data(), 0, 4 * sizeof(unsigned long long), s));
      NearestArgs const na{gs,          gs + npairs,  npairs,     pair_ls,   pair_quad,
                           tree->length, qoff,        src,        npi,       lso,
                           nls,          lx,          ly,         u.data(),  frames.data(),
                           liv,          static_cast<float>(g), opt, ols,    od,
                           fb.data(),    fb.data() + 2};
      KernelTimer timer("nearest", s);
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nearest_filtered_kernel,
                                                        kNearWarps * 32, 0) != cudaSuccess ||
          per_sm < 1) {
        (void)cudaGetLastError();
        per_sm = 1;
      }
      nearest_filtered_kernel<<<grid_for(npairs * 32, kNearWarps * 32,
                                         sm_grid(static_cast<unsigned>(per_sm))),
                                kNearWarps * 32, 0, s>>>(na);
      CSPT_CHECK_LAUNCH();
      unsigned long long st[4];
      CSPT_CUDA_TRY(cudaMemcpyAsync(st, fb.data(), sizeof(st), cudaMemcpyDeviceToHost, s));
      CSPT_CUDA_TRY(cudaStreamSynchronize(s));
      last_fallbacks()     = st[0];
      last_group_scans()   = st[1];
      last_f64_segments()  = st[3];
      return;
    }
  }
  size_t const ng = read_back(gs + npairs, s);
  {
    KernelTimer timer("nearest", s);
    nearest_kernel<T, false><<<grid_for(ng * 32, 256, sm_grid(32u)), 256, 0, s>>>(
      gs, ng, npairs, pair_ls, pair_quad, tree->length, qoff, src, npi, lso, nls, lx, ly, opt,
      ols, od);
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
                                          void* od, void const* ordered)
{
  if (dtype == CSPT_FLOAT64)
    run<double>(pair_ls, pair_quad, npairs, tree, point_indices, npi,
                static_cast<double const*>(x), static_cast<double const*>(y), lso, nlso,
                static_cast<double const*>(lx), static_cast<double const*>(ly), method, alloc,
                opt, ols, static_cast<double*>(od), static_cast<double const*>(ordered));
  else
    run<float>(pair_ls, pair_quad, npairs, tree, point_indices, npi, static_cast<float const*>(x),
               static_cast<float const*>(y), lso, nlso, static_cast<float const*>(lx),
               static_cast<float const*>(ly), method, alloc, opt, ols, static_cast<float*>(od),
               static_cast<float const*>(ordered));
}

}  // namespace cspt
