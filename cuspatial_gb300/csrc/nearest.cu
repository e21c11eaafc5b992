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
#include "leaf_frame.cuh"
#include "scan.cuh"

namespace cspt {

uint64_t& last_fallbacks()
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

// ---------------------------------------------------------------------------
// float32 filter (float64 inputs)
// ---------------------------------------------------------------------------
constexpr int kSegChunk = 8;  // segments per pruning box

struct LinestringIndexView {
  long long const* aix;  // anchors in grid steps
  long long const* aiy;
  float const* maxoff;   // largest |float32 offset| of the linestring
  uint32_t const* chunk_base;
  float4 const* chunk_box;  // (minx, miny, maxx, maxy) of 8 segments, anchor frame
  float4 const* seg32;      // per segment start vertex: (ax, ay, bx, by), anchor frame
  uint8_t const* exact;     // non-finite coordinates: exact path only
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
                 long long* aix, long long* aiy, float* maxoff, float4* chunk_box, float4* seg32)
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
    }
    m = warp_max(m);
    if (lane == 0) {
      aix[l]    = static_cast<long long>(rx);
      aiy[l]    = static_cast<long long>(ry);
      maxoff[l] = m;
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

__global__ void __launch_bounds__(256)
  nearest_filtered_kernel(uint32_t const* __restrict__ group_start,
                          uint32_t const* __restrict__ ngroups_p, size_t npairs,
                          uint32_t const* __restrict__ pair_ls,
                          uint32_t const* __restrict__ pair_quad, uint32_t const* __restrict__ qlen,
                          uint32_t const* __restrict__ qoff,
                          uint32_t const* __restrict__ point_indices, size_t npi,
                          double const* __restrict__ x, double const* __restrict__ y,
                          uint32_t const* __restrict__ lso, size_t nls,
                          double const* __restrict__ lx, double const* __restrict__ ly,
                          float2 const* __restrict__ u, LeafFrame const* __restrict__ frames,
                          LinestringIndexView li, float gf, uint32_t* __restrict__ opt,
                          uint32_t* __restrict__ ols, double* __restrict__ od,
                          unsigned long long* __restrict__ fallbacks)
{
  int const lane      = threadIdx.x & 31;
  size_t const nwarps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t const ng   = *ngroups_p;
  bool const gok      = gf >= 1.17549435e-38f && gf < 1.0e30f;
  uint32_t nfb        = 0;
  for (size_t gi = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; gi < ng;
       gi += nwarps) {
    uint32_t const k0   = group_start[gi];
    uint32_t const k1   = gi + 1 < ng ? group_start[gi + 1] : static_cast<uint32_t>(npairs);
    uint32_t const quad = pair_quad[k0];
    uint32_t const len  = qlen[quad];
    uint64_t const off  = qoff[quad];
    LeafFrame const lf  = frames[gi];
    for (uint32_t c = lane; c < len; c += 32) {
      uint64_t const pos = off + c;
      if (pos >= npi) continue;
      float2 const uv = u[pos];
      bool full       = lf.nonfinite || !gok;
      // pass 1: an upper bound on the best squared distance
      float U = INFINITY;
      for (uint32_t k = k0; k < k1 && !full; ++k) {
        uint32_t const lid = pair_ls[k];
        if (lid >= nls) continue;
        long long const dix = li.aix[lid] - lf.ix, diy = li.aiy[lid] - lf.iy;
        if (li.exact[lid] || dix <= -16777216LL || dix >= 16777216LL || diy <= -16777216LL ||
            diy >= 16777216LL) {
          full = true;
          break;
        }
        float const qx = uv.x - static_cast<float>(static_cast<int>(dix)) * gf;
        float const qy = uv.y - static_cast<float>(static_cast<int>(diy)) * gf;
        float const m  = fmaxf(fmaxf(li.maxoff[lid], lf.m), fmaxf(fabsf(qx), fabsf(qy)));
        float const dm = 1.1920928955078125e-07f * m;  // 2 u32 M
        float const tol = 4.76837158203125e-07f * m;
        uint32_t const v0 = lso[lid], v1 = lso[lid + 1];
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
      bool have64 = false;
      auto load64 = [&]() {
        if (!have64) {
          uint32_t const pi = point_indices[pos];
          px                = x[pi];
          py                = y[pi];
          have64            = true;
        }
      };
      bool have = false, skipped = false, nonzero = false;
      uint32_t bid = 0;
      double bd    = 0.0;
      if (!full) {
        // pass 2: float64 on every segment that can reach U (widened so
        // that distances left out are larger even after the square root)
        float const Uw = U * 1.0000000009313226f + 7.52316384526264e-37f;
        for (uint32_t k = k0; k < k1; ++k) {
          uint32_t const lid = pair_ls[k];
          if (lid >= nls) continue;
          long long const dix = li.aix[lid] - lf.ix, diy = li.aiy[lid] - lf.iy;
          float const qx = uv.x - static_cast<float>(static_cast<int>(dix)) * gf;
          float const qy = uv.y - static_cast<float>(static_cast<int>(diy)) * gf;
          float const m  = fmaxf(fmaxf(li.maxoff[lid], lf.m), fmaxf(fabsf(qx), fabsf(qy)));
          float const dm = 1.1920928955078125e-07f * m;
          float const tol = 4.76837158203125e-07f * m;
          uint32_t const v0 = lso[lid], v1 = lso[lid + 1];
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
              load64();
              dmin = fmin(dmin, segment_dist2<double>(px, py, lx[sg], ly[sg], lx[sg + 1],
                                                      ly[sg + 1]));
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
        // only zero distances among the candidates while others were left
        // out: the winner is the nearest non-zero one, find it exactly
        if (!have || (!nonzero && skipped)) full = true;
      }
      if (full) {
        ++nfb;
        load64();
        have = false;
        for (uint32_t k = k0; k < k1; ++k) {
          uint32_t const lid = pair_ls[k];
          if (lid >= nls) continue;
          double const d = linestring_distance<double>(px, py, lx, ly, lso[lid], lso[lid + 1]);
          if (!have || take_rhs<double>(bd, bid, d, lid)) {
            bid = lid;
            bd  = d;
          }
          have = true;
        }
      }
      if (have) {
        opt[pos] = static_cast<uint32_t>(pos);
        ols[pos] = bid;
        od[pos]  = bd;
      }
    }
  }
  if (fallbacks) {
    for (int o = 16; o > 0; o >>= 1) nfb += __shfl_xor_sync(0xFFFFFFFFu, nfb, o);
    if (lane == 0 && nfb) atomicAdd(fallbacks, static_cast<unsigned long long>(nfb));
  }
}

template <typename T>
void run(uint32_t const* pair_ls, uint32_t const* pair_quad, size_t npairs,
         cspt_quadtree const* tree, uint32_t const* point_indices, size_t npi, T const* x,
         T const* y, uint32_t const* lso, size_t nlso, T const* lx, T const* ly,
         cspt_method method, Allocator const& alloc, uint32_t* opt, uint32_t* ols, T* od)
{
  cudaStream_t const s = alloc.stream();
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
      ls_fill_kernel<<<lgrd, 256, 0, s>>>(lso, nls, lx, ly, box.data(), grid.data(),
                                          cbase.data(), aix.data(), aiy.data(), maxoff.data(),
                                          cbox.data(), seg32.data());
      CSPT_CHECK_LAUNCH();
      double const g = read_back(grid.data(), s);
      // leaf frames of the groups
      Buffer<float2> u(alloc, npi);
      Buffer<LeafFrame> frames(alloc, npairs);
      leaf_frame_kernel<<<grid_for(npairs * 32, 256, sm_grid(32u)), 256, 0, s>>>(
        gs, gs + npairs, pair_quad, tree->length, qoff, point_indices, npi, x, y, grid.data(),
        u.data(), frames.data());
      CSPT_CHECK_LAUNCH();
      LinestringIndexView liv{aix.data(),   aiy.data(),  maxoff.data(), cbase.data(),
                              cbox.data(),  seg32.data(), lexact.data()};
      Buffer<unsigned long long> fb(alloc, 1);
      CSPT_CUDA_TRY(cudaMemsetAsync(fb.data(), 0, sizeof(unsigned long long), s));
      KernelTimer timer("nearest", s);
      nearest_filtered_kernel<<<grid_for(npairs * 32, 256, sm_grid(32u)), 256, 0, s>>>(
        gs, gs + npairs, npairs, pair_ls, pair_quad, tree->length, qoff, point_indices, npi, x,
        y, lso, nls, lx, ly, u.data(), frames.data(), liv, static_cast<float>(g), opt, ols, od,
        fb.data());
      CSPT_CHECK_LAUNCH();
      last_fallbacks() = read_back(fb.data(), s);
      return;
    }
  }
  size_t const ng = read_back(gs + npairs, s);
  {
    KernelTimer timer("nearest", s);
    nearest_kernel<T, false><<<grid_for(ng * 32, 256, sm_grid(32u)), 256, 0, s>>>(
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
