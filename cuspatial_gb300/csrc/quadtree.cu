// Morton-key point quadtree on sm_103a.
//
// Reference: cpp/include/cuspatial/detail/point_quadtree.cuh:190-272 (clamps,
// construct_quadtree), detail/index/construction/phase_1.cuh:60-381 (keys,
// sort, bottom-up levels) and phase_2.cuh:56-345 (pruning, offsets).
//
// The reference builds every level bottom-up with reduce_by_key and then
// prunes.  Here the tree is read directly off the sorted keys: position i of
// the sorted key array starts a node at level l exactly when the keys at i-1
// and i differ in their level-l prefix, i.e. when l >= lvl[i] with
// lvl[i] = max(0, d-1 - floor(msb(key[i] ^ key[i-1]) / 2)).  One scan per
// level ranks those starts; node sizes are differences of starts, child
// counts are differences of next-level ranks, and a node at level l >= 1 is
// kept iff its parent holds more than max_size points — the reference's
// remove_unqualified_quads rule (phase_2.cuh:206-236).  Leaves keep the first
// sorted position they cover, which is what the reference's flattened-key
// scan (phase_2.cuh:98-141) produces.
#include <functional>
#include <limits>
#include <vector>

#include "common.cuh"
#include "radix_sort.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

constexpr uint8_t kNoStart = 0xFF;

// phase_1.cuh:73-85: out-of-box points take the last key of the deepest
// level; others interleave the truncated cell coordinates.
template <typename T>
__global__ void morton_keys_kernel(T const* __restrict__ x, T const* __restrict__ y, size_t n,
                                   T minx, T miny, T maxx, T maxy, T scale, T rscale, int d,
                                   uint32_t* __restrict__ keys, T* __restrict__ xy)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    T const px = x[i], py = y[i];
    if (xy) {  // the points interleaved, in input order (for the ordered copy)
      if constexpr (sizeof(T) == 8)
        reinterpret_cast<double2*>(xy)[i] = make_double2(px, py);
      else
        reinterpret_cast<float2*>(xy)[i] = make_float2(px, py);
    }
    uint32_t k;
    if (outside_closed(px, minx, maxx) || outside_closed(py, miny, maxy)) {
      k = static_cast<uint32_t>((1 << (2 * d)) - 1);
    } else {
      uint16_t const cx = cell_of_quotient(px - minx, scale, rscale);
      uint16_t const cy = cell_of_quotient(py - miny, scale, rscale);
      k                 = (spread16(cy) << 1) | spread16(cx);
    }
    keys[i] = k;
  }
}

__global__ void start_level_kernel(uint32_t const* __restrict__ skeys, size_t n, int d,
                                   uint8_t* __restrict__ lvl)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint8_t l = 0;
    if (i > 0) {
      uint32_t const diff = skeys[i] ^ skeys[i - 1];
      if (diff == 0) {
        l = kNoStart;
      } else {
        int const h  = 31 - __clz(diff);
        int const lv = d - 1 - h / 2;
        l            = static_cast<uint8_t>(lv < 0 ? 0 : lv);
      }
    }
    lvl[i] = l;
  }
}

// sizes of the nodes of one level: count[k] = start[k+1] - start[k]
__global__ void node_count_kernel(uint32_t const* __restrict__ starts, size_t nl, size_t n,
                                  uint32_t* __restrict__ count)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < nl;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    size_t const e = (k + 1 < nl) ? starts[k + 1] : n;
    count[k]       = static_cast<uint32_t>(e - starts[k]);
  }
}

// finest level (d-1): every position whose key differs from its predecessor
// Histogram of the start levels: hist[v] = positions whose coarsest start
// level is v (kNoStart is not counted; v < d <= 16).  Level l has
// sum_{v <= l} hist[v] nodes, so one read gives every level's size.
__global__ void __launch_bounds__(256)
  level_histogram_kernel(uint8_t const* __restrict__ lvl, size_t n, uint32_t* __restrict__ hist)
{
  uint32_t c[16];
#pragma unroll
  for (int b = 0; b < 16; ++b) c[b] = 0;
  size_t const stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  size_t const tid    = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
  size_t const n4     = n / 4;
  uint32_t const* l4  = reinterpret_cast<uint32_t const*>(lvl);
  for (size_t i = tid; i < n4; i += stride) {
    uint32_t const w = l4[i];
#pragma unroll
    for (int b = 0; b < 16; ++b) c[b] += __popc(__vcmpeq4(w, 0x01010101u * b)) >> 3;
  }
  for (size_t i = n4 * 4 + tid; i < n; i += stride) {
    uint32_t const v = lvl[i];
#pragma unroll
    for (int b = 0; b < 16; ++b) c[b] += v == static_cast<uint32_t>(b) ? 1u : 0u;
  }
  __shared__ uint32_t sh[16];
  if (threadIdx.x < 16) sh[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    uint32_t const w = __reduce_add_sync(0xFFFFFFFFu, c[b]);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&sh[b], w);
  }
  __syncthreads();
  if (threadIdx.x < 16 && sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

struct FinestStart {
  uint8_t const* lvl;
  __device__ uint32_t operator()(size_t i) const { return lvl[i] != kNoStart ? 1u : 0u; }
};
struct FinestStore {
  uint8_t const* lvl;
  uint32_t* S;
  uint8_t* LV;
  __device__ void operator()(size_t i, uint32_t e, uint32_t f) const
  {
    if (f) {
      S[e]  = static_cast<uint32_t>(i);
      LV[e] = lvl[i];
    }
  }
};
// level l from level l+1: the starts whose lvl is <= l
struct CoarserStart {
  uint8_t const* LV;
  int l;
  __device__ uint32_t operator()(size_t k) const
  {
    return static_cast<int>(LV[k]) <= l ? 1u : 0u;
  }
};
struct CoarserStore {
  uint32_t const* FS;
  uint8_t const* FLV;
  uint32_t* S;
  uint32_t* X;
  uint8_t* LV;
  uint32_t* FP;
  __device__ void operator()(size_t k, uint32_t e, uint32_t f) const
  {
    if (f) {
      S[e]  = FS[k];
      X[e]  = static_cast<uint32_t>(k);
      LV[e] = FLV[k];
    }
    FP[k] = e + f - 1u;  // the level-l node holding level-(l+1) start k
  }
};

// Point counts, child counts and the keep rule of one level's nodes.  A
// level-l node (l >= 1) survives iff its parent holds more than max_size
// points (phase_2.cuh:206-236).
__global__ void level_nodes_kernel(uint32_t const* __restrict__ S, uint32_t const* __restrict__ X,
                                   size_t nl, size_t n, size_t n_finer,
                                   uint32_t const* __restrict__ P,
                                   uint32_t const* __restrict__ parent_count, uint32_t max_size,
                                   uint32_t* __restrict__ count, uint32_t* __restrict__ child,
                                   uint8_t* __restrict__ keep)
{
  for (size_t j = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; j < nl;
       j += static_cast<size_t>(gridDim.x) * blockDim.x) {
    size_t const e = j + 1 < nl ? S[j + 1] : n;
    count[j]       = static_cast<uint32_t>(e - S[j]);
    if (child) {
      size_t const ce = j + 1 < nl ? X[j + 1] : n_finer;
      child[j]        = static_cast<uint32_t>(ce - X[j]);
    }
    keep[j] = P ? (parent_count[P[j]] > max_size ? 1 : 0) : 1;
  }
}

__global__ void compact_nodes_kernel(size_t nl, uint8_t const* __restrict__ keep,
                                     uint32_t const* __restrict__ pos,
                                     uint32_t const* __restrict__ S,
                                     uint32_t const* __restrict__ count,
                                     uint32_t const* __restrict__ child,
                                     uint32_t const* __restrict__ skeys, int shift,
                                     uint32_t* __restrict__ okey, uint32_t* __restrict__ ocount,
                                     uint32_t* __restrict__ ochild, uint32_t* __restrict__ ostart)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < nl;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    if (!keep[k]) continue;
    uint32_t const o = pos[k];
    okey[o]          = skeys[S[k]] >> shift;
    ocount[o]        = count[k];
    ochild[o]        = child ? child[k] : 0u;
    ostart[o]        = S[k];
  }
}

struct LevelNodes {
  Buffer<uint32_t> key, count, child, start;
  size_t size = 0;
};

__global__ void assemble_kernel(uint32_t const* __restrict__ key, uint32_t const* __restrict__ cnt,
                                uint32_t const* __restrict__ child,
                                uint32_t const* __restrict__ start, size_t nk, uint8_t level,
                                bool may_be_internal, uint32_t max_size, size_t out_base,
                                uint32_t* __restrict__ okey, uint8_t* __restrict__ olevel,
                                uint8_t* __restrict__ ointernal, uint32_t* __restrict__ olength,
                                uint32_t* __restrict__ ooffset,
                                uint32_t* __restrict__ internal_children)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < nk;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    size_t const o      = out_base + k;
    bool const internal = may_be_internal && cnt[k] > max_size;
    okey[o]             = key[k];
    olevel[o]           = level;
    ointernal[o]        = internal ? 1 : 0;
    olength[o]          = internal ? child[k] : cnt[k];
    ooffset[o]          = start[k];
    internal_children[o] = internal ? child[k] : 0u;
  }
}

__global__ void internal_offset_kernel(uint8_t const* __restrict__ internal,
                                       uint32_t const* __restrict__ child_pos, size_t q,
                                       uint32_t level_1_size, uint32_t* __restrict__ offset)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < q;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    if (internal[k]) offset[k] = child_pos[k] + level_1_size;
  }
}

// rows of an interleaved point array in quadtree order: dst[p] = src[pi[p]]
// (pi a permutation of [0, n)), four independent 16-byte (float64) or 8-byte
// (float32) gathers in flight per thread.
template <typename V>
__global__ void __launch_bounds__(256)
  gather_rows_kernel(uint32_t const* __restrict__ pi, size_t n, V const* __restrict__ src,
                     V* __restrict__ dst)
{
  constexpr int kPer = 4;
  size_t const step  = static_cast<size_t>(gridDim.x) * blockDim.x * kPer;
  for (size_t b = static_cast<size_t>(blockIdx.x) * blockDim.x * kPer + threadIdx.x; b < n;
       b += step) {
    uint32_t i[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      size_t const p = b + static_cast<size_t>(j) * blockDim.x;
      i[j]           = p < n ? pi[p] : 0u;
    }
    V v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      size_t const p = b + static_cast<size_t>(j) * blockDim.x;
      if (p < n && i[j] < n) v[j] = src[i[j]];
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      size_t const p = b + static_cast<size_t>(j) * blockDim.x;
      if (p < n && i[j] < n) dst[p] = v[j];
    }
  }
}

// Host input: the points are copied from host memory (hx, hy) into the
// caller's device arrays (dx, dy, which build() then reads as x and y) in
// chunks on a second stream, and the Morton keys of each chunk are computed
// as soon as its copy has landed.  after_copies (may be null) is called with
// that stream once the points' copies are enqueued, so that a caller can
// queue more work behind them.
template <typename T>
struct HostInput {
  T const* hx;
  T const* hy;
  T* dx;
  T* dy;
  std::function<void(cudaStream_t)> const* after_copies;
};
constexpr size_t kHostChunks = 8;

template <typename T>
void build(T const* x, T const* y, size_t n, double x1d, double x2d, double y1d, double y2d,
           double scaled, int max_depth_in, int32_t max_size_in, Allocator const& alloc,
           uint32_t** out_point_indices, cspt_quadtree* out, HostInput<T> const* host = nullptr,
           T* ordered = nullptr)
{
  cudaStream_t const s = alloc.stream();
  *out                 = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
  *out_point_indices   = nullptr;
  if (n == 0) return;
  CSPT_EXPECTS(n < (size_t{1} << 32), "quadtree_on_points supports fewer than 2^32 points");

  // detail/point_quadtree.cuh:258-268 — order the corners, clamp the
  // parameters (in the coordinate type, as the reference does).
  T const x1 = static_cast<T>(x1d), x2 = static_cast<T>(x2d);
  T const y1 = static_cast<T>(y1d), y2 = static_cast<T>(y2d);
  T const minx = x1 < x2 ? x1 : x2, maxx = x1 < x2 ? x2 : x1;
  T const miny = y1 < y2 ? y1 : y2, maxy = y1 < y2 ? y2 : y1;
  uint32_t const max_size = static_cast<uint32_t>(max_size_in < 1 ? 1 : max_size_in);
  int const d             = max_depth_in < 0 ? 0 : (max_depth_in > 15 ? 15 : max_depth_in);
  T const span            = (maxx - minx) > (maxy - miny) ? (maxx - minx) : (maxy - miny);
  T const min_scale       = span / static_cast<T>((1 << d) + 2);
  T scale                 = static_cast<T>(scaled);
  scale                   = scale > min_scale ? scale : min_scale;

  unsigned const blk = 256;
  unsigned const grd = grid_for(n, blk, sm_grid(16u));
  KernelTimer timer("quadtree_build", s);

  Buffer<uint32_t> keys(alloc, n), keys_alt(alloc, n);
  Buffer<uint32_t> idx(alloc, n), idx_alt(alloc, n);
  // ordered copy requested: the key pass also writes the points interleaved
  // (input order), so the gather after the sort reads one vector per point
  Buffer<T> xy_in(alloc, ordered ? 2 * n : 0);
  T* const xy0 = ordered ? xy_in.data() : nullptr;
  // cells reach 2^d + 2, so the key needs 2(d+1) bits (2(d+2) below d = 2)
  int const key_bits = d >= 2 ? 2 * d + 2 : 2 * d + 4;
  int const sort_bits = key_bits > 32 ? 32 : key_bits;
  bool alt = false;
  bool sorted = false;
  if (!host) {
    KernelTimer kt("quadtree_keys", s);
    morton_keys_kernel<T><<<grd, blk, 0, s>>>(x, y, n, minx, miny, maxx, maxy, scale,
                                              T{1} / scale, d, keys.data(), xy0);
    CSPT_CHECK_LAUNCH();
  } else {
    cudaStream_t const copy = side_stream();
    StreamJoin copies(s, copy);  // before `keys` is released, also on an exception
    stream_wait(copy, s);        // the destinations may come from work on s
    size_t const nch = std::max<size_t>(1, std::min<size_t>(kHostChunks, n >> 20));
    // With several chunks each is sorted as soon as its keys exist, while
    // the next chunks are still crossing the link; the sorted chunks are
    // then merged (stable: equal keys keep their input order), which leaves
    // a short merge instead of the whole sort after the last copy.
    std::vector<size_t> runs{0};
    bool chunk_alt = false;
    for (size_t c = 0; c < nch; ++c) {
      size_t const i0 = n * c / nch, m = n * (c + 1) / nch - i0;
      CSPT_CUDA_TRY(cudaMemcpyAsync(host->dx + i0, host->hx + i0, m * sizeof(T),
                                    cudaMemcpyHostToDevice, copy));
      CSPT_CUDA_TRY(cudaMemcpyAsync(host->dy + i0, host->hy + i0, m * sizeof(T),
                                    cudaMemcpyHostToDevice, copy));
      stream_wait(s, copy);
      morton_keys_kernel<T><<<grid_for(m, blk, sm_grid(16u)), blk, 0, s>>>(
        x + i0, y + i0, m, minx, miny, maxx, maxy, scale, T{1} / scale, d, keys.data() + i0,
        xy0 ? xy0 + 2 * i0 : nullptr);
      CSPT_CHECK_LAUNCH();
      if (nch > 1) {
        chunk_alt = radix_sort_pairs<uint32_t>(keys.data() + i0, idx.data() + i0,
                                               keys_alt.data() + i0, idx_alt.data() + i0, m, 0,
                                               sort_bits, true, alloc,
                                               static_cast<uint32_t>(i0));
        runs.push_back(i0 + m);
      }
    }
    if (host->after_copies) (*host->after_copies)(copy);
    copies.join();
    if (nch > 1) {
      KernelTimer kt("quadtree_sort", s);
      // every chunk took the same number of passes, so all runs sit in the
      // same pair of buffers
      bool const moved = chunk_alt ? merge_sorted_runs<uint32_t>(keys_alt.data(), idx_alt.data(),
                                                                keys.data(), idx.data(), runs, s)
                                   : merge_sorted_runs<uint32_t>(keys.data(), idx.data(),
                                                                keys_alt.data(), idx_alt.data(),
                                                                runs, s);
      alt    = chunk_alt != moved;
      sorted = true;
    }
  }
  if (!sorted) {
    KernelTimer kt("quadtree_sort", s);
    alt = radix_sort_pairs<uint32_t>(keys.data(), idx.data(), keys_alt.data(), idx_alt.data(), n,
                                     0, sort_bits, true, alloc);
  }
  Buffer<uint32_t>& skeys = alt ? keys_alt : keys;
  Buffer<uint32_t>& sidx  = alt ? idx_alt : idx;
  (alt ? keys : keys_alt).reset();
  // The ordered copy needs only the permutation: the gather (bound by
  // memory) runs on a second stream beside the levels (a chain of small
  // launches), and the caller's stream waits for it before the build returns
  // and before the interleaved input is released (order_join is destroyed
  // before xy_in, also on an exception).
  cudaStream_t const os = ordered ? side_stream() : nullptr;
  StreamJoin order_join(s, os);
  if (ordered) {
    stream_wait(os, s);  // the permutation and the interleaved input are on s
    KernelTimer kt("quadtree_order", os);
    unsigned const og = grid_for((n + 3) / 4, 256, sm_grid(8u));
    if constexpr (sizeof(T) == 8)
      gather_rows_kernel<double2><<<og, 256, 0, os>>>(
        sidx.data(), n, reinterpret_cast<double2 const*>(xy0), reinterpret_cast<double2*>(ordered));
    else
      gather_rows_kernel<float2><<<og, 256, 0, os>>>(
        sidx.data(), n, reinterpret_cast<float2 const*>(xy0), reinterpret_cast<float2*>(ordered));
    CSPT_CHECK_LAUNCH();
  }

  KernelTimer levels_timer("quadtree_levels", s);
  Buffer<uint8_t> lvl(alloc, n);
  start_level_kernel<<<grd, blk, 0, s>>>(skeys.data(), n, d, lvl.data());
  CSPT_CHECK_LAUNCH();

  Buffer<uint32_t> total(alloc, 1);
  uint8_t const* lv = lvl.data();

  if (d <= 1) {
    // detail/point_quadtree.cuh:155-188: a tree of the bottom quadrants only
    Buffer<uint32_t> starts(alloc, n);
    uint32_t* st = starts.data();
    scan_apply<uint32_t>(
      [lv] __device__(size_t i) { return lv[i] != kNoStart ? 1u : 0u; },
      [lv, st] __device__(size_t i, uint32_t e, uint32_t f) {
        if (f) st[e] = static_cast<uint32_t>(i);
      },
      n, total.data(), alloc);
    size_t const q = read_back(total.data(), s);
    Buffer<uint32_t> okey(alloc, q), olen(alloc, q), ooff(alloc, q);
    Buffer<uint8_t> olev(alloc, q), oint(alloc, q);
    node_count_kernel<<<grid_for(q, blk, sm_grid(16u)), blk, 0, s>>>(st, q, n, olen.data());
    CSPT_CHECK_LAUNCH();
    uint32_t const* sk = skeys.data();
    uint32_t* ok       = okey.data();
    uint32_t* oo       = ooff.data();
    scan_apply<uint32_t>([] __device__(size_t) { return 1u; },
                         [sk, st, ok, oo] __device__(size_t k, uint32_t, uint32_t) {
                           ok[k] = sk[st[k]];
                           oo[k] = st[k];
                         },
                         q, static_cast<uint32_t*>(nullptr), alloc);
    CSPT_CUDA_TRY(cudaMemsetAsync(olev.data(), 0, q, s));
    CSPT_CUDA_TRY(cudaMemsetAsync(oint.data(), 0, q, s));
    *out_point_indices = sidx.release();
    *out = cspt_quadtree{okey.release(), olev.release(), oint.release(), olen.release(),
                         ooff.release(), q};
    return;
  }

  // Levels, bottom-up.  A position starts a level-l node iff lvl <= l, so
  // the level-l starts are the level-(l+1) starts whose lvl is <= l: each
  // level is ranked by a scan over the next finer level only (about 1.3 N
  // elements in all instead of d N).  For a level-l node j: S = first sorted
  // position, X = its index among the level-(l+1) starts; for a level-(l+1)
  // start k: P = the level-l node holding it (its parent).  Every level's
  // size comes from one histogram of lvl, and the kept nodes of all levels
  // are counted on the device and read once: the host waits twice in all.
  std::vector<size_t> level_size(d);
  {
    Buffer<uint32_t> hist(alloc, 16);
    CSPT_CUDA_TRY(cudaMemsetAsync(hist.data(), 0, 16 * sizeof(uint32_t), s));
    level_histogram_kernel<<<grid_for((n + 3) / 4, blk, sm_grid(8u)), blk, 0, s>>>(lv, n,
                                                                                  hist.data());
    CSPT_CHECK_LAUNCH();
    uint32_t h[16];
    CSPT_CUDA_TRY(cudaMemcpyAsync(h, hist.data(), sizeof(h), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    size_t run = 0;
    for (int l = 0; l < d; ++l) level_size[l] = run += h[l];
  }
  struct Raw {
    Buffer<uint32_t> S, X, P, count;
    Buffer<uint8_t> LV;
    size_t n = 0;
  };
  std::vector<Raw> raw(d);
  {
    Raw& R = raw[d - 1];
    R.S    = Buffer<uint32_t>(alloc, level_size[d - 1]);
    R.LV   = Buffer<uint8_t>(alloc, level_size[d - 1]);
    scan_apply<uint32_t>(FinestStart{lv}, FinestStore{lv, R.S.data(), R.LV.data()}, n,
                         static_cast<uint32_t*>(nullptr), alloc);
    R.n = level_size[d - 1];
  }
  for (int l = d - 2; l >= 0; --l) {
    Raw& F = raw[l + 1];
    Raw& R = raw[l];
    R.n    = level_size[l];
    R.S    = Buffer<uint32_t>(alloc, R.n);
    R.X    = Buffer<uint32_t>(alloc, R.n);
    R.LV   = Buffer<uint8_t>(alloc, R.n);
    F.P    = Buffer<uint32_t>(alloc, F.n);
    scan_apply<uint32_t>(CoarserStart{F.LV.data(), l},
                         CoarserStore{F.S.data(), F.LV.data(), R.S.data(), R.X.data(),
                                      R.LV.data(), F.P.data()},
                         F.n, static_cast<uint32_t*>(nullptr), alloc);
    F.LV.reset();
  }
  raw[0].LV.reset();
  size_t const level_1_size = raw[0].n;
  std::vector<LevelNodes> levels(d);
  Buffer<uint32_t> kept(alloc, d);  // kept nodes per level
  for (int l = 0; l < d; ++l) {
    Raw& R        = raw[l];
    size_t const nl = R.n;
    R.count       = Buffer<uint32_t>(alloc, nl);
    Buffer<uint32_t> child(alloc, l + 1 < d ? nl : 0);
    Buffer<uint8_t> keep(alloc, nl);
    if (nl) {
      level_nodes_kernel<<<grid_for(nl, blk, sm_grid(16u)), blk, 0, s>>>(
        R.S.data(), R.X.data(), nl, n, l + 1 < d ? raw[l + 1].n : 0, l > 0 ? R.P.data() : nullptr,
        l > 0 ? raw[l - 1].count.data() : nullptr, max_size, R.count.data(),
        l + 1 < d ? child.data() : nullptr, keep.data());
      CSPT_CHECK_LAUNCH();
    }
    // compact the kept nodes of the level (at most nl of them)
    LevelNodes& L = levels[l];
    Buffer<uint32_t> pos(alloc, nl);
    uint8_t const* kp = keep.data();
    uint32_t* ps      = pos.data();
    scan_apply<uint32_t>([kp] __device__(size_t k) { return static_cast<uint32_t>(kp[k]); },
                         [ps] __device__(size_t k, uint32_t e, uint32_t) { ps[k] = e; }, nl,
                         kept.data() + l, alloc);
    L.key   = Buffer<uint32_t>(alloc, nl);
    L.count = Buffer<uint32_t>(alloc, nl);
    L.child = Buffer<uint32_t>(alloc, nl);
    L.start = Buffer<uint32_t>(alloc, nl);
    if (nl) {
      compact_nodes_kernel<<<grid_for(nl, blk, sm_grid(16u)), blk, 0, s>>>(
        nl, kp, ps, R.S.data(), R.count.data(), l + 1 < d ? child.data() : nullptr,
        skeys.data(), 2 * (d - 1 - l), L.key.data(), L.count.data(), L.child.data(),
        L.start.data());
      CSPT_CHECK_LAUNCH();
    }
    // the parent level's counts are no longer needed
    if (l > 0) {
      raw[l - 1].count.reset();
      raw[l - 1].S.reset();
      raw[l - 1].X.reset();
      raw[l - 1].P.reset();
    }
    R.P.reset();
  }
  raw.clear();
  lvl.reset();
  {
    std::vector<uint32_t> hk(d);
    CSPT_CUDA_TRY(
      cudaMemcpyAsync(hk.data(), kept.data(), d * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    for (int l = 0; l < d; ++l) levels[l].size = hk[l];
  }

  size_t q = 0;
  for (auto& L : levels) q += L.size;
  Buffer<uint32_t> okey(alloc, q), olen(alloc, q), ooff(alloc, q), ichild(alloc, q);
  Buffer<uint8_t> olev(alloc, q), oint(alloc, q);
  size_t base = 0;
  for (int l = 0; l < d; ++l) {
    LevelNodes& L = levels[l];
    if (L.size) {
      assemble_kernel<<<grid_for(L.size, blk, sm_grid(16u)), blk, 0, s>>>(
        L.key.data(), L.count.data(), L.child.data(), L.start.data(), L.size,
        static_cast<uint8_t>(l), l <= d - 2, max_size, base, okey.data(), olev.data(),
        oint.data(), olen.data(), ooff.data(), ichild.data());
      CSPT_CHECK_LAUNCH();
    }
    base += L.size;
    L = LevelNodes{};
  }
  // detail/point_quadtree.cuh:82-109: internal offsets = level_1_size + scan
  exclusive_scan<uint32_t>(ichild.data(), ichild.data(), q, static_cast<uint32_t*>(nullptr),
                           alloc);
  internal_offset_kernel<<<grid_for(q, blk, sm_grid(16u)), blk, 0, s>>>(
    oint.data(), ichild.data(), q, static_cast<uint32_t>(level_1_size), ooff.data());
  CSPT_CHECK_LAUNCH();
  *out_point_indices = sidx.release();
  *out = cspt_quadtree{okey.release(), olev.release(), oint.release(), olen.release(),
                       ooff.release(), q};
}

// The points in quadtree order, interleaved: xy[pos] = (x[pi[pos]],
// y[pi[pos]]).  Each thread keeps four independent gathers in flight; the
// index reads and the 16-byte (float64) or 8-byte (float32) stores are
// coalesced.  An index at or beyond npts is never read through: its point
// becomes (NaN, NaN).
template <typename T, typename V>
__global__ void __launch_bounds__(256)
  ordered_points_kernel(uint32_t const* __restrict__ pi, size_t n, T const* __restrict__ x,
                        T const* __restrict__ y, size_t npts, V* __restrict__ xy)
{
  constexpr int kPer = 4;
  size_t const step  = static_cast<size_t>(gridDim.x) * blockDim.x * kPer;
  for (size_t b = static_cast<size_t>(blockIdx.x) * blockDim.x * kPer + threadIdx.x; b < n;
       b += step) {
    uint32_t i[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      size_t const p = b + static_cast<size_t>(j) * blockDim.x;
      i[j]           = p < n ? pi[p] : 0xFFFFFFFFu;
    }
    V v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      bool const ok = i[j] < npts;
      v[j].x        = ok ? x[i[j]] : std::numeric_limits<T>::quiet_NaN();
      v[j].y        = ok ? y[i[j]] : std::numeric_limits<T>::quiet_NaN();
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      size_t const p = b + static_cast<size_t>(j) * blockDim.x;
      if (p < n) xy[p] = v[j];
    }
  }
}

}  // namespace

void points_in_quadtree_order(uint32_t const* point_indices, size_t n, void const* x,
                              void const* y, size_t npts, cspt_dtype dtype, void* out_xy,
                              cudaStream_t s)
{
  if (n == 0) return;
  unsigned const grd = grid_for((n + 3) / 4, 256, sm_grid(8u));
  if (dtype == CSPT_FLOAT64)
    ordered_points_kernel<double, double2><<<grd, 256, 0, s>>>(
      point_indices, n, static_cast<double const*>(x), static_cast<double const*>(y), npts,
      static_cast<double2*>(out_xy));
  else
    ordered_points_kernel<float, float2><<<grd, 256, 0, s>>>(
      point_indices, n, static_cast<float const*>(x), static_cast<float const*>(y), npts,
      static_cast<float2*>(out_xy));
  CSPT_CHECK_LAUNCH();
}

void quadtree_on_points(void const* x, void const* y, size_t n, cspt_dtype dtype, double x_min,
                        double x_max, double y_min, double y_max, double scale, int max_depth,
                        int32_t max_size, Allocator const& alloc, uint32_t** out_point_indices,
                        cspt_quadtree* out_tree, void* ordered)
{
  if (dtype == CSPT_FLOAT64)
    build<double>(static_cast<double const*>(x), static_cast<double const*>(y), n, x_min, x_max,
                  y_min, y_max, scale, max_depth, max_size, alloc, out_point_indices, out_tree,
                  nullptr, static_cast<double*>(ordered));
  else
    build<float>(static_cast<float const*>(x), static_cast<float const*>(y), n, x_min, x_max,
                 y_min, y_max, scale, max_depth, max_size, alloc, out_point_indices, out_tree,
                 nullptr, static_cast<float*>(ordered));
}

void quadtree_on_points_from_host(void const* host_x, void const* host_y, void* dev_x,
                                  void* dev_y, size_t n, cspt_dtype dtype, double x_min,
                                  double x_max, double y_min, double y_max, double scale,
                                  int max_depth, int32_t max_size, Allocator const& alloc,
                                  uint32_t** out_point_indices, cspt_quadtree* out_tree,
                                  void* ordered,
                                  std::function<void(cudaStream_t)> const* after_copies)
{
  if (dtype == CSPT_FLOAT64) {
    HostInput<double> const h{static_cast<double const*>(host_x),
                              static_cast<double const*>(host_y), static_cast<double*>(dev_x),
                              static_cast<double*>(dev_y), after_copies};
    build<double>(h.dx, h.dy, n, x_min, x_max, y_min, y_max, scale, max_depth, max_size, alloc,
                  out_point_indices, out_tree, &h, static_cast<double*>(ordered));
  } else {
    HostInput<float> const h{static_cast<float const*>(host_x), static_cast<float const*>(host_y),
                             static_cast<float*>(dev_x), static_cast<float*>(dev_y),
                             after_copies};
    build<float>(h.dx, h.dy, n, x_min, x_max, y_min, y_max, scale, max_depth, max_size, alloc,
                 out_point_indices, out_tree, &h, static_cast<float*>(ordered));
  }
}

}  // namespace cspt
