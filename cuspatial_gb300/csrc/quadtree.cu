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
                                   T minx, T miny, T maxx, T maxy, T scale, int d,
                                   uint32_t* __restrict__ keys)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    T const px = x[i], py = y[i];
    uint32_t k;
    if (px < minx || px > maxx || py < miny || py > maxy) {
      k = static_cast<uint32_t>((1 << (2 * d)) - 1);
    } else {
      uint16_t const cx = static_cast<uint16_t>((px - minx) / scale);
      uint16_t const cy = static_cast<uint16_t>((py - miny) / scale);
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

// children of the previous level's nodes = next-level starts inside them
__global__ void child_count_kernel(uint32_t const* __restrict__ prev_starts, size_t nprev,
                                   uint32_t const* __restrict__ rank_cur, size_t n,
                                   uint32_t* __restrict__ child)
{
  for (size_t p = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; p < nprev;
       p += static_cast<size_t>(gridDim.x) * blockDim.x) {
    size_t const e = (p + 1 < nprev) ? prev_starts[p + 1] : n;
    child[p]       = rank_cur[e] - rank_cur[prev_starts[p]];
  }
}

// A level-l node (l >= 1) survives iff its parent holds more than max_size
// points (phase_2.cuh:206-236).
__global__ void keep_kernel(uint32_t const* __restrict__ starts, size_t nl,
                            uint8_t const* __restrict__ lvl, int prev_level,
                            uint32_t const* __restrict__ rank_prev,
                            uint32_t const* __restrict__ count_prev, uint32_t max_size,
                            uint8_t* __restrict__ keep)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < nl;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t const i      = starts[k];
    uint32_t const is_beg = (lvl[i] != kNoStart && lvl[i] <= prev_level) ? 1u : 0u;
    uint32_t const parent = rank_prev[i] + is_beg - 1u;
    keep[k]               = count_prev[parent] > max_size ? 1 : 0;
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

template <typename T>
void build(T const* x, T const* y, size_t n, double x1d, double x2d, double y1d, double y2d,
           double scaled, int max_depth_in, int32_t max_size_in, Allocator const& alloc,
           uint32_t** out_point_indices, cspt_quadtree* out)
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
  unsigned const grd = grid_for(n, blk, 152u * 16u);
  KernelTimer timer("quadtree_build", s);

  Buffer<uint32_t> keys(alloc, n), keys_alt(alloc, n);
  Buffer<uint32_t> idx(alloc, n), idx_alt(alloc, n);
  morton_keys_kernel<T>
    <<<grd, blk, 0, s>>>(x, y, n, minx, miny, maxx, maxy, scale, d, keys.data());
  CSPT_CHECK_LAUNCH();
  // cells reach 2^d + 2, so the key needs 2(d+1) bits (2(d+2) below d = 2)
  int const key_bits = d >= 2 ? 2 * d + 2 : 2 * d + 4;
  bool const alt     = radix_sort_pairs<uint32_t>(keys.data(), idx.data(), keys_alt.data(),
                                              idx_alt.data(), n, 0, key_bits > 32 ? 32 : key_bits,
                                              true, alloc);
  Buffer<uint32_t>& skeys = alt ? keys_alt : keys;
  Buffer<uint32_t>& sidx  = alt ? idx_alt : idx;
  (alt ? keys : keys_alt).reset();

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
    node_count_kernel<<<grid_for(q, blk, 152u * 16u), blk, 0, s>>>(st, q, n, olen.data());
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

  // Levels 0..d-1, top-down.
  Buffer<uint32_t> rank_prev(alloc, n + 1), rank_cur(alloc, n + 1);
  Buffer<uint32_t> starts_prev, starts_cur;
  Buffer<uint32_t> count_prev, count_cur;
  Buffer<uint8_t> keep_prev, keep_cur;
  size_t n_prev = 0;
  std::vector<LevelNodes> levels(d);
  size_t level_1_size = 0;

  // emits the kept nodes of level `lv_out` once its child counts are known
  auto emit = [&](int lv_out, Buffer<uint32_t>& starts, Buffer<uint32_t>& counts,
                  Buffer<uint32_t>* childs, Buffer<uint8_t>* keep, size_t nl) {
    LevelNodes& L      = levels[lv_out];
    uint32_t const* st = starts.data();
    uint8_t const* kp  = keep ? keep->data() : nullptr;
    Buffer<uint32_t> pos(alloc, nl);
    uint32_t* ps = pos.data();
    scan_apply<uint32_t>(
      [kp] __device__(size_t k) { return kp ? static_cast<uint32_t>(kp[k]) : 1u; },
      [ps] __device__(size_t k, uint32_t e, uint32_t) { ps[k] = e; }, nl, total.data(), alloc);
    size_t const m = read_back(total.data(), s);
    L.size         = m;
    L.key          = Buffer<uint32_t>(alloc, m);
    L.count        = Buffer<uint32_t>(alloc, m);
    L.child        = Buffer<uint32_t>(alloc, m);
    L.start        = Buffer<uint32_t>(alloc, m);
    uint32_t *ok = L.key.data(), *oc = L.count.data(), *och = L.child.data(),
             *os = L.start.data();
    uint32_t const* sk  = skeys.data();
    uint32_t const* cn  = counts.data();
    uint32_t const* chp = childs ? childs->data() : nullptr;
    int const shift     = 2 * (d - 1 - lv_out);
    scan_apply<uint32_t>([] __device__(size_t) { return 0u; },
                         [=] __device__(size_t k, uint32_t, uint32_t) {
                           if (kp && !kp[k]) return;
                           uint32_t const o = ps[k];
                           ok[o]            = sk[st[k]] >> shift;
                           oc[o]            = cn[k];
                           och[o]           = chp ? chp[k] : 0u;
                           os[o]            = st[k];
                         },
                         nl, static_cast<uint32_t*>(nullptr), alloc);
  };

  for (int l = 0; l < d; ++l) {
    // rank the level-l starts and gather their positions
    starts_cur     = Buffer<uint32_t>(alloc, n);
    uint32_t* rk   = rank_cur.data();
    uint32_t* st   = starts_cur.data();
    int const ll   = l;
    scan_apply<uint32_t>(
      [lv, ll] __device__(size_t i) {
        return (lv[i] != kNoStart && static_cast<int>(lv[i]) <= ll) ? 1u : 0u;
      },
      [rk, st] __device__(size_t i, uint32_t e, uint32_t f) {
        rk[i] = e;
        if (f) st[e] = static_cast<uint32_t>(i);
      },
      n, rank_cur.data() + n, alloc);
    size_t const nl = read_back(rank_cur.data() + n, s);
    if (l == 0) level_1_size = nl;
    count_cur = Buffer<uint32_t>(alloc, nl);
    node_count_kernel<<<grid_for(nl, blk, 152u * 16u), blk, 0, s>>>(st, nl, n, count_cur.data());
    CSPT_CHECK_LAUNCH();
    keep_cur = Buffer<uint8_t>(alloc, nl);
    if (l == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(keep_cur.data(), 1, nl, s));
    } else {
      keep_kernel<<<grid_for(nl, blk, 152u * 16u), blk, 0, s>>>(
        st, nl, lv, l - 1, rank_prev.data(), count_prev.data(), max_size, keep_cur.data());
      CSPT_CHECK_LAUNCH();
      // the previous level's child counts, then emit it
      Buffer<uint32_t> child_prev(alloc, n_prev);
      child_count_kernel<<<grid_for(n_prev, blk, 152u * 16u), blk, 0, s>>>(
        starts_prev.data(), n_prev, rank_cur.data(), n, child_prev.data());
      CSPT_CHECK_LAUNCH();
      emit(l - 1, starts_prev, count_prev, &child_prev, l - 1 == 0 ? nullptr : &keep_prev,
           n_prev);
    }
    std::swap(rank_prev, rank_cur);
    starts_prev = std::move(starts_cur);
    count_prev  = std::move(count_cur);
    keep_prev   = std::move(keep_cur);
    n_prev      = nl;
  }
  emit(d - 1, starts_prev, count_prev, nullptr, &keep_prev, n_prev);
  starts_prev.reset();
  count_prev.reset();
  keep_prev.reset();
  rank_prev.reset();
  rank_cur.reset();
  lvl.reset();

  size_t q = 0;
  for (auto& L : levels) q += L.size;
  Buffer<uint32_t> okey(alloc, q), olen(alloc, q), ooff(alloc, q), ichild(alloc, q);
  Buffer<uint8_t> olev(alloc, q), oint(alloc, q);
  size_t base = 0;
  for (int l = 0; l < d; ++l) {
    LevelNodes& L = levels[l];
    if (L.size) {
      assemble_kernel<<<grid_for(L.size, blk, 152u * 16u), blk, 0, s>>>(
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
  internal_offset_kernel<<<grid_for(q, blk, 152u * 16u), blk, 0, s>>>(
    oint.data(), ichild.data(), q, static_cast<uint32_t>(level_1_size), ooff.data());
  CSPT_CHECK_LAUNCH();
  *out_point_indices = sidx.release();
  *out = cspt_quadtree{okey.release(), olev.release(), oint.release(), olen.release(),
                       ooff.release(), q};
}

}  // namespace

void quadtree_on_points(void const* x, void const* y, size_t n, cspt_dtype dtype, double x_min,
                        double x_max, double y_min, double y_max, double scale, int max_depth,
                        int32_t max_size, Allocator const& alloc, uint32_t** out_point_indices,
                        cspt_quadtree* out_tree)
{
  if (dtype == CSPT_FLOAT64) {
    build<double>(static_cast<double const*>(x), static_cast<double const*>(y), n, x_min, x_max,
                  y_min, y_max, scale, max_depth, max_size, alloc, out_point_indices, out_tree);
  } else {
    build<float>(static_cast<float const*>(x), static_cast<float const*>(y), n, x_min, x_max,
                 y_min, y_max, scale, max_depth, max_size, alloc, out_point_indices, out_tree);
  }
}

}  // namespace cspt
