// A forest of point quadtrees, one per instance, built in one pass.
//
// Instance i owns points [pt_begin_i, pt_end_i) of concatenated x/y columns
// and has its own quadtree_on_points parameters.  The forest holds the
// concatenation of the per-instance results:
//   * point_indices: instance i's sorted point order at [pt_begin_i,
//     pt_end_i), values local to the instance (pidx) and global (sidx);
//   * quadtree: instance i's nodes at [node_offsets_i, node_offsets_{i+1}),
//     child and point offsets local to the instance, plus goff = the leaf's
//     first position in the global sorted order.
// Each instance's part equals what quadtree_on_points returns for it alone
// (cpp/include/cuspatial/detail/point_quadtree.cuh:237-272).
//
// Points carry the composite key (instance << kb) | morton key and are
// sorted once, each instance's points within their own range (they are
// instance-major already, so a segmented radix sort of the Morton bits
// gives the composite order): instances stay contiguous and each instance's
// points take their own stable Morton order.  The single-tree construction (quadtree.cu) carries
// over level by level with three changes: a sorted position starts a node at
// every level when it is the first point of its instance, a level-l node
// exists only for instances with max_depth > l, and node ends are clipped to
// the instance's last point.  Kept nodes are then laid out instance-major,
// level-major within the instance.
#pragma once

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "join_kernel.cuh"
#include "radix_sort.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

constexpr int kLevels       = 16;
constexpr uint8_t kNoStart  = 0xFF;
constexpr unsigned kBlk     = 256;
inline unsigned grid_cap() { return sm_grid(16u); }

struct Inst {
  double minx, miny, maxx, maxy, scale, rscale;
  uint32_t d, max_size;
  uint32_t pt_begin, pt_end;
  uint32_t poly_begin, poly_end;
  uint32_t node_base, nq, L0;
};

// the instance whose [begin, next begin) holds v; begins has ni + 1 sorted
// entries and begins[0] <= v < begins[ni]
__device__ inline uint32_t find_instance(uint32_t const* __restrict__ begins, uint32_t ni,
                                         uint32_t v)
{
  uint32_t lo = 0, hi = ni;
  while (hi - lo > 1) {
    uint32_t const mid = (lo + hi) >> 1;
    if (begins[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

#define CSPT_GRID_STRIDE(i, n)                                                           \
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < (n); \
       i += static_cast<size_t>(gridDim.x) * blockDim.x)

// Point positions in tiles of 2^kTileShift: tile_inst[t] = the instance of
// the tile's first position, tile_inst[ntiles] = ni - 1.  A position's
// instance then lies in [tile_inst[t], tile_inst[t + 1]], usually one entry.
constexpr int kTileShift = 10;
inline size_t position_tiles(size_t n) { return (n + (size_t{1} << kTileShift) - 1) >> kTileShift; }

__global__ void tile_instance_kernel(uint32_t const* __restrict__ begins, uint32_t ni, size_t ntiles,
                                     uint32_t* __restrict__ tile_inst)
{
  CSPT_GRID_STRIDE(t, ntiles + 1)
  {
    tile_inst[t] = t < ntiles ? find_instance(begins, ni, static_cast<uint32_t>(t << kTileShift))
                              : ni - 1u;
  }
}

// find_instance narrowed by the tile table
__device__ inline uint32_t instance_of(uint32_t const* __restrict__ begins,
                                       uint32_t const* __restrict__ tile_inst, uint32_t v)
{
  uint32_t const t = v >> kTileShift;
  uint32_t lo = tile_inst[t], hi = tile_inst[t + 1] + 1u;
  while (hi - lo > 1) {
    uint32_t const mid = (lo + hi) >> 1;
    if (begins[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// phase_1.cuh:73-85 per instance, tagged with the instance
template <typename K>
__global__ void keys_kernel(double const* __restrict__ x, double const* __restrict__ y, size_t n,
                            uint32_t const* __restrict__ pt_begin,
                            uint32_t const* __restrict__ tile_inst,
                            Inst const* __restrict__ inst, int kb, K* __restrict__ keys)
{
  CSPT_GRID_STRIDE(i, n)
  {
    uint32_t const k = instance_of(pt_begin, tile_inst, static_cast<uint32_t>(i));
    Inst const& I    = inst[k];
    double const px = x[i], py = y[i];
    uint32_t key;
    if (outside_closed(px, I.minx, I.maxx) || outside_closed(py, I.miny, I.maxy)) {
      key = (1u << (2 * I.d)) - 1u;
    } else {
      uint16_t const cx = cell_of_quotient(px - I.minx, I.scale, I.rscale);
      uint16_t const cy = cell_of_quotient(py - I.miny, I.scale, I.rscale);
      key               = (spread16(cy) << 1) | spread16(cx);
    }
    keys[i] = (static_cast<K>(k) << kb) | key;
  }
}

template <typename K>
__global__ void start_level_kernel(K const* __restrict__ sk, size_t n, int kb,
                                   Inst const* __restrict__ inst, uint8_t* __restrict__ lvl,
                                   uint8_t* __restrict__ lim)
{
  K const mask = (K{1} << kb) - 1u;
  CSPT_GRID_STRIDE(i, n)
  {
    K const c = sk[i];
    uint32_t const k = static_cast<uint32_t>(c >> kb);
    int const d      = static_cast<int>(inst[k].d);
    uint8_t l        = 0;
    if (i > 0 && (sk[i - 1] >> kb) == k) {
      uint32_t const diff = static_cast<uint32_t>((c ^ sk[i - 1]) & mask);
      if (diff == 0) {
        l = kNoStart;
      } else {
        int const lv = d - 1 - (31 - __clz(diff)) / 2;
        l            = static_cast<uint8_t>(lv < 0 ? 0 : lv);
      }
    }
    lvl[i] = l;
    lim[i] = static_cast<uint8_t>(d);
  }
}

// The candidate list: the positions that start a node at some level of their
// instance (lvl below the instance's depth; a repeated key never does).
// Every level's starts are a subsequence of it, so the levels are ranked
// over this list instead of over all points.
struct AnyStart {
  uint8_t const* lvl;
  uint8_t const* lim;
  __device__ uint32_t operator()(size_t i) const { return lvl[i] < lim[i] ? 1u : 0u; }
};
struct AnyStore {
  uint8_t const* lvl;
  uint8_t const* lim;
  uint32_t* apos;
  uint8_t* alvl;
  uint8_t* alim;
  __device__ void operator()(size_t i, uint32_t e, uint32_t f) const
  {
    if (f) {
      apos[e] = static_cast<uint32_t>(i);
      alvl[e] = lvl[i];
      alim[e] = lim[i];
    }
  }
};

// level-l starts among the candidates
struct StartFlag {
  uint8_t const* alvl;
  uint8_t const* alim;
  int l;
  __device__ uint32_t operator()(size_t j) const
  {
    return (static_cast<int>(alvl[j]) <= l && l < static_cast<int>(alim[j])) ? 1u : 0u;
  }
};
// rank[j] = level-l starts before candidate j; a start's sorted position and
// candidate index
struct RankStore {
  uint32_t const* apos;
  uint32_t* rank;
  uint32_t* starts;
  uint32_t* starts_c;
  __device__ void operator()(size_t j, uint32_t e, uint32_t f) const
  {
    rank[j] = e;
    if (f) {
      starts[e]   = apos[j];
      starts_c[e] = static_cast<uint32_t>(j);
    }
  }
};

__device__ inline uint32_t node_end(uint32_t const* starts, size_t nl, size_t k, uint32_t iend)
{
  uint32_t const e = (k + 1 < nl) ? starts[k + 1] : iend;
  return e < iend ? e : iend;
}

// point counts and instances of one level's nodes
template <typename K>
__global__ void count_kernel(uint32_t const* __restrict__ starts, size_t nl,
                             K const* __restrict__ sk, int kb,
                             Inst const* __restrict__ inst, uint32_t* __restrict__ count,
                             uint32_t* __restrict__ ninst)
{
  CSPT_GRID_STRIDE(k, nl)
  {
    uint32_t const s = starts[k];
    uint32_t const i = static_cast<uint32_t>(sk[s] >> kb);
    count[k]         = node_end(starts, nl, k, inst[i].pt_end) - s;
    ninst[k]         = i;
  }
}

// Children of the level-(l-1) nodes: the level-l starts from the node's
// candidate to the next level-(l-1) node's (or the end of the list).  A node
// ends earlier only at its instance's end, and the instances between it and
// the next level-(l-1) node have no level-(l-1) node, hence no level-l one.
__global__ void child_count_kernel(uint32_t const* __restrict__ prev_starts_c, size_t nprev,
                                   uint32_t const* __restrict__ rank_cur, uint32_t ncand,
                                   uint32_t* __restrict__ child)
{
  CSPT_GRID_STRIDE(p, nprev)
  {
    uint32_t const e = p + 1 < nprev ? prev_starts_c[p + 1] : ncand;
    child[p]         = rank_cur[e] - rank_cur[prev_starts_c[p]];
  }
}

// phase_2.cuh:206-236 with the instance's max_size
__global__ void keep_kernel(uint32_t const* __restrict__ starts_c, size_t nl,
                            uint32_t const* __restrict__ ninst, uint8_t const* __restrict__ alvl,
                            int prev_level, uint32_t const* __restrict__ rank_prev,
                            uint32_t const* __restrict__ count_prev,
                            Inst const* __restrict__ inst, uint8_t* __restrict__ keep)
{
  CSPT_GRID_STRIDE(k, nl)
  {
    uint32_t const j      = starts_c[k];
    uint32_t const is_beg = static_cast<int>(alvl[j]) <= prev_level ? 1u : 0u;
    uint32_t const parent = rank_prev[j] + is_beg - 1u;
    keep[k]               = count_prev[parent] > inst[ninst[k]].max_size ? 1 : 0;
  }
}

struct KeepIn {
  uint8_t const* kp;
  __device__ uint32_t operator()(size_t k) const { return kp ? kp[k] : 1u; }
};
struct PosOut {
  uint32_t* ps;
  __device__ void operator()(size_t k, uint32_t e, uint32_t) const { ps[k] = e; }
};

template <typename K>
__global__ void compact_level_kernel(size_t nl, uint8_t const* __restrict__ kp,
                                     uint32_t const* __restrict__ ps,
                                     uint32_t const* __restrict__ starts,
                                     uint32_t const* __restrict__ cnt,
                                     uint32_t const* __restrict__ child,
                                     uint32_t const* __restrict__ ninst,
                                     K const* __restrict__ sk, int kb,
                                     Inst const* __restrict__ inst, int level,
                                     uint32_t* __restrict__ okey, uint32_t* __restrict__ ocount,
                                     uint32_t* __restrict__ ochild, uint32_t* __restrict__ ostart,
                                     uint32_t* __restrict__ oinst)
{
  K const mask = (K{1} << kb) - 1u;
  CSPT_GRID_STRIDE(k, nl)
  {
    if (kp && !kp[k]) continue;
    uint32_t const o   = ps[k];
    uint32_t const i   = ninst[k];
    int const shift    = 2 * (static_cast<int>(inst[i].d) - 1 - level);
    uint32_t const key = static_cast<uint32_t>(sk[starts[k]] & mask);
    okey[o]            = shift > 0 ? key >> shift : key;
    ocount[o]          = cnt[k];
    ochild[o]          = child ? child[k] : 0u;
    ostart[o]          = starts[k];
    oinst[o]           = i;
  }
}

// Node counts per level: hist[v * 16 + w] = candidates with start level v
// in an instance of depth w; level l has the candidates with v <= l < w.
// Equal (v, w) codes of a warp are added once (they cluster).
__global__ void level_pair_histogram_kernel(uint8_t const* __restrict__ alvl,
                                            uint8_t const* __restrict__ alim, size_t nc,
                                            uint32_t* __restrict__ hist)
{
  __shared__ uint32_t sh[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  unsigned const lane = threadIdx.x & 31u;
  for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x); b < nc;
       b += static_cast<size_t>(gridDim.x) * blockDim.x) {  // uniform per warp
    size_t const j       = b + threadIdx.x;
    unsigned const code  = j < nc ? (alvl[j] & 15u) * 16u + (alim[j] & 15u) : 0xFFFFu;
    unsigned const peers = __match_any_sync(0xFFFFFFFFu, code);
    if (code != 0xFFFFu && static_cast<unsigned>(__ffs(peers) - 1) == lane)
      atomicAdd(&sh[code], static_cast<uint32_t>(__popc(peers)));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// first / one-past-last compacted index of each instance within a level of
// *mp nodes (device count)
__global__ void level_span_kernel(uint32_t const* __restrict__ oinst, uint32_t const* mp,
                                  int level, uint32_t* __restrict__ first,
                                  uint32_t* __restrict__ end)
{
  size_t const m = *mp;
  CSPT_GRID_STRIDE(k, m)
  {
    uint32_t const i = oinst[k];
    if (k == 0 || oinst[k - 1] != i) first[i * kLevels + level] = static_cast<uint32_t>(k);
    if (k + 1 == m || oinst[k + 1] != i) end[i * kLevels + level] = static_cast<uint32_t>(k + 1);
  }
}

// Node bases of the instances and, per (instance, level), the shift from a
// compacted level index to the output node index.
__global__ void __launch_bounds__(1024)
  layout_kernel(uint32_t const* __restrict__ first, uint32_t const* __restrict__ end,
                uint32_t ni, Inst* __restrict__ inst, long long* __restrict__ out_shift,
                uint64_t* __restrict__ node_offsets, int* __restrict__ error)
{
  uint32_t const per   = (ni + 1023u) / 1024u;
  uint32_t const begin = threadIdx.x * per;
  uint32_t const stop  = min(ni, begin + per);
  uint64_t sum         = 0;
  for (uint32_t i = begin; i < stop; ++i)
    for (int l = 0; l < kLevels; ++l) sum += end[i * kLevels + l] - first[i * kLevels + l];
  __shared__ uint64_t total;
  uint64_t base = block_exclusive_scan<uint64_t, 1024>(sum, &total);
  for (uint32_t i = begin; i < stop; ++i) {
    uint64_t lb = 0;
    for (int l = 0; l < kLevels; ++l) {
      uint32_t const f = first[i * kLevels + l], e = end[i * kLevels + l];
      out_shift[i * kLevels + l] =
        static_cast<long long>(base + lb) - static_cast<long long>(f);
      lb += e - f;
    }
    inst[i].node_base = static_cast<uint32_t>(base);
    inst[i].nq        = static_cast<uint32_t>(lb);
    inst[i].L0        = end[i * kLevels] - first[i * kLevels];
    if (lb >= (uint64_t{1} << 28) || base + lb >= (uint64_t{1} << 32)) atomicExch(error, 1);
    node_offsets[i] = base;
    base += lb;
  }
  if (threadIdx.x == 0) node_offsets[ni] = total;
}

__global__ void assemble_kernel(uint32_t const* __restrict__ key, uint32_t const* __restrict__ cnt,
                                uint32_t const* __restrict__ child,
                                uint32_t const* __restrict__ start,
                                uint32_t const* __restrict__ oinst, size_t m, int level,
                                Inst const* __restrict__ inst,
                                long long const* __restrict__ out_shift,
                                uint32_t* __restrict__ okey, uint8_t* __restrict__ olevel,
                                uint8_t* __restrict__ ointernal, uint32_t* __restrict__ olength,
                                uint32_t* __restrict__ ooffset, uint32_t* __restrict__ ichild,
                                uint32_t* __restrict__ node_inst)
{
  CSPT_GRID_STRIDE(k, m)
  {
    uint32_t const i    = oinst[k];
    Inst const& I       = inst[i];
    size_t const o      = static_cast<size_t>(out_shift[i * kLevels + level] + static_cast<long long>(k));
    bool const internal = level + 2 <= static_cast<int>(I.d) && cnt[k] > I.max_size;
    okey[o]             = key[k];
    olevel[o]           = static_cast<uint8_t>(level);
    ointernal[o]        = internal ? 1 : 0;
    olength[o]          = internal ? child[k] : cnt[k];
    ooffset[o]          = start[k] - I.pt_begin;
    ichild[o]           = internal ? child[k] : 0u;
    node_inst[o]        = i;
  }
}

// detail/point_quadtree.cuh:82-109 per instance: internal offsets are the
// instance's level-0 count plus the scan of child counts within the instance
__global__ void offsets_kernel(uint8_t const* __restrict__ internal,
                               uint32_t const* __restrict__ scanned,
                               uint32_t const* __restrict__ node_inst,
                               Inst const* __restrict__ inst, size_t q,
                               uint32_t* __restrict__ offset, uint32_t* __restrict__ goff)
{
  CSPT_GRID_STRIDE(o, q)
  {
    Inst const& I = inst[node_inst[o]];
    if (internal[o]) {
      offset[o] = I.L0 + scanned[o] - scanned[I.node_base];
      goff[o]   = 0u;
    } else {
      goff[o] = offset[o] + I.pt_begin;
    }
  }
}

template <typename K>
__global__ void local_indices_kernel(uint32_t const* __restrict__ sidx,
                                     K const* __restrict__ sk, int kb,
                                     Inst const* __restrict__ inst, size_t n,
                                     uint32_t* __restrict__ out)
{
  CSPT_GRID_STRIDE(i, n) { out[i] = sidx[i] - inst[sk[i] >> kb].pt_begin; }
}

__global__ void row_offsets_kernel(uint32_t const* __restrict__ pair_begin,
                                   uint64_t const* __restrict__ pair_out, uint32_t ni,
                                   uint64_t* __restrict__ row_offsets)
{
  CSPT_GRID_STRIDE(i, static_cast<size_t>(ni) + 1) { row_offsets[i] = pair_out[pair_begin[i]]; }
}

// rows -> instance-local point positions (and polygon indices when the
// instances own polygon ranges)
__global__ void localize_kernel(uint32_t* __restrict__ op, uint32_t* __restrict__ oq, size_t m,
                                uint32_t const* __restrict__ pt_begin,
                                uint32_t const* __restrict__ tile_inst,
                                Inst const* __restrict__ inst, bool local_polygons)
{
  CSPT_GRID_STRIDE(j, m)
  {
    uint32_t const pos = oq[j];
    Inst const& I      = inst[instance_of(pt_begin, tile_inst, pos)];
    oq[j]              = pos - I.pt_begin;
    if (local_polygons) op[j] = op[j] - I.poly_begin;
  }
}


// the tree a box of instance `of(b)` walks
template <typename InstanceOf>
struct ForestTrees {
  InstanceOf of;
  Inst const* inst;
  __device__ BoxTree<double> operator()(size_t b) const
  {
    Inst const& I = inst[of(b)];
    return BoxTree<double>{I.node_base, I.nq,     I.L0,    I.pt_begin,
                           I.minx,      I.miny,   I.scale, static_cast<int>(I.d)};
  }
};

class Forest {
 public:
  explicit Forest(Allocator const& alloc) : alloc_(&alloc) {}

  // Validates the parameters (the reference's join checks,
  // quadtree_bbox_filtering.cu:100-106), applies the clamps of
  // detail/point_quadtree.cuh:258-268 and uploads the instance table.
  // poly_off (host, may be null) gives the instances' polygon ranges.
  void setup(size_t ni, uint64_t const* h_pt_off, cspt_instance_params const* params,
             uint64_t const* h_poly_off)
  {
    Allocator const& a   = *alloc_;
    cudaStream_t const s = a.stream();
    ni_                  = ni;
    n_                   = h_pt_off[ni];
    CSPT_EXPECTS(n_ < (size_t{1} << 32), "fewer than 2^32 points are supported");
    std::vector<Inst> hi(ni);
    std::vector<uint32_t> h_ptb(ni + 1), h_pob(ni + 1);
    dmax_ = 1;
    for (size_t i = 0; i < ni; ++i) {
      cspt_instance_params const& p = params[i];
      CSPT_EXPECTS(h_pt_off[i] <= h_pt_off[i + 1] &&
                     (!h_poly_off || h_poly_off[i] <= h_poly_off[i + 1]),
                   "instance offsets must be non-decreasing");
      CSPT_EXPECTS(p.scale > 0, "scale must be positive");
      CSPT_EXPECTS(p.x_min < p.x_max && p.y_min < p.y_max,
                   "invalid bounding box (x_min, x_max, y_min, y_max)");
      CSPT_EXPECTS(p.max_depth > 0 && p.max_depth < 16,
                   "maximum depth must be positive and less than 16");
      Inst& I           = hi[i];
      I.minx            = p.x_min;
      I.miny            = p.y_min;
      I.maxx            = p.x_max;
      I.maxy            = p.y_max;
      I.d               = static_cast<uint32_t>(p.max_depth);
      double const span = std::max(p.x_max - p.x_min, p.y_max - p.y_min);
      double const ms   = span / static_cast<double>((1 << p.max_depth) + 2);
      I.scale           = p.scale > ms ? p.scale : ms;
      I.rscale          = 1.0 / I.scale;
      I.max_size        = static_cast<uint32_t>(p.max_size < 1 ? 1 : p.max_size);
      I.pt_begin        = static_cast<uint32_t>(h_pt_off[i]);
      I.pt_end          = static_cast<uint32_t>(h_pt_off[i + 1]);
      I.poly_begin      = h_poly_off ? static_cast<uint32_t>(h_poly_off[i]) : 0u;
      I.poly_end        = h_poly_off ? static_cast<uint32_t>(h_poly_off[i + 1]) : 0u;
      I.node_base = I.nq = I.L0 = 0;
      h_ptb[i]                  = I.pt_begin;
      h_pob[i]                  = I.poly_begin;
      dmax_                     = std::max(dmax_, p.max_depth);
    }
    h_ptb[ni] = static_cast<uint32_t>(n_);
    h_pob[ni] = h_poly_off ? static_cast<uint32_t>(h_poly_off[ni]) : 0u;
    inst_       = Buffer<Inst>(a, ni);
    pt_begin_   = Buffer<uint32_t>(a, ni + 1);
    poly_begin_ = Buffer<uint32_t>(a, ni + 1);
    CSPT_CUDA_TRY(cudaMemcpyAsync(inst_.data(), hi.data(), ni * sizeof(Inst),
                                  cudaMemcpyHostToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(pt_begin_.data(), h_ptb.data(), (ni + 1) * 4,
                                  cudaMemcpyHostToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(poly_begin_.data(), h_pob.data(), (ni + 1) * 4,
                                  cudaMemcpyHostToDevice, s));
    // radix sort tiles within instances: the points are instance-major
    // already, so only the Morton bits are sorted
    std::vector<uint64_t> bounds{0};
    for (size_t i = 1; i < ni; ++i) bounds.push_back(h_pt_off[i]);
    bounds.push_back(n_);
    std::vector<SortTile> hs;
    segment_sort_tiles(bounds, hs);
    sort_tiles_ = Buffer<SortTile>(a, hs.size());
    if (!hs.empty())
      CSPT_CUDA_TRY(cudaMemcpyAsync(sort_tiles_.data(), hs.data(), hs.size() * sizeof(SortTile),
                                    cudaMemcpyHostToDevice, s));
    size_t const ntiles = position_tiles(n_);
    tile_inst_          = Buffer<uint32_t>(a, ntiles + 1);
    if (ni) {
      tile_instance_kernel<<<grid_for(ntiles + 1, kBlk, grid_cap()), kBlk, 0, s>>>(
        pt_begin_.data(), static_cast<uint32_t>(ni), ntiles, tile_inst_.data());
      CSPT_CHECK_LAUNCH();
    }
    // the host arrays above must outlive the copies
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
  }

  void build(double const* x, double const* y)
  {
    Allocator const& a   = *alloc_;
    cudaStream_t const s = a.stream();
    size_t const n       = n_;
    node_off_            = Buffer<uint64_t>(a, ni_ + 1);
    if (n == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(node_off_.data(), 0, (ni_ + 1) * 8, s));
      return;
    }
    KernelTimer timer("forest_build", s);
    int const kb = dmax_ >= 2 ? 2 * dmax_ + 2 : 2 * dmax_ + 4;
    int ib       = 0;
    while ((uint64_t{1} << ib) < ni_) ++ib;
    // 32-bit composite keys when the instance and Morton bits fit: a third
    // less traffic in every sort pass
    if (kb + ib < 32)
      build_sorted<uint32_t>(x, y, kb);
    else
      build_sorted<uint64_t>(x, y, kb);
  }

  template <typename K>
  void build_sorted(double const* x, double const* y, int kb)
  {
    Allocator const& a   = *alloc_;
    cudaStream_t const s = a.stream();
    uint32_t const ni    = static_cast<uint32_t>(ni_);
    size_t const n       = n_;
    unsigned const grd   = grid_for(n, kBlk, grid_cap());

    Buffer<K> keys(a, n), keys_alt(a, n);
    Buffer<uint32_t> idx(a, n), idx_alt(a, n);
    keys_kernel<K><<<grd, kBlk, 0, s>>>(x, y, n, pt_begin_.data(), tile_inst_.data(), inst_.data(),
                                        kb, keys.data());
    CSPT_CHECK_LAUNCH();
    bool const alt = radix_sort_segments<K>(keys.data(), idx.data(), keys_alt.data(),
                                            idx_alt.data(), n, 0, kb, true, sort_tiles_.data(),
                                            static_cast<unsigned>(sort_tiles_.size()), a);
    Buffer<K>& sk = alt ? keys_alt : keys;
    sidx_         = std::move(alt ? idx_alt : idx);
    (alt ? keys : keys_alt).reset();
    (alt ? idx : idx_alt).reset();

    Buffer<uint8_t> lvl(a, n), lim(a, n);
    start_level_kernel<K><<<grd, kBlk, 0, s>>>(sk.data(), n, kb, inst_.data(), lvl.data(),
                                               lim.data());
    CSPT_CHECK_LAUNCH();
    pidx_ = Buffer<uint32_t>(a, n);
    local_indices_kernel<K><<<grd, kBlk, 0, s>>>(sidx_.data(), sk.data(), kb, inst_.data(), n,
                                                 pidx_.data());
    CSPT_CHECK_LAUNCH();

    // the candidate list: one scan over all points, then every level over it
    Buffer<uint32_t> total(a, 1);
    Buffer<uint32_t> apos(a, n);
    Buffer<uint8_t> alvl(a, n), alim(a, n);
    scan_apply<uint32_t>(AnyStart{lvl.data(), lim.data()},
                         AnyStore{lvl.data(), lim.data(), apos.data(), alvl.data(), alim.data()},
                         n, total.data(), a);
    size_t const nc = read_back(total.data(), s);
    lvl.reset();
    lim.reset();

    struct Level {
      Buffer<uint32_t> key, count, child, start, inst;
      size_t size = 0;
    };
    std::vector<Level> levels(dmax_);
    Buffer<uint32_t> first(a, ni_ * kLevels), end(a, ni_ * kLevels);
    CSPT_CUDA_TRY(cudaMemsetAsync(first.data(), 0, ni_ * kLevels * 4, s));
    CSPT_CUDA_TRY(cudaMemsetAsync(end.data(), 0, ni_ * kLevels * 4, s));
    Buffer<uint32_t> rank_prev(a, nc + 1), rank_cur(a, nc + 1);
    Buffer<uint32_t> starts_prev, starts_cur, startc_prev, startc_cur, count_prev, count_cur,
      inst_prev, inst_cur;
    Buffer<uint8_t> keep_prev, keep_cur;
    size_t n_prev = 0;

    // every level's node count from one histogram of the candidates
    std::vector<size_t> level_size(dmax_, 0);
    {
      Buffer<uint32_t> hist(a, 256);
      CSPT_CUDA_TRY(cudaMemsetAsync(hist.data(), 0, 256 * sizeof(uint32_t), s));
      if (nc) {
        level_pair_histogram_kernel<<<grid_for(nc, kBlk, grid_cap()), kBlk, 0, s>>>(
          alvl.data(), alim.data(), nc, hist.data());
        CSPT_CHECK_LAUNCH();
      }
      uint32_t h[256];
      CSPT_CUDA_TRY(cudaMemcpyAsync(h, hist.data(), sizeof(h), cudaMemcpyDeviceToHost, s));
      CSPT_CUDA_TRY(cudaStreamSynchronize(s));
      for (int l = 0; l < dmax_; ++l)
        for (int v = 0; v <= l; ++v)
          for (int w = l + 1; w < 16; ++w) level_size[l] += h[v * 16 + w];
    }
    // kept nodes per level, counted on the device; the level arrays hold up
    // to the level's node count
    Buffer<uint32_t> kept(a, dmax_);
    auto emit = [&](int lv, Buffer<uint32_t>& starts, Buffer<uint32_t>& counts,
                    Buffer<uint32_t>* childs, Buffer<uint32_t>& ninst, Buffer<uint8_t>* keep,
                    size_t nl) {
      Level& L          = levels[lv];
      uint8_t const* kp = keep ? keep->data() : nullptr;
      Buffer<uint32_t> pos(a, nl);
      scan_apply<uint32_t>(KeepIn{kp}, PosOut{pos.data()}, nl, kept.data() + lv, a);
      L.key   = Buffer<uint32_t>(a, nl);
      L.count = Buffer<uint32_t>(a, nl);
      L.child = Buffer<uint32_t>(a, nl);
      L.start = Buffer<uint32_t>(a, nl);
      L.inst  = Buffer<uint32_t>(a, nl);
      if (nl) {
        compact_level_kernel<K><<<grid_for(nl, kBlk, grid_cap()), kBlk, 0, s>>>(
          nl, kp, pos.data(), starts.data(), counts.data(), childs ? childs->data() : nullptr,
          ninst.data(), sk.data(), kb, inst_.data(), lv, L.key.data(), L.count.data(),
          L.child.data(), L.start.data(), L.inst.data());
        CSPT_CHECK_LAUNCH();
        level_span_kernel<<<grid_for(nl, kBlk, grid_cap()), kBlk, 0, s>>>(
          L.inst.data(), kept.data() + lv, lv, first.data(), end.data());
        CSPT_CHECK_LAUNCH();
      }
    };

    for (int l = 0; l < dmax_; ++l) {
      starts_cur = Buffer<uint32_t>(a, nc);
      startc_cur = Buffer<uint32_t>(a, nc);
      scan_apply<uint32_t>(StartFlag{alvl.data(), alim.data(), l},
                           RankStore{apos.data(), rank_cur.data(), starts_cur.data(),
                                     startc_cur.data()},
                           nc, rank_cur.data() + nc, a);
      size_t const nl = level_size[l];
      count_cur       = Buffer<uint32_t>(a, nl);
      inst_cur        = Buffer<uint32_t>(a, nl);
      keep_cur        = Buffer<uint8_t>(a, nl);
      unsigned const g = grid_for(nl, kBlk, grid_cap());
      if (nl) {
        count_kernel<K><<<g, kBlk, 0, s>>>(starts_cur.data(), nl, sk.data(), kb, inst_.data(),
                                           count_cur.data(), inst_cur.data());
        CSPT_CHECK_LAUNCH();
      }
      if (l == 0) {
        if (nl) CSPT_CUDA_TRY(cudaMemsetAsync(keep_cur.data(), 1, nl, s));
      } else {
        if (nl) {
          keep_kernel<<<g, kBlk, 0, s>>>(startc_cur.data(), nl, inst_cur.data(), alvl.data(),
                                         l - 1, rank_prev.data(), count_prev.data(),
                                         inst_.data(), keep_cur.data());
          CSPT_CHECK_LAUNCH();
        }
        Buffer<uint32_t> child_prev(a, n_prev);
        if (n_prev) {
          child_count_kernel<<<grid_for(n_prev, kBlk, grid_cap()), kBlk, 0, s>>>(
            startc_prev.data(), n_prev, rank_cur.data(), static_cast<uint32_t>(nc),
            child_prev.data());
          CSPT_CHECK_LAUNCH();
        }
        emit(l - 1, starts_prev, count_prev, &child_prev, inst_prev,
             l - 1 == 0 ? nullptr : &keep_prev, n_prev);
      }
      std::swap(rank_prev, rank_cur);
      starts_prev = std::move(starts_cur);
      startc_prev = std::move(startc_cur);
      count_prev  = std::move(count_cur);
      inst_prev   = std::move(inst_cur);
      keep_prev   = std::move(keep_cur);
      n_prev      = nl;
    }
    emit(dmax_ - 1, starts_prev, count_prev, nullptr, inst_prev, dmax_ - 1 == 0 ? nullptr : &keep_prev,
         n_prev);
    starts_prev.reset();
    startc_prev.reset();
    count_prev.reset();
    inst_prev.reset();
    keep_prev.reset();
    rank_prev.reset();
    rank_cur.reset();
    apos.reset();
    alvl.reset();
    alim.reset();
    sk.reset();

    Buffer<long long> shift(a, ni_ * kLevels);
    Buffer<int> err(a, 1);
    CSPT_CUDA_TRY(cudaMemsetAsync(err.data(), 0, sizeof(int), s));
    layout_kernel<<<1, 1024, 0, s>>>(first.data(), end.data(), ni, inst_.data(), shift.data(),
                                     node_off_.data(), err.data());
    CSPT_CHECK_LAUNCH();
    int herr = 0;
    std::vector<uint32_t> hk(dmax_);
    CSPT_CUDA_TRY(cudaMemcpyAsync(&herr, err.data(), sizeof(int), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(hk.data(), kept.data(), dmax_ * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    CSPT_EXPECTS(herr == 0, "an instance's quadtree has too many nodes for the batched form");
    size_t q = 0;
    for (int l = 0; l < dmax_; ++l) q += levels[l].size = hk[l];
    q_        = q;
    key_      = Buffer<uint32_t>(a, q);
    length_   = Buffer<uint32_t>(a, q);
    offset_   = Buffer<uint32_t>(a, q);
    goff_     = Buffer<uint32_t>(a, q);
    level_    = Buffer<uint8_t>(a, q);
    internal_ = Buffer<uint8_t>(a, q);
    if (q == 0) return;
    Buffer<uint32_t> ichild(a, q), node_inst(a, q);
    for (int l = 0; l < dmax_; ++l) {
      Level& L = levels[l];
      if (L.size) {
        assemble_kernel<<<grid_for(L.size, kBlk, grid_cap()), kBlk, 0, s>>>(
          L.key.data(), L.count.data(), L.child.data(), L.start.data(), L.inst.data(), L.size,
          l, inst_.data(), shift.data(), key_.data(), level_.data(), internal_.data(),
          length_.data(), offset_.data(), ichild.data(), node_inst.data());
        CSPT_CHECK_LAUNCH();
      }
      L = Level{};
    }
    exclusive_scan<uint32_t>(ichild.data(), ichild.data(), q, static_cast<uint32_t*>(nullptr), a);
    offsets_kernel<<<grid_for(q, kBlk, grid_cap()), kBlk, 0, s>>>(
      internal_.data(), ichild.data(), node_inst.data(), inst_.data(), q, offset_.data(),
      goff_.data());
    CSPT_CHECK_LAUNCH();
  }


  TreeView view() const
  {
    return TreeView{key_.data(), level_.data(), internal_.data(), length_.data(), offset_.data(),
                    q_};
  }
  cspt_quadtree tree() const
  {
    return cspt_quadtree{key_.data(), level_.data(), internal_.data(), length_.data(),
                         offset_.data(), q_};
  }

  Allocator const* alloc_;
  size_t ni_ = 0, n_ = 0, q_ = 0;
  int dmax_  = 1;
  Buffer<Inst> inst_;
  Buffer<uint32_t> pt_begin_, poly_begin_, tile_inst_;
  Buffer<SortTile> sort_tiles_;
  Buffer<uint32_t> sidx_, pidx_;
  Buffer<uint32_t> key_, length_, offset_, goff_;
  Buffer<uint8_t> level_, internal_;
  Buffer<uint64_t> node_off_;
};

}  // namespace
}  // namespace cspt
