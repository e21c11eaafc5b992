// Stable LSD radix sort of (key, uint32 value) pairs, 8-bit digits over a bit
// range, so Morton keys of depth d cost ceil(2(d+1)/8) passes instead of 4.
//
// Per pass: per-tile digit histograms -> exclusive scan in digit-major order
// -> stable scatter.  Within a tile each warp ranks its 256 consecutive items
// with __match_any_sync; tiles, warps, rounds and lanes follow input order,
// which keeps the sort stable.  A segmented form sorts each of many
// contiguous segments in place (tiles never cross a segment boundary).
#pragma once

#include <vector>

#include "common.cuh"
#include "scan.cuh"

namespace cspt {

constexpr int kSortBlock = 256;  // one thread per 8-bit digit in the scatter
constexpr int kSortWarps = kSortBlock / 32;
// Rounds of 32 items per warp.  A fixed constant, not a build option: the
// sort's templates are instantiated in several translation units, and one
// program must see one tile size in all of them.
constexpr int kSortRound = 8;
constexpr int kSortTile  = kSortBlock * kSortRound;
constexpr unsigned kNoDigit = 0xFFFFu;

// Where a tile's items lie and where its digit counts go.
// PlainTiles: fixed tiles over [0, n); counts digit-major over all tiles, so
// one exclusive scan of the counts gives each (digit, tile) its output start.
struct PlainTiles {
  size_t n;
  unsigned ntiles;
  __device__ void range(unsigned t, size_t& b, size_t& e) const
  {
    b = static_cast<size_t>(t) * kSortTile;
    e = b + kSortTile < n ? b + kSortTile : n;
  }
  __device__ size_t slot(unsigned t, unsigned d) const
  {
    return static_cast<size_t>(d) * ntiles + t;
  }
};
// SegmentTiles: tiles that never cross a segment boundary; counts
// segment-major, then digit-major within the segment.  One exclusive scan
// then sorts every segment within its own range: segments stay in place, so
// keys already ordered by their high bits per segment need only their low
// bits sorted.
struct SortTile {
  uint32_t begin, end;   // items [begin, end)
  uint32_t first, count; // the segment's first tile and its number of tiles
};
struct SegmentTiles {
  SortTile const* tiles;
  __device__ void range(unsigned t, size_t& b, size_t& e) const
  {
    b = tiles[t].begin;
    e = tiles[t].end;
  }
  __device__ size_t slot(unsigned t, unsigned d) const
  {
    SortTile const& T = tiles[t];
    return static_cast<size_t>(T.first) * 256 + static_cast<size_t>(d) * T.count + (t - T.first);
  }
};

template <typename K, typename Tiles>
__global__ void __launch_bounds__(kSortBlock)
  radix_histogram_kernel(K const* keys, Tiles tiles, int shift, unsigned mask, uint32_t* counts)
{
  __shared__ uint32_t hist[kSortWarps][256];
  for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortBlock) (&hist[0][0])[i] = 0;
  __syncthreads();
  int const warp = threadIdx.x >> 5;
  int const lane = threadIdx.x & 31;
  size_t tb, te;
  tiles.range(blockIdx.x, tb, te);
  size_t const base = tb + warp * (32 * kSortRound);
#pragma unroll
  for (int r = 0; r < kSortRound; ++r) {
    size_t const i = base + r * 32 + lane;
    if (i < te) {
      unsigned const d = static_cast<unsigned>((keys[i] >> shift) & mask);
      atomicAdd(&hist[warp][d], 1u);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kSortBlock) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s += hist[w][d];
    counts[tiles.slot(blockIdx.x, d)] = s;
  }
}

static_assert(kSortBlock == 256, "the scatter assigns one thread per digit");

// Stable scatter of one tile: items are ranked per warp with
// __match_any_sync (rounds in input order), placed in shared memory in the
// tile's digit order, then written out in that order, so the global writes
// of each digit's run are contiguous.
template <typename K, typename Tiles>
__global__ void __launch_bounds__(kSortBlock)
  radix_scatter_kernel(K const* keys_in, uint32_t const* vals_in, K* keys_out, uint32_t* vals_out,
                       Tiles tiles, int shift, unsigned mask, uint32_t const* offsets,
                       uint32_t iota_base)
{
  __shared__ uint32_t wcount[kSortWarps][256];
  __shared__ uint32_t tile_start[256];
  __shared__ uint32_t global_base[256];
  __shared__ K skey[kSortTile];
  __shared__ uint32_t sval[kSortTile];
  __shared__ uint32_t total_s;
  for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortBlock) (&wcount[0][0])[i] = 0;
  __syncthreads();
  int const warp       = threadIdx.x >> 5;
  int const lane       = threadIdx.x & 31;
  unsigned const lt    = (1u << lane) - 1u;
  size_t tb, te;
  tiles.range(blockIdx.x, tb, te);
  size_t const base    = tb + warp * (32 * kSortRound);
  K key[kSortRound];
  uint32_t val[kSortRound];
  uint32_t pos[kSortRound];
  unsigned dig[kSortRound];
#pragma unroll
  for (int r = 0; r < kSortRound; ++r) {
    size_t const i = base + r * 32 + lane;
    bool const ok  = i < te;
    key[r]         = ok ? keys_in[i] : K{0};
    val[r]         = ok ? (vals_in ? vals_in[i] : static_cast<uint32_t>(i) + iota_base) : 0u;
    dig[r]         = ok ? static_cast<unsigned>((key[r] >> shift) & mask) : kNoDigit;
    unsigned const peers = __match_any_sync(0xFFFFFFFFu, dig[r]);
    unsigned const below = __popc(peers & lt);
    uint32_t prior       = 0;
    if (ok) prior = wcount[warp][dig[r]];
    pos[r] = prior + below;
    __syncwarp();
    // the lowest lane of each digit group advances the warp's counter
    if (ok && below == 0) wcount[warp][dig[r]] = prior + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit (one thread each): prefix over warps, the tile's digit start
  // and the digit's global base
  {
    int const d    = threadIdx.x;  // kSortBlock == 256 digits
    uint32_t run   = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      uint32_t const c = wcount[w][d];
      wcount[w][d]     = run;
      run += c;
    }
    uint32_t const start = block_exclusive_scan<uint32_t, kSortBlock>(run, &total_s);
    tile_start[d]        = start;
    global_base[d]       = offsets[tiles.slot(blockIdx.x, d)];
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortRound; ++r) {
    if (dig[r] != kNoDigit) {
      uint32_t const t = tile_start[dig[r]] + wcount[warp][dig[r]] + pos[r];
      skey[t]          = key[r];
      sval[t]          = val[r];
    }
  }
  __syncthreads();
  uint32_t const m = total_s;
  for (uint32_t t = threadIdx.x; t < m; t += kSortBlock) {
    K const k        = skey[t];
    unsigned const d = static_cast<unsigned>((k >> shift) & mask);
    uint32_t const g = global_base[d] + (t - tile_start[d]);
    keys_out[g]      = k;
    vals_out[g]      = sval[t];
  }
}

// Sorts (keys, vals) by bits [begin_bit, end_bit) of the key.  When
// iota_vals is set the incoming contents of vals are ignored and vals[i] =
// iota_base + i is used instead.  The result lands in (keys, vals) or in (keys_alt,
// vals_alt); the return value is true when it is in the _alt buffers.
// n must be below 2^32.
template <typename K, typename Tiles>
bool radix_sort_tiles(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                      int begin_bit, int end_bit, bool iota_vals, Tiles tiles, unsigned ntiles,
                      Allocator const& alloc, uint32_t iota_base = 0)
{
  cudaStream_t const s = alloc.stream();
  if (n == 0) return false;
  if (end_bit <= begin_bit) {
    if (iota_vals) {
      scan_apply<uint32_t>(
        [] __device__(size_t) { return 1u; },
        [vals, iota_base] __device__(size_t i, uint32_t e, uint32_t) { vals[i] = e + iota_base; },
        n, static_cast<uint32_t*>(nullptr), alloc);
    }
    return false;
  }
  Buffer<uint32_t> counts(alloc, static_cast<size_t>(ntiles) * 256);
  bool in_alt = false;
  bool first  = true;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    K* kin         = in_alt ? keys_alt : keys;
    uint32_t* vin  = in_alt ? vals_alt : vals;
    K* kout        = in_alt ? keys : keys_alt;
    uint32_t* vout = in_alt ? vals : vals_alt;
    int const width     = end_bit - shift < 8 ? end_bit - shift : 8;
    unsigned const mask = (1u << width) - 1u;
    radix_histogram_kernel<K, Tiles>
      <<<ntiles, kSortBlock, 0, s>>>(kin, tiles, shift, mask, counts.data());
    CSPT_CHECK_LAUNCH();
    exclusive_scan<uint32_t>(counts.data(), counts.data(), static_cast<size_t>(ntiles) * 256,
                             static_cast<uint32_t*>(nullptr), alloc);
    radix_scatter_kernel<K, Tiles><<<ntiles, kSortBlock, 0, s>>>(
      kin, (first && iota_vals) ? nullptr : vin, kout, vout, tiles, shift, mask, counts.data(),
      iota_base);
    CSPT_CHECK_LAUNCH();
    in_alt = !in_alt;
    first  = false;
  }
  return in_alt;
}

template <typename K>
bool radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                      int begin_bit, int end_bit, bool iota_vals, Allocator const& alloc,
                      uint32_t iota_base = 0)
{
  unsigned const ntiles = static_cast<unsigned>((n + kSortTile - 1) / kSortTile);
  return radix_sort_tiles<K>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, iota_vals,
                             PlainTiles{n, ntiles}, ntiles, alloc, iota_base);
}

// The same within segments: tiles (device) never cross a segment boundary
// and cover [0, n); each segment is sorted in place by bits [begin_bit,
// end_bit).
template <typename K>
bool radix_sort_segments(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                         int begin_bit, int end_bit, bool iota_vals, SortTile const* tiles,
                         unsigned ntiles, Allocator const& alloc)
{
  return radix_sort_tiles<K>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, iota_vals,
                             SegmentTiles{tiles}, ntiles, alloc);
}

// Tiles of at most kSortTile items over segments [bounds[j], bounds[j+1])
// (host; empty segments get none).
inline void segment_sort_tiles(std::vector<uint64_t> const& bounds, std::vector<SortTile>& out)
{
  out.clear();
  for (size_t j = 0; j + 1 < bounds.size(); ++j) {
    uint64_t const b = bounds[j], e = bounds[j + 1];
    if (e <= b) continue;
    uint32_t const first = static_cast<uint32_t>(out.size());
    uint32_t const count = static_cast<uint32_t>((e - b + kSortTile - 1) / kSortTile);
    for (uint32_t k = 0; k < count; ++k) {
      uint64_t const tb = b + static_cast<uint64_t>(k) * kSortTile;
      uint64_t const te = tb + kSortTile < e ? tb + kSortTile : e;
      out.push_back(SortTile{static_cast<uint32_t>(tb), static_cast<uint32_t>(te), first, count});
    }
  }
}

// ---------------------------------------------------------------------------
// Stable merge of sorted runs (merge path), for data sorted chunk by chunk as
// it arrives.  A pass merges runs 2k and 2k+1 of `src` into `dst` (an
// unpaired last run is copied).  Each block owns kMergeTile outputs of one
// pair: it finds where its diagonal range starts and ends in the two runs
// (ties go to the left run, whose positions come first), stages both slices
// in shared memory, merges kMergeItems outputs per thread and writes the tile
// out in order.
// ---------------------------------------------------------------------------
constexpr int kMergeBlock   = 256;
constexpr int kMergeItems   = 8;
constexpr int kMergeTile    = kMergeBlock * kMergeItems;
constexpr int kMaxMergePairs = 8;

struct MergePair {
  uint32_t a0, na, nb;  // left run [a0, a0 + na), right run [a0 + na, a0 + na + nb)
  uint32_t tile0;       // the pair's first output tile
};
struct MergePlan {
  MergePair p[kMaxMergePairs];
  int n;
};

// outputs taken from a among the first d of the stable merge of a and b
template <typename K>
__device__ inline uint32_t merge_split(K const* a, uint32_t na, K const* b, uint32_t nb,
                                       uint32_t d)
{
  uint32_t lo = d > nb ? d - nb : 0u, hi = d < na ? d : na;
  while (lo < hi) {
    uint32_t const mid = (lo + hi) >> 1;
    if (a[mid] <= b[d - 1 - mid])
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

template <typename K>
__global__ void __launch_bounds__(kMergeBlock)
  merge_runs_kernel(K const* __restrict__ ks, uint32_t const* __restrict__ vs, K* __restrict__ kd,
                    uint32_t* __restrict__ vd, MergePlan plan)
{
  __shared__ K sk[kMergeTile];
  __shared__ uint32_t sv[kMergeTile];
  __shared__ uint32_t split[2];
  int p = 0;
  while (p + 1 < plan.n && plan.p[p + 1].tile0 <= blockIdx.x) ++p;
  MergePair const P = plan.p[p];
  uint32_t const n  = P.na + P.nb;
  uint32_t const d0 = (blockIdx.x - P.tile0) * static_cast<uint32_t>(kMergeTile);
  uint32_t const d1 = min(n, d0 + static_cast<uint32_t>(kMergeTile));
  K const* a        = ks + P.a0;
  K const* b        = a + P.na;
  if (threadIdx.x == 0) split[0] = merge_split(a, P.na, b, P.nb, d0);
  if (threadIdx.x == 32) split[1] = merge_split(a, P.na, b, P.nb, d1);
  __syncthreads();
  uint32_t const i0 = split[0], i1 = split[1];
  uint32_t const la = i1 - i0, lb = (d1 - i1) - (d0 - i0);
  uint32_t const j0 = d0 - i0;
  for (uint32_t t = threadIdx.x; t < la; t += kMergeBlock) {
    sk[t] = a[i0 + t];
    sv[t] = vs[P.a0 + i0 + t];
  }
  for (uint32_t t = threadIdx.x; t < lb; t += kMergeBlock) {
    sk[la + t] = b[j0 + t];
    sv[la + t] = vs[P.a0 + P.na + j0 + t];
  }
  __syncthreads();
  uint32_t const m  = d1 - d0;
  uint32_t const ld = threadIdx.x * kMergeItems;
  K okey[kMergeItems];
  uint32_t oval[kMergeItems];
  if (ld < m) {
    uint32_t i = merge_split(sk, la, sk + la, lb, ld), j = ld - i;
#pragma unroll
    for (int k = 0; k < kMergeItems; ++k) {
      if (ld + k < m) {
        bool const left = j >= lb || (i < la && sk[i] <= sk[la + j]);
        okey[k]         = left ? sk[i] : sk[la + j];
        oval[k]         = left ? sv[i] : sv[la + j];
        i += left ? 1u : 0u;
        j += left ? 0u : 1u;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kMergeItems; ++k) {
    if (ld + k < m) {
      sk[ld + k] = okey[k];
      sv[ld + k] = oval[k];
    }
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < m; t += kMergeBlock) {
    kd[P.a0 + d0 + t] = sk[t];
    vd[P.a0 + d0 + t] = sv[t];
  }
}

// Merges the sorted runs [bounds[r], bounds[r+1]) of (keys, vals) into one
// (at most 2 kMaxMergePairs runs); returns true when the result is in the
// _alt buffers.
template <typename K>
bool merge_sorted_runs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt,
                       std::vector<size_t> bounds, cudaStream_t s)
{
  CSPT_EXPECTS(bounds.size() >= 2 && bounds.size() - 1 <= 2 * kMaxMergePairs,
               "too many sorted runs to merge");
  bool in_alt = false;
  while (bounds.size() > 2) {
    K const* ks        = in_alt ? keys_alt : keys;
    uint32_t const* vs = in_alt ? vals_alt : vals;
    K* kd              = in_alt ? keys : keys_alt;
    uint32_t* vd       = in_alt ? vals : vals_alt;
    size_t const runs  = bounds.size() - 1;
    MergePlan plan{};
    std::vector<size_t> next{bounds[0]};
    uint32_t tiles = 0;
    size_t r       = 0;
    for (; r + 1 < runs; r += 2) {
      uint32_t const na = static_cast<uint32_t>(bounds[r + 1] - bounds[r]);
      uint32_t const nb = static_cast<uint32_t>(bounds[r + 2] - bounds[r + 1]);
      plan.p[plan.n++]  = MergePair{static_cast<uint32_t>(bounds[r]), na, nb, tiles};
      tiles += (na + nb + kMergeTile - 1) / kMergeTile;
      next.push_back(bounds[r + 2]);
    }
    if (r < runs) {  // the unpaired last run
      size_t const b0 = bounds[r], m = bounds[r + 1] - bounds[r];
      CSPT_CUDA_TRY(cudaMemcpyAsync(kd + b0, ks + b0, m * sizeof(K), cudaMemcpyDeviceToDevice, s));
      CSPT_CUDA_TRY(
        cudaMemcpyAsync(vd + b0, vs + b0, m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
      next.push_back(bounds[r + 1]);
    }
    if (tiles) {
      merge_runs_kernel<K><<<tiles, kMergeBlock, 0, s>>>(ks, vs, kd, vd, plan);
      CSPT_CHECK_LAUNCH();
    }
    bounds = std::move(next);
    in_alt = !in_alt;
  }
  return in_alt;
}

}  // namespace cspt
