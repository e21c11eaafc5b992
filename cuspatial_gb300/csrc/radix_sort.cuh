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
#ifndef CSPT_SORT_ROUND
#define CSPT_SORT_ROUND 8
#endif
constexpr int kSortRound = CSPT_SORT_ROUND;  // rounds of 32 items per warp
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
                       Tiles tiles, int shift, unsigned mask, uint32_t const* offsets)
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
    val[r]         = ok ? (vals_in ? vals_in[i] : static_cast<uint32_t>(i)) : 0u;
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
// iota_vals is set the incoming contents of vals are ignored and vals[i] = i
// is used instead.  The result lands in (keys, vals) or in (keys_alt,
// vals_alt); the return value is true when it is in the _alt buffers.
// n must be below 2^32.
template <typename K, typename Tiles>
bool radix_sort_tiles(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                      int begin_bit, int end_bit, bool iota_vals, Tiles tiles, unsigned ntiles,
                      Allocator const& alloc)
{
  cudaStream_t const s = alloc.stream();
  if (n == 0) return false;
  if (end_bit <= begin_bit) {
    if (iota_vals) {
      scan_apply<uint32_t>([] __device__(size_t) { return 1u; },
                           [vals] __device__(size_t i, uint32_t e, uint32_t) { vals[i] = e; }, n,
                           static_cast<uint32_t*>(nullptr), alloc);
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
      kin, (first && iota_vals) ? nullptr : vin, kout, vout, tiles, shift, mask, counts.data());
    CSPT_CHECK_LAUNCH();
    in_alt = !in_alt;
    first  = false;
  }
  return in_alt;
}

template <typename K>
bool radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                      int begin_bit, int end_bit, bool iota_vals, Allocator const& alloc)
{
  unsigned const ntiles = static_cast<unsigned>((n + kSortTile - 1) / kSortTile);
  return radix_sort_tiles<K>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, iota_vals,
                             PlainTiles{n, ntiles}, ntiles, alloc);
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

}  // namespace cspt
