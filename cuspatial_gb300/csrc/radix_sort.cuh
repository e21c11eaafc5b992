// Stable LSD radix sort of (key, uint32 value) pairs, 8-bit digits over a bit
// range, so Morton keys of depth d cost ceil(2(d+1)/8) passes instead of 4.
//
// Per pass: per-tile digit histograms -> exclusive scan in digit-major order
// -> stable scatter.  Within a tile each warp ranks its 256 consecutive items
// with __match_any_sync; tiles, warps, rounds and lanes follow input order,
// which keeps the sort stable.
#pragma once

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

template <typename K>
__global__ void __launch_bounds__(kSortBlock)
  radix_histogram_kernel(K const* keys, size_t n, int shift, unsigned mask, uint32_t* counts,
                         unsigned ntiles)
{
  __shared__ uint32_t hist[kSortWarps][256];
  for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortBlock) (&hist[0][0])[i] = 0;
  __syncthreads();
  int const warp    = threadIdx.x >> 5;
  int const lane    = threadIdx.x & 31;
  size_t const base = static_cast<size_t>(blockIdx.x) * kSortTile + warp * (32 * kSortRound);
#pragma unroll
  for (int r = 0; r < kSortRound; ++r) {
    size_t const i = base + r * 32 + lane;
    if (i < n) {
      unsigned const d = static_cast<unsigned>((keys[i] >> shift) & mask);
      atomicAdd(&hist[warp][d], 1u);
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kSortBlock) {
    uint32_t s = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) s += hist[w][d];
    counts[static_cast<size_t>(d) * ntiles + blockIdx.x] = s;
  }
}

static_assert(kSortBlock == 256, "the scatter assigns one thread per digit");

// Stable scatter of one tile: items are ranked per warp with
// __match_any_sync (rounds in input order), placed in shared memory in the
// tile's digit order, then written out in that order, so the global writes
// of each digit's run are contiguous.
template <typename K>
__global__ void __launch_bounds__(kSortBlock)
  radix_scatter_kernel(K const* keys_in, uint32_t const* vals_in, K* keys_out, uint32_t* vals_out,
                       size_t n, int shift, unsigned mask, uint32_t const* offsets,
                       unsigned ntiles)
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
  size_t const tbase   = static_cast<size_t>(blockIdx.x) * kSortTile;
  size_t const base    = tbase + warp * (32 * kSortRound);
  K key[kSortRound];
  uint32_t val[kSortRound];
  uint32_t pos[kSortRound];
  unsigned dig[kSortRound];
#pragma unroll
  for (int r = 0; r < kSortRound; ++r) {
    size_t const i = base + r * 32 + lane;
    bool const ok  = i < n;
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
    global_base[d]       = offsets[static_cast<size_t>(d) * ntiles + blockIdx.x];
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
template <typename K>
bool radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, size_t n,
                      int begin_bit, int end_bit, bool iota_vals, Allocator const& alloc)
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
  unsigned const ntiles = static_cast<unsigned>((n + kSortTile - 1) / kSortTile);
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
    radix_histogram_kernel<K>
      <<<ntiles, kSortBlock, 0, s>>>(kin, n, shift, mask, counts.data(), ntiles);
    CSPT_CHECK_LAUNCH();
    exclusive_scan<uint32_t>(counts.data(), counts.data(), static_cast<size_t>(ntiles) * 256,
                             static_cast<uint32_t*>(nullptr), alloc);
    radix_scatter_kernel<K><<<ntiles, kSortBlock, 0, s>>>(
      kin, (first && iota_vals) ? nullptr : vin, kout, vout, n, shift, mask, counts.data(), ntiles);
    CSPT_CHECK_LAUNCH();
    in_alt = !in_alt;
    first  = false;
  }
  return in_alt;
}

}  // namespace cspt
