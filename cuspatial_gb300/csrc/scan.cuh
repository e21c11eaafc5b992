// Device-wide exclusive scan and stream compaction (reduce / scan-partials /
// downsweep, tiles of 2048 items per 256-thread block).
#pragma once

#include "common.cuh"

namespace cspt {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile  = kScanBlock * kScanItems;

template <typename T>
__device__ inline T warp_inclusive_scan(T v)
{
  int const lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T const u = __shfl_up_sync(0xFFFFFFFFu, v, off);
    if (lane >= off) v += u;
  }
  return v;
}

// Exclusive scan of one value per thread across the block; returns the
// thread's exclusive prefix and sets *block_total.
template <typename T, int BLOCK>
__device__ inline T block_exclusive_scan(T v, T* block_total)
{
  __shared__ T warp_sums[BLOCK / 32];
  int const lane = threadIdx.x & 31;
  int const warp = threadIdx.x >> 5;
  T const incl   = warp_inclusive_scan(v);
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T s        = lane < BLOCK / 32 ? warp_sums[lane] : T{0};
    T const si = warp_inclusive_scan(s);
    if (lane < BLOCK / 32) warp_sums[lane] = si - s;
    if (lane == BLOCK / 32 - 1) *block_total = si;
  }
  __syncthreads();
  T const r = incl - v + warp_sums[warp];
  __syncthreads();
  return r;
}

template <typename T, typename InF>
__global__ void __launch_bounds__(kScanBlock) scan_reduce_kernel(InF in, size_t n, T* partials)
{
  size_t const base = static_cast<size_t>(blockIdx.x) * kScanTile;
  T s               = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    size_t const i = base + static_cast<size_t>(j) * kScanBlock + threadIdx.x;
    if (i < n) s += in(i);
  }
  __shared__ T total;
  (void)block_exclusive_scan<T, kScanBlock>(s, &total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

template <typename T>
__global__ void __launch_bounds__(1024) scan_partials_kernel(T* partials, size_t nparts, T* total)
{
  __shared__ T carry_s;
  __shared__ T warp_sums[32];
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (size_t base = 0; base < nparts; base += 1024) {
    size_t const i = base + threadIdx.x;
    T const v      = i < nparts ? partials[i] : T{0};
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T const incl   = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      T const s  = warp_sums[lane];
      T const si = warp_inclusive_scan(s);
      warp_sums[lane] = si - s;
    }
    __syncthreads();
    T const carry = carry_s;
    T const excl  = incl - v + warp_sums[warp] + carry;
    if (i < nparts) partials[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry_s = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry_s;
}

// Calls out(i, exclusive_prefix_of_i, in(i)) for every i in [0, n).
// Items are read and handed to `out` in striped order (item j * 256 + t of
// the tile by thread t: coalesced), and scanned in blocked order (thread t
// owns items [8 t, 8 t + 8)) through a shared-memory transpose padded by one
// word per 32 (no bank conflicts for 4-byte items).
template <typename T, typename InF, typename OutF>
__global__ void __launch_bounds__(kScanBlock)
  scan_down_kernel(InF in, OutF out, size_t n, T const* partials)
{
  __shared__ T s_items[kScanTile + kScanTile / 32];
  size_t const base = static_cast<size_t>(blockIdx.x) * kScanTile;
  T sv[kScanItems];  // this thread's items, striped
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint32_t const li = static_cast<uint32_t>(j) * kScanBlock + threadIdx.x;
    size_t const i    = base + li;
    sv[j]             = i < n ? in(i) : T{0};
    s_items[li + (li >> 5)] = sv[j];
  }
  __syncthreads();
  T vals[kScanItems];
  T s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint32_t const li = threadIdx.x * kScanItems + static_cast<uint32_t>(j);
    vals[j]           = s_items[li + (li >> 5)];
    s += vals[j];
  }
  __shared__ T total;
  T run = block_exclusive_scan<T, kScanBlock>(s, &total) + partials[blockIdx.x];
  // block_exclusive_scan ends with a barrier: every thread has read its
  // items before the prefixes overwrite them
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint32_t const li       = threadIdx.x * kScanItems + static_cast<uint32_t>(j);
    s_items[li + (li >> 5)] = run;
    run += vals[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    uint32_t const li = static_cast<uint32_t>(j) * kScanBlock + threadIdx.x;
    size_t const i    = base + li;
    if (i < n) out(i, s_items[li + (li >> 5)], sv[j]);
  }
}

// Generic driver.  `total` (device pointer, may be null) receives the sum.
template <typename T, typename InF, typename OutF>
void scan_apply(InF in, OutF out, size_t n, T* total, Allocator const& alloc)
{
  cudaStream_t const s = alloc.stream();
  if (n == 0) {
    if (total) CSPT_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(T), s));
    return;
  }
  size_t const nparts = (n + kScanTile - 1) / kScanTile;
  Buffer<T> partials(alloc, nparts);
  scan_reduce_kernel<T, InF><<<static_cast<unsigned>(nparts), kScanBlock, 0, s>>>(
    in, n, partials.data());
  CSPT_CHECK_LAUNCH();
  scan_partials_kernel<T><<<1, 1024, 0, s>>>(partials.data(), nparts, total);
  CSPT_CHECK_LAUNCH();
  scan_down_kernel<T, InF, OutF><<<static_cast<unsigned>(nparts), kScanBlock, 0, s>>>(
    in, out, n, partials.data());
  CSPT_CHECK_LAUNCH();
}

template <typename T>
struct ArrayIn {
  T const* p;
  __device__ T operator()(size_t i) const { return p[i]; }
};
template <typename T>
struct ArrayOut {
  T* p;
  __device__ void operator()(size_t i, T excl, T) const { p[i] = excl; }
};

// Plain exclusive scan of an array.
template <typename T>
void exclusive_scan(T const* in, T* out, size_t n, T* total, Allocator const& alloc)
{
  scan_apply<T>(ArrayIn<T>{in}, ArrayOut<T>{out}, n, total, alloc);
}

}  // namespace cspt

namespace cspt {

// scan_apply over caller-provided partials (at least ceil(n / kScanTile)
// elements): launches the same three kernels and allocates nothing.
template <typename T, typename InF, typename OutF>
void scan_apply_prealloc(InF in, OutF out, size_t n, T* total, T* partials, cudaStream_t s)
{
  if (n == 0) {
    if (total) CSPT_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(T), s));
    return;
  }
  size_t const nparts = (n + kScanTile - 1) / kScanTile;
  scan_reduce_kernel<T, InF><<<static_cast<unsigned>(nparts), kScanBlock, 0, s>>>(in, n, partials);
  CSPT_CHECK_LAUNCH();
  scan_partials_kernel<T><<<1, 1024, 0, s>>>(partials, nparts, total);
  CSPT_CHECK_LAUNCH();
  scan_down_kernel<T, InF, OutF>
    <<<static_cast<unsigned>(nparts), kScanBlock, 0, s>>>(in, out, n, partials);
  CSPT_CHECK_LAUNCH();
}

}  // namespace cspt
