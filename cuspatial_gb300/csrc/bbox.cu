// Polygon and linestring bounding boxes: one warp per geometry.
//
// Reference: cpp/include/cuspatial/detail/bounding_boxes.cuh:37-184 — every
// vertex becomes the box [v - r, v + r]; boxes are merged per geometry id by
// reduce_by_key.  Since rounding is monotone, min_v fl(v - r) = fl(min_v v - r),
// so the warp reduces raw coordinates and applies r once.  reduce_by_key emits
// no row for a geometry without vertices, so rows are placed at the rank of
// the geometry among non-empty ones; the rows left at the end are NaN.
#include <climits>

#include "common.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

template <typename T>
__device__ inline T dmin(T a, T b)
{
  return fmin(a, b);
}
// Order-preserving integer image of a non-NaN double (-0 sorts below +0).
__device__ inline long long order_key(double v)
{
  long long const b = __double_as_longlong(v);
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
__device__ inline double from_order_key(long long k)
{
  return __longlong_as_double(k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL));
}
template <typename T>
__device__ inline T dmax(T a, T b)
{
  return fmax(a, b);
}

template <typename T>
__global__ void bbox_kernel(uint32_t const* __restrict__ vbegin_off,
                            uint32_t const* __restrict__ vend_off, uint32_t const* __restrict__ via,
                            size_t ngeom, T const* __restrict__ x, T const* __restrict__ y,
                            uint32_t const* __restrict__ row, T r, T* __restrict__ ominx,
                            T* __restrict__ ominy, T* __restrict__ omaxx, T* __restrict__ omaxy)
{
  int const lane     = threadIdx.x & 31;
  size_t const warps = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  for (size_t g = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; g < ngeom;
       g += warps) {
    // vertex range: via (ring offsets) indirection for polygons, direct else
    size_t vb, ve;
    if (via) {
      vb = via[vbegin_off[g]];
      ve = via[vend_off[g]];
    } else {
      vb = vbegin_off[g];
      ve = vend_off[g];
    }
    if (ve <= vb) continue;
    T mnx, mny, mxx, mxy;
    if constexpr (std::is_same<T, double>::value) {
      // fmin / fmax (NaN skipped) on an order-preserving integer image: the
      // integer pipe instead of this part's slow float64 min/max
      long long k0 = LLONG_MAX, k1 = LLONG_MAX, k2 = LLONG_MIN, k3 = LLONG_MIN;
      for (size_t v = vb + lane; v < ve; v += 32) {
        double const px = x[v], py = y[v];
        if (px == px) {
          long long const kx = order_key(px);
          k0                 = min(k0, kx);
          k2                 = max(k2, kx);
        }
        if (py == py) {
          long long const ky = order_key(py);
          k1                 = min(k1, ky);
          k3                 = max(k3, ky);
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        k0 = min(k0, __shfl_xor_sync(0xFFFFFFFFu, k0, off));
        k1 = min(k1, __shfl_xor_sync(0xFFFFFFFFu, k1, off));
        k2 = max(k2, __shfl_xor_sync(0xFFFFFFFFu, k2, off));
        k3 = max(k3, __shfl_xor_sync(0xFFFFFFFFu, k3, off));
      }
      double const nan = std::numeric_limits<double>::quiet_NaN();
      mnx = k0 == LLONG_MAX ? nan : from_order_key(k0);
      mny = k1 == LLONG_MAX ? nan : from_order_key(k1);
      mxx = k2 == LLONG_MIN ? nan : from_order_key(k2);
      mxy = k3 == LLONG_MIN ? nan : from_order_key(k3);
    } else {
      mnx = x[vb];
      mny = y[vb];
      mxx = x[vb];
      mxy = y[vb];
      for (size_t v = vb + lane; v < ve; v += 32) {
        T const px = x[v], py = y[v];
        mnx        = dmin(mnx, px);
        mny        = dmin(mny, py);
        mxx        = dmax(mxx, px);
        mxy        = dmax(mxy, py);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        mnx = dmin(mnx, __shfl_xor_sync(0xFFFFFFFFu, mnx, off));
        mny = dmin(mny, __shfl_xor_sync(0xFFFFFFFFu, mny, off));
        mxx = dmax(mxx, __shfl_xor_sync(0xFFFFFFFFu, mxx, off));
        mxy = dmax(mxy, __shfl_xor_sync(0xFFFFFFFFu, mxy, off));
      }
    }
    if (lane == 0) {
      uint32_t const o = row[g];
      ominx[o]         = mnx - r;
      ominy[o]         = mny - r;
      omaxx[o]         = mxx + r;
      omaxy[o]         = mxy + r;
    }
  }
}

template <typename T>
void run(uint32_t const* goff, size_t ngeom, uint32_t const* via, T const* x, T const* y, T r,
         T* ominx, T* ominy, T* omaxx, T* omaxy, Allocator const& alloc)
{
  cudaStream_t const s = alloc.stream();
  if (ngeom == 0) return;
  KernelTimer timer("bounding_boxes", s);
  Buffer<uint32_t> row(alloc, ngeom);
  Buffer<uint32_t> nonempty(alloc, 1);
  uint32_t* rw = row.data();
  scan_apply<uint32_t>(
    [goff, via] __device__(size_t g) {
      uint32_t b = goff[g], e = goff[g + 1];
      if (via) {
        b = via[b];
        e = via[e];
      }
      return e > b ? 1u : 0u;
    },
    [rw] __device__(size_t g, uint32_t e, uint32_t) { rw[g] = e; }, ngeom, nonempty.data(),
    alloc);
  bbox_kernel<T><<<grid_for(ngeom * 32, 256, sm_grid(32u)), 256, 0, s>>>(
    goff, goff + 1, via, ngeom, x, y, rw, r, ominx, ominy, omaxx, omaxy);
  CSPT_CHECK_LAUNCH();
  // rows past the number of non-empty geometries: NaN (the reference leaves
  // them unwritten).  The count is only known on the device, so the fill
  // covers the tail from it.
  uint32_t const* ne = nonempty.data();
  scan_apply<uint32_t>([] __device__(size_t) { return 0u; },
                       [=] __device__(size_t i, uint32_t, uint32_t) {
                         if (i >= *ne) {
                           T const nan = std::numeric_limits<T>::quiet_NaN();
                           ominx[i] = ominy[i] = omaxx[i] = omaxy[i] = nan;
                         }
                       },
                       ngeom, static_cast<uint32_t*>(nullptr), alloc);
}

}  // namespace

void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc)
{
  (void)nro;
  (void)nv;
  size_t const np = npo > 0 ? npo - 1 : 0;
  if (dtype == CSPT_FLOAT64)
    run<double>(poly_offsets, np, ring_offsets, static_cast<double const*>(x),
                static_cast<double const*>(y), r, static_cast<double*>(ominx),
                static_cast<double*>(ominy), static_cast<double*>(omaxx),
                static_cast<double*>(omaxy), alloc);
  else
    run<float>(poly_offsets, np, ring_offsets, static_cast<float const*>(x),
               static_cast<float const*>(y), static_cast<float>(r), static_cast<float*>(ominx),
               static_cast<float*>(ominy), static_cast<float*>(omaxx),
               static_cast<float*>(omaxy), alloc);
}

void linestring_bounding_boxes(uint32_t const* ls_offsets, size_t nlo, void const* x,
                               void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                               void* ominy, void* omaxx, void* omaxy, Allocator const& alloc)
{
  (void)nv;
  size_t const nl = nlo > 0 ? nlo - 1 : 0;
  if (dtype == CSPT_FLOAT64)
    run<double>(ls_offsets, nl, nullptr, static_cast<double const*>(x),
                static_cast<double const*>(y), r, static_cast<double*>(ominx),
                static_cast<double*>(ominy), static_cast<double*>(omaxx),
                static_cast<double*>(omaxy), alloc);
  else
    run<float>(ls_offsets, nl, nullptr, static_cast<float const*>(x),
               static_cast<float const*>(y), static_cast<float>(r), static_cast<float*>(ominx),
               static_cast<float*>(ominy), static_cast<float*>(omaxx),
               static_cast<float*>(omaxy), alloc);
}

}  // namespace cspt

// ---------------------------------------------------------------------------
// cspt_polygon_bounding_boxes_noalloc: the same boxes without any device
// allocation, for callers that must not allocate (code running inside a CUDA
// graph capture or a real-time loop, where cudaMalloc would synchronise the
// device, and hosts that hand out all device memory themselves).  Its scratch
// (row index per polygon, scan partials, non-empty count) lives in the
// file-scope array below, which every GPU that loads the library keeps until
// exit: 4 MiB + 2 KiB, enough for 1,048,576 polygons.
// ---------------------------------------------------------------------------
#include <array>
#include <mutex>

namespace cspt {
namespace {

constexpr size_t kNoAllocMaxPolygons = size_t{1} << 20;
constexpr size_t kNoAllocPartials    = (kNoAllocMaxPolygons + kScanTile - 1) / kScanTile;
constexpr size_t kNoAllocWords       = kNoAllocMaxPolygons + kNoAllocPartials + 64;

// Device scratch shared by every call on a device; each call rewrites the
// rows, partials and count it later reads, so nothing needs clearing.
static __device__ __align__(256) uint32_t g_bbox_noalloc_scratch[kNoAllocWords];

// The address of the scratch on the current device.  Resolved once per
// device with cudaGetSymbolAddress (with that device current); the host-side
// name of the array is not a device address.
uint32_t* noalloc_scratch_on_current_device()
{
  static std::mutex mu;
  static std::array<uint32_t*, 256> addr{};
  int dev = 0;
  CSPT_CUDA_TRY(cudaGetDevice(&dev));
  CSPT_EXPECTS(dev >= 0 && dev < static_cast<int>(addr.size()), "device ordinal out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    CSPT_CUDA_TRY(cudaGetSymbolAddress(&p, g_bbox_noalloc_scratch));
    addr[dev] = static_cast<uint32_t*>(p);
  }
  return addr[dev];
}

template <typename T>
__global__ void nan_tail_kernel(uint32_t const* __restrict__ nonempty, size_t n, T* a, T* b, T* c,
                                T* d)
{
  T const nan      = std::numeric_limits<T>::quiet_NaN();
  uint32_t const m = *nonempty;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    if (i >= m) a[i] = b[i] = c[i] = d[i] = nan;
  }
}

struct NonEmptyPolygon {
  uint32_t const* po;
  uint32_t const* ro;
  __device__ uint32_t operator()(size_t g) const { return ro[po[g + 1]] > ro[po[g]] ? 1u : 0u; }
};
struct StoreRow {
  uint32_t* row;
  __device__ void operator()(size_t g, uint32_t e, uint32_t) const { row[g] = e; }
};

template <typename T>
void run_noalloc(uint32_t const* po, size_t np, uint32_t const* ro, T const* x, T const* y, T r,
                 T* ominx, T* ominy, T* omaxx, T* omaxy, uint32_t* scratch, cudaStream_t s)
{
  uint32_t* row      = scratch;
  uint32_t* partials = scratch + kNoAllocMaxPolygons;
  uint32_t* nonempty = partials + kNoAllocPartials;
  scan_apply_prealloc<uint32_t>(NonEmptyPolygon{po, ro}, StoreRow{row}, np, nonempty, partials, s);
  bbox_kernel<T><<<grid_for(np * 32, 256, sm_grid(32u)), 256, 0, s>>>(
    po, po + 1, ro, np, x, y, row, r, ominx, ominy, omaxx, omaxy);
  CSPT_CHECK_LAUNCH();
  nan_tail_kernel<T>
    <<<grid_for(np, 256, sm_grid(16u)), 256, 0, s>>>(nonempty, np, ominx, ominy, omaxx, omaxy);
  CSPT_CHECK_LAUNCH();
}

}  // namespace
}  // namespace cspt

extern "C" cspt_status cspt_polygon_bounding_boxes_noalloc(
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* x, const void* y, size_t num_vertices, cspt_dtype dtype,
  double expansion_radius, void* out_min_x, void* out_min_y, void* out_max_x, void* out_max_y,
  void* stream)
{
  using namespace cspt;
  return guarded([&] {
    if (dtype != CSPT_FLOAT32 && dtype != CSPT_FLOAT64)
      throw Error{CSPT_UNSUPPORTED, "Only floating-point types are supported"};
    size_t const np = num_poly_offsets > 0 ? num_poly_offsets - 1 : 0;
    if (np == 0) return;
    CSPT_EXPECTS(np <= kNoAllocMaxPolygons,
                 "cspt_polygon_bounding_boxes_noalloc handles at most 1048576 polygons; use "
                 "cspt_polygon_bounding_boxes for larger inputs");
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    if (num_ring_offsets < 2 || num_vertices == 0) return;
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    uint32_t* scratch    = noalloc_scratch_on_current_device();
    if (dtype == CSPT_FLOAT64)
      run_noalloc<double>(poly_offsets, np, ring_offsets, static_cast<double const*>(x),
                          static_cast<double const*>(y), expansion_radius,
                          static_cast<double*>(out_min_x), static_cast<double*>(out_min_y),
                          static_cast<double*>(out_max_x), static_cast<double*>(out_max_y),
                          scratch, s);
    else
      run_noalloc<float>(poly_offsets, np, ring_offsets, static_cast<float const*>(x),
                         static_cast<float const*>(y), static_cast<float>(expansion_radius),
                         static_cast<float*>(out_min_x), static_cast<float*>(out_min_y),
                         static_cast<float*>(out_max_x), static_cast<float*>(out_max_y), scratch,
                         s);
  });
}
