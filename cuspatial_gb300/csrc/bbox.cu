// Polygon and linestring bounding boxes: one warp per geometry.
//
// Reference: cpp/include/cuspatial/detail/bounding_boxes.cuh:37-184 — every
// vertex becomes the box [v - r, v + r]; boxes are merged per geometry id by
// reduce_by_key.  Since rounding is monotone, min_v fl(v - r) = fl(min_v v - r),
// so the warp reduces raw coordinates and applies r once.  reduce_by_key emits
// no row for a geometry without vertices, so rows are placed at the rank of
// the geometry among non-empty ones; the rows left at the end are NaN.
#include "common.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

template <typename T>
__device__ inline T dmin(T a, T b)
{
  return fmin(a, b);
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
    T mnx = x[vb], mny = y[vb], mxx = x[vb], mxy = y[vb];
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
  bbox_kernel<T><<<grid_for(ngeom * 32, 256, 152u * 32u), 256, 0, s>>>(
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
