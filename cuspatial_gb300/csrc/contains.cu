// contains_properly in quadtree mode: the reference's composition of the
// join path with its own parameters, plus the two index mappings its callers
// apply to the rows.
//
// Reference: python/cuspatial/cuspatial/core/binpreds/contains.py:19-74
// (parameters and composition: max_depth 15, max_size ceil(sqrt(points)),
// the polygons' vertex extent as the tree's box, the smallest scale that the
// quadtree accepts without clamping; point_index replaced by
// point_indices[point_index]) and core/binpreds/contains_geometry_processor.py:
// 72-116 (each part's multipolygon).
//
// The chain runs through this library's own entry points, so validation and
// empty-input rules are those of the individual calls.  Two small kernels
// are added: the vertex extent (an integer min/max over order-preserving
// keys) and the row mapping (point position -> input point, part -> its
// multipolygon), fused into one pass over the rows.
#include <climits>
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"

namespace cspt {
namespace {

constexpr unsigned kContainsBlock = 256;

__device__ inline long long order_key64(double v)
{
  long long const b = __double_as_longlong(v);
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}
inline double from_order_key64(long long k)
{
  long long const b = k >= 0 ? k : (k ^ 0x7FFFFFFFFFFFFFFFLL);
  double v;
  std::memcpy(&v, &b, sizeof v);
  return v;
}

// ext = {min x, min y, -max x, -max y} as order keys (all minimised);
// NaN coordinates are skipped.
template <typename T>
__global__ void __launch_bounds__(kContainsBlock)
  extent_kernel(T const* __restrict__ vx, T const* __restrict__ vy, size_t nv,
                long long* __restrict__ ext)
{
  long long k[4] = {LLONG_MAX, LLONG_MAX, LLONG_MAX, LLONG_MAX};
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nv;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    double const x = static_cast<double>(vx[i]);
    double const y = static_cast<double>(vy[i]);
    if (x == x) {
      k[0] = min(k[0], order_key64(x));
      k[2] = min(k[2], order_key64(-x));
    }
    if (y == y) {
      k[1] = min(k[1], order_key64(y));
      k[3] = min(k[3], order_key64(-y));
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    long long v = k[j];
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    if ((threadIdx.x & 31) == 0 && v != LLONG_MAX) atomicMin(ext + j, v);
  }
}

// part -> multipolygon: geometry g owns parts [go[g], go[g+1])
__global__ void __launch_bounds__(kContainsBlock)
  part_geometry_kernel(uint32_t const* __restrict__ go, size_t ngeom, size_t nparts,
                       uint32_t* __restrict__ part_geom)
{
  for (size_t g = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; g < ngeom;
       g += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t const b = go[g], e = go[g + 1];
    for (uint32_t p = b; p < e && p < nparts; ++p) part_geom[p] = static_cast<uint32_t>(g);
  }
}

// rows: point position -> input point (in place), part -> multipolygon
__global__ void __launch_bounds__(kContainsBlock)
  map_rows_kernel(uint32_t* __restrict__ point, uint32_t const* __restrict__ part, size_t m,
                  uint32_t const* __restrict__ point_indices, size_t npi,
                  uint32_t const* __restrict__ part_geom, size_t nparts,
                  uint32_t* __restrict__ geom)
{
  for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < m;
       k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t const pos = point[k];
    point[k]           = pos < npi ? point_indices[pos] : 0xFFFFFFFFu;
    uint32_t const p   = part[k];
    geom[k]            = part_geom ? (p < nparts ? part_geom[p] : 0xFFFFFFFFu) : p;
  }
}

void check(cspt_status st)
{
  if (st != CSPT_OK) throw Error{st, std::string(cspt_last_error_message())};
}

}  // namespace

void quadtree_contains_properly(void const* x, void const* y, size_t n, uint32_t const* go,
                                size_t ngo, uint32_t const* po, size_t npo, uint32_t const* ro,
                                size_t nro, void const* vx, void const* vy, size_t nv,
                                cspt_dtype dtype, cspt_method method, cspt_allocator const* mr,
                                void* stream, uint32_t** out_point, uint32_t** out_part,
                                uint32_t** out_geom, size_t* out_n)
{
  cudaStream_t const s = static_cast<cudaStream_t>(stream);
  Allocator alloc(mr, s);
  size_t const npoly = npo - 1;
  size_t const es    = dtype == CSPT_FLOAT64 ? 8 : 4;

  // vertex extent (contains.py:48-51)
  double ext[4];
  {
    Buffer<long long> e(alloc, 4);
    long long const init[4] = {LLONG_MAX, LLONG_MAX, LLONG_MAX, LLONG_MAX};
    CSPT_CUDA_TRY(cudaMemcpyAsync(e.data(), init, sizeof init, cudaMemcpyHostToDevice, s));
    unsigned const grd = grid_for(nv, kContainsBlock, static_cast<unsigned>(num_sms()) * 4u);
    if (dtype == CSPT_FLOAT64)
      extent_kernel<double><<<grd, kContainsBlock, 0, s>>>(
        static_cast<double const*>(vx), static_cast<double const*>(vy), nv, e.data());
    else
      extent_kernel<float><<<grd, kContainsBlock, 0, s>>>(
        static_cast<float const*>(vx), static_cast<float const*>(vy), nv, e.data());
    CSPT_CHECK_LAUNCH();
    long long h[4];
    CSPT_CUDA_TRY(cudaMemcpyAsync(h, e.data(), sizeof h, cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    for (int j = 0; j < 4; ++j) {
      CSPT_EXPECTS(h[j] != LLONG_MAX, "polygon coordinates must not all be NaN");
      double const v = from_order_key64(h[j]);
      ext[j]         = j < 2 ? v : -v;
    }
  }
  // the coordinates' own precision, as the column reductions return them
  double x_min = ext[0], y_min = ext[1], x_max = ext[2], y_max = ext[3];
  double scale;
  int const max_depth = 15;
  if (dtype == CSPT_FLOAT64) {
    scale = std::max(x_max - x_min, y_max - y_min) / static_cast<double>((1 << max_depth) + 2);
  } else {
    float const w = static_cast<float>(x_max) - static_cast<float>(x_min);
    float const h = static_cast<float>(y_max) - static_cast<float>(y_min);
    scale         = static_cast<double>(std::max(w, h) / static_cast<float>((1 << max_depth) + 2));
  }
  int32_t const min_size = static_cast<int32_t>(std::ceil(std::sqrt(static_cast<double>(n))));

  // contains.py:52-61
  uint32_t* pi = nullptr;
  cspt_quadtree tree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
  uint32_t *pb = nullptr, *pq = nullptr, *op = nullptr, *oq = nullptr;
  size_t npairs = 0, m = 0;
  void* box[4]  = {nullptr, nullptr, nullptr, nullptr};
  auto release  = [&] {
    if (pi) alloc.deallocate(pi, n * 4);
    cspt_quadtree_free(mr, &tree, stream);
    for (void*& b : box)
      if (b) alloc.deallocate(b, npoly * es);
    if (pb) alloc.deallocate(pb, npairs * 4);
    if (pq) alloc.deallocate(pq, npairs * 4);
  };
  try {
    check(cspt_quadtree_on_points(x, y, n, dtype, x_min, x_max, y_min, y_max, scale,
                                  static_cast<int8_t>(max_depth), min_size, mr, stream, &pi,
                                  &tree));
    for (void*& b : box) b = alloc.allocate(npoly * es);
    check(cspt_polygon_bounding_boxes(po, npo, ro, nro, vx, vy, nv, dtype, 0.0, box[0], box[1],
                                      box[2], box[3], stream));
    check(cspt_join_quadtree_and_bounding_boxes(&tree, box[0], box[1], box[2], box[3], npoly,
                                                dtype, x_min, x_max, y_min, y_max, scale,
                                                static_cast<int8_t>(max_depth), mr, stream, &pb,
                                                &pq, &npairs));
    check(cspt_quadtree_point_in_polygon(pb, pq, npairs, &tree, pi, n, x, y, n, po, npo, ro,
                                         nro, vx, vy, nv, dtype, method, mr, stream, &op, &oq,
                                         &m));
    // contains.py:65-70 and the part -> multipolygon map
    uint32_t* geom = m ? static_cast<uint32_t*>(alloc.allocate(m * 4)) : nullptr;
    if (m) {
      Buffer<uint32_t> part_geom;
      if (go && ngo > 1) {
        part_geom = Buffer<uint32_t>(alloc, npoly);
        CSPT_CUDA_TRY(cudaMemsetAsync(part_geom.data(), 0xFF, npoly * 4, s));
        part_geometry_kernel<<<grid_for(ngo - 1, kContainsBlock), kContainsBlock, 0, s>>>(
          go, ngo - 1, npoly, part_geom.data());
        CSPT_CHECK_LAUNCH();
      }
      map_rows_kernel<<<grid_for(m, kContainsBlock, static_cast<unsigned>(num_sms()) * 8u),
                        kContainsBlock, 0, s>>>(oq, op, m, pi, n,
                                                part_geom.size() ? part_geom.data() : nullptr,
                                                npoly, geom);
      CSPT_CHECK_LAUNCH();
      CSPT_CUDA_TRY(cudaStreamSynchronize(s));  // part_geom and pi are released below
    }
    *out_point = oq;
    *out_part  = op;
    *out_geom  = geom;
    *out_n     = m;
  } catch (...) {
    if (op) alloc.deallocate(op, m * 4);
    if (oq) alloc.deallocate(oq, m * 4);
    release();
    throw;
  }
  release();
}

}  // namespace cspt
