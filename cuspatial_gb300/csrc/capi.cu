// extern "C" entry points: argument validation and empty-input rules of the
// libcuspatial column API, then dispatch to the kernels.
#include <atomic>
#include <functional>
#include <map>
#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace cspt {

// defined in the kernel translation units
void quadtree_on_points(void const* x, void const* y, size_t n, cspt_dtype dtype, double x_min,
                        double x_max, double y_min, double y_max, double scale, int max_depth,
                        int32_t max_size, Allocator const& alloc, uint32_t** out_point_indices,
                        cspt_quadtree* out_tree, void* ordered = nullptr);
void quadtree_on_points_from_host(void const* host_x, void const* host_y, void* dev_x,
                                  void* dev_y, size_t n, cspt_dtype dtype, double x_min,
                                  double x_max, double y_min, double y_max, double scale,
                                  int max_depth, int32_t max_size, Allocator const& alloc,
                                  uint32_t** out_point_indices, cspt_quadtree* out_tree,
                                  void* ordered                                    = nullptr,
                                  std::function<void(cudaStream_t)> const* after_copies = nullptr);
void point_in_polygon_join_host(void const* hx, void const* hy, size_t n, cspt_dtype dtype,
                                double x_min, double x_max, double y_min, double y_max,
                                double scale, int max_depth, int32_t max_size,
                                uint32_t const* hpo, size_t npo, uint32_t const* hro,
                                size_t nro, void const* hvx, void const* hvy, size_t nv,
                                cspt_method method, cspt_allocator const* mr, cudaStream_t s,
                                HostRows const& out, size_t* out_n, uint64_t* out_refined);
uint64_t& last_fallbacks();
uint64_t& last_group_scans();
uint64_t& last_f64_segments();
uint64_t& last_edge_free_pairs();
void points_in_quadtree_order(uint32_t const* point_indices, size_t n, void const* x,
                              void const* y, size_t npts, cspt_dtype dtype, void* out_xy,
                              cudaStream_t s);
void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);
void linestring_bounding_boxes(uint32_t const* ls_offsets, size_t nlo, void const* x,
                               void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                               void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);
void join_quadtree_and_bounding_boxes(cspt_quadtree const* tree, void const* bminx,
                                      void const* bminy, void const* bmaxx, void const* bmaxy,
                                      size_t nb, cspt_dtype dtype, double x_min, double y_min,
                                      double scale, int max_depth, Allocator const& alloc,
                                      uint32_t** out_box, uint32_t** out_node, size_t* out_n);
void quadtree_point_in_polygon(uint32_t const* pair_poly, uint32_t const* pair_quad,
                               size_t npairs, cspt_quadtree const* tree,
                               uint32_t const* point_indices, size_t npi, void const* x,
                               void const* y, uint32_t const* po, size_t npo, uint32_t const* ro,
                               size_t nro, void const* vx, void const* vy, size_t nv,
                               cspt_dtype dtype, cspt_method method, Allocator const& alloc,
                               uint32_t** out_poly, uint32_t** out_point, size_t* out_n,
                               uint64_t* out_refined, HostRows const* host = nullptr,
                               void const* ordered = nullptr);
void quadtree_point_to_nearest_linestring(uint32_t const* pair_ls, uint32_t const* pair_quad,
                                          size_t npairs, cspt_quadtree const* tree,
                                          uint32_t const* point_indices, size_t npi,
                                          void const* x, void const* y, uint32_t const* lso,
                                          size_t nlso, void const* lx, void const* ly,
                                          cspt_dtype dtype, cspt_method method,
                                          Allocator const& alloc, uint32_t* opt, uint32_t* ols,
                                          void* od, void const* ordered = nullptr);
void point_in_polygon(void const* x, void const* y, size_t n, uint32_t const* po, size_t npo,
                      uint32_t const* ro, size_t nro, void const* vx, void const* vy, size_t nv,
                      cspt_dtype dtype, cspt_method method, Allocator const& alloc, int32_t* out,
                      uint64_t* out_refined);
void pairwise_point_in_polygon(void const* x, void const* y, size_t n, uint32_t const* po,
                               uint32_t const* ro, void const* vx, void const* vy, size_t nv,
                               cspt_dtype dtype, cspt_method method, Allocator const& alloc,
                               uint8_t* out, uint64_t* out_refined);
void quadtree_contains_properly(void const* x, void const* y, size_t n, uint32_t const* go,
                                size_t ngo, uint32_t const* po, size_t npo, uint32_t const* ro,
                                size_t nro, void const* vx, void const* vy, size_t nv,
                                cspt_dtype dtype, cspt_method method, cspt_allocator const* mr,
                                void* stream, uint32_t** out_point, uint32_t** out_part,
                                uint32_t** out_geom, size_t* out_n);
void pairwise_point_linestring(size_t n, uint32_t const* pgo, size_t npgo, void const* x,
                               void const* y, size_t np, uint32_t const* lgo, size_t nlgo,
                               uint32_t const* lpo, size_t nlpo, void const* lx, void const* ly,
                               size_t nv, cspt_dtype dtype, cspt_method method,
                               Allocator const& alloc, void* od, int32_t* opt, int32_t* ols,
                               int32_t* oseg, void* oxy, uint64_t* out_refined);

namespace {
thread_local std::string t_last_error;

// Pairs of a pairwise (multi)point - (multi)linestring call: multipoints
// count geometry offsets, single points count points; multilinestrings
// count geometry offsets, single linestrings count part offsets.
struct PlPairs {
  size_t points, linestrings;
};
PlPairs pl_pairs(uint32_t const* pgo, size_t npgo, size_t np, uint32_t const* lgo, size_t nlgo,
                 size_t nlpo)
{
  PlPairs r;
  r.points      = pgo ? (npgo > 0 ? npgo - 1 : 0) : np;
  r.linestrings = lgo ? (nlgo > 0 ? nlgo - 1 : 0) : (nlpo > 0 ? nlpo - 1 : 0);
  return r;
}
thread_local uint64_t t_last_refined = 0;

void check_dtype(cspt_dtype dtype)
{
  if (dtype != CSPT_FLOAT32 && dtype != CSPT_FLOAT64)
    throw Error{CSPT_UNSUPPORTED, "Only floating-point types are supported"};
}
cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }
}  // namespace

void set_last_error(std::string const& msg) { t_last_error = msg; }
void clear_last_error() { t_last_error.clear(); }

int num_sms()
{
  // one entry per device ordinal, filled on first use with that device current
  constexpr int kMaxDevices = 64;
  static std::atomic<int> sms[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    (void)cudaGetLastError();
    dev = 0;
  }
  int n = sms[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    (void)cudaGetLastError();
    n = 152;  // GB300
  }
  sms[dev].store(n, std::memory_order_relaxed);
  return n;
}

cudaMemPool_t library_pool()
{
  constexpr int kMaxDevices = 64;
  static std::atomic<cudaMemPool_t> pools[kMaxDevices];
  static std::mutex mu;
  int dev = 0;
  CSPT_CUDA_TRY(cudaGetDevice(&dev));
  CSPT_EXPECTS(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
  cudaMemPool_t p = pools[dev].load(std::memory_order_acquire);
  if (p) return p;
  std::lock_guard<std::mutex> lk(mu);
  p = pools[dev].load(std::memory_order_relaxed);
  if (p) return p;
  cudaMemPoolProps props{};
  props.allocType     = cudaMemAllocationTypePinned;
  props.handleTypes   = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id   = dev;
  CSPT_CUDA_TRY(cudaMemPoolCreate(&p, &props));
  uint64_t keep = std::numeric_limits<uint64_t>::max();
  CSPT_CUDA_TRY(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
  pools[dev].store(p, std::memory_order_release);
  return p;
}

cudaStream_t library_stream()
{
  constexpr int kMaxDevices = 64;
  static std::atomic<cudaStream_t> streams[kMaxDevices];
  static std::mutex mu;
  int dev = 0;
  CSPT_CUDA_TRY(cudaGetDevice(&dev));
  CSPT_EXPECTS(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
  cudaStream_t st = streams[dev].load(std::memory_order_acquire);
  if (st) return st;
  std::lock_guard<std::mutex> lk(mu);
  st = streams[dev].load(std::memory_order_relaxed);
  if (st) return st;
  CSPT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  streams[dev].store(st, std::memory_order_release);
  return st;
}

cudaStream_t side_stream(int k)
{
  struct Streams {
    std::vector<cudaStream_t> by_device;  // kSideStreams per device
    ~Streams()
    {
      for (cudaStream_t st : by_device)
        if (st) (void)cudaStreamDestroy(st);
    }
  };
  thread_local Streams t;
  CSPT_EXPECTS(k >= 0 && k < kSideStreams, "side stream index out of range");
  int dev = 0;
  CSPT_CUDA_TRY(cudaGetDevice(&dev));
  size_t const i = static_cast<size_t>(dev) * kSideStreams + static_cast<size_t>(k);
  if (i >= t.by_device.size()) t.by_device.resize(i + 1, nullptr);
  if (!t.by_device[i])
    CSPT_CUDA_TRY(cudaStreamCreateWithFlags(&t.by_device[i], cudaStreamNonBlocking));
  return t.by_device[i];
}

void stream_wait(cudaStream_t waiter, cudaStream_t on)
{
  cudaEvent_t e = nullptr;
  CSPT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaError_t err = cudaEventRecord(e, on);
  if (err == cudaSuccess) err = cudaStreamWaitEvent(waiter, e, 0);
  (void)cudaEventDestroy(e);
  CSPT_CUDA_TRY(err);
}

void StreamJoin::join()
{
  if (!side_) return;
  cudaStream_t const side = side_;
  side_                   = nullptr;
  cudaEvent_t e           = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess &&
      cudaEventRecord(e, side) == cudaSuccess && cudaStreamWaitEvent(main_, e, 0) == cudaSuccess) {
    (void)cudaEventDestroy(e);
    return;
  }
  (void)cudaGetLastError();
  if (e) (void)cudaEventDestroy(e);
  (void)cudaStreamSynchronize(side);  // the host waits instead
}

uint64_t last_refined() { return t_last_refined; }

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_profile{0};
std::mutex g_prof_mu;
struct Pending {
  std::string name;
  cudaEvent_t start, stop;
};
std::vector<Pending> g_pending;
std::map<std::string, std::pair<double, uint64_t>> g_totals;

void resolve_pending()
{
  for (auto& p : g_pending) {
    float ms = 0.0f;
    if (cudaEventSynchronize(p.stop) == cudaSuccess &&
        cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
      auto& t = g_totals[p.name];
      t.first += ms;
      t.second += 1;
    }
    cudaEventDestroy(p.start);
    cudaEventDestroy(p.stop);
  }
  g_pending.clear();
  (void)cudaGetLastError();
}
}  // namespace

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

// Each named stage is also an NVTX range (key, sort, tree, boxes, join
// traversal, index, frames, pip, expansion, nearest, ...), so a profiler's
// timeline shows the library's stages; without a profiler attached the
// range calls return at once.
KernelTimer::KernelTimer(char const* name, cudaStream_t stream) : name_(name), stream_(stream)
{
  nvtxRangePushA(name);
  if (!g_profile.load(std::memory_order_relaxed)) return;
  if (cudaEventCreate(&start_) != cudaSuccess || cudaEventCreate(&stop_) != cudaSuccess) {
    (void)cudaGetLastError();
    start_ = stop_ = nullptr;
    return;
  }
  cudaEventRecord(start_, stream_);
}

KernelTimer::~KernelTimer()
{
  nvtxRangePop();
  if (!start_) return;
  cudaEventRecord(stop_, stream_);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_pending.push_back(Pending{name_, start_, stop_});
}

}  // namespace cspt

using namespace cspt;

extern "C" {

const char* cspt_last_error_message(void) { return t_last_error.c_str(); }

const char* cspt_version(void) { return "cuspatial_gb300 0.1 (sm_103a)"; }

// Diagnostics without a reference counterpart: kernel launch counter and
// event timing of the named kernels (pip_bits, pip_expand, join_count,
// join_write, nearest, quadtree_build).
uint64_t cspt_launch_count(void) { return g_launches.load(); }

cspt_status cspt_pool_trim(size_t min_bytes_to_keep)
{
  return guarded([&] {
    CSPT_CUDA_TRY(cudaDeviceSynchronize());
    CSPT_CUDA_TRY(cudaMemPoolTrimTo(library_pool(), min_bytes_to_keep));
  });
}

void cspt_profile_enable(int on)
{
  std::lock_guard<std::mutex> lk(g_prof_mu);
  resolve_pending();
  g_totals.clear();
  g_profile.store(on ? 1 : 0);
}

int cspt_profile_read(const char* name, double* total_ms, uint64_t* launches)
{
  std::lock_guard<std::mutex> lk(g_prof_mu);
  resolve_pending();
  auto it = g_totals.find(name ? name : "");
  if (it == g_totals.end()) {
    if (total_ms) *total_ms = 0.0;
    if (launches) *launches = 0;
    return 0;
  }
  if (total_ms) *total_ms = it->second.first;
  if (launches) *launches = it->second.second;
  return 1;
}

// Candidates re-evaluated in float64 by the last filtered point-in-polygon
// call on this thread (diagnostic; not part of the reference interface).
uint64_t cspt_last_refined_count(void) { return t_last_refined; }

uint64_t cspt_last_edge_free_pairs(void) { return last_edge_free_pairs(); }

void cspt_last_nearest_stats(uint64_t* points_folded_whole, uint64_t* groups_scanned,
                             uint64_t* float64_segments)
{
  if (points_folded_whole) *points_folded_whole = last_fallbacks();
  if (groups_scanned) *groups_scanned = last_group_scans();
  if (float64_segments) *float64_segments = last_f64_segments();
}

void cspt_free(const cspt_allocator* mr, void* ptr, size_t bytes, void* stream)
{
  Allocator(mr, as_stream(stream)).deallocate(ptr, bytes);
}

void cspt_quadtree_free(const cspt_allocator* mr, cspt_quadtree* tree, void* stream)
{
  if (!tree) return;
  Allocator a(mr, as_stream(stream));
  size_t const q = tree->num_nodes;
  a.deallocate(tree->key, q * 4);
  a.deallocate(tree->level, q);
  a.deallocate(tree->is_internal_node, q);
  a.deallocate(tree->length, q * 4);
  a.deallocate(tree->offset, q * 4);
  *tree = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
}

cspt_status cspt_quadtree_on_points(const void* x, const void* y, size_t num_points,
                                    cspt_dtype dtype, double x_min, double x_max, double y_min,
                                    double y_max, double scale, int8_t max_depth,
                                    int32_t max_size, const cspt_allocator* mr, void* stream,
                                    uint32_t** out_point_indices, cspt_quadtree* out_tree)
{
  return guarded([&] {
    CSPT_EXPECTS(out_point_indices && out_tree, "output pointers must not be null");
    *out_point_indices = nullptr;
    *out_tree          = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    check_dtype(dtype);
    if (num_points == 0) return;  // point_quadtree.cu:167-177
    CSPT_EXPECTS(x && y, "x and y columns must have the same length");
    Allocator alloc(mr, as_stream(stream));
    quadtree_on_points(x, y, num_points, dtype, x_min, x_max, y_min, y_max, scale, max_depth,
                       max_size, alloc, out_point_indices, out_tree);
  });
}

cspt_status cspt_quadtree_on_points_host(const void* host_x, const void* host_y,
                                         size_t num_points, cspt_dtype dtype, double x_min,
                                         double x_max, double y_min, double y_max, double scale,
                                         int8_t max_depth, int32_t max_size, void* device_x,
                                         void* device_y, const cspt_allocator* mr, void* stream,
                                         uint32_t** out_point_indices, cspt_quadtree* out_tree)
{
  return guarded([&] {
    CSPT_EXPECTS(out_point_indices && out_tree, "output pointers must not be null");
    *out_point_indices = nullptr;
    *out_tree          = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    check_dtype(dtype);
    if (num_points == 0) return;  // point_quadtree.cu:167-177
    CSPT_EXPECTS(host_x && host_y && device_x && device_y,
                 "x and y columns must have the same length");
    Allocator alloc(mr, as_stream(stream));
    quadtree_on_points_from_host(host_x, host_y, device_x, device_y, num_points, dtype, x_min,
                                 x_max, y_min, y_max, scale, max_depth, max_size, alloc,
                                 out_point_indices, out_tree);
  });
}

cspt_status cspt_quadtree_on_points_ordered(const void* x, const void* y, size_t num_points,
                                            cspt_dtype dtype, double x_min, double x_max,
                                            double y_min, double y_max, double scale,
                                            int8_t max_depth, int32_t max_size,
                                            const cspt_allocator* mr, void* stream,
                                            uint32_t** out_point_indices,
                                            cspt_quadtree* out_tree, void* out_ordered_xy)
{
  return guarded([&] {
    CSPT_EXPECTS(out_point_indices && out_tree, "output pointers must not be null");
    *out_point_indices = nullptr;
    *out_tree          = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    check_dtype(dtype);
    if (num_points == 0) return;  // point_quadtree.cu:167-177
    CSPT_EXPECTS(x && y, "x and y columns must have the same length");
    size_t const vec = dtype == CSPT_FLOAT64 ? 16 : 8;
    CSPT_EXPECTS(out_ordered_xy && reinterpret_cast<uintptr_t>(out_ordered_xy) % vec == 0,
                 "the ordered points must start on a " + std::to_string(vec) +
                   "-byte boundary");
    Allocator alloc(mr, as_stream(stream));
    quadtree_on_points(x, y, num_points, dtype, x_min, x_max, y_min, y_max, scale, max_depth,
                       max_size, alloc, out_point_indices, out_tree, out_ordered_xy);
  });
}

cspt_status cspt_quadtree_on_points_host_ordered(
  const void* host_x, const void* host_y, size_t num_points, cspt_dtype dtype, double x_min,
  double x_max, double y_min, double y_max, double scale, int8_t max_depth, int32_t max_size,
  void* device_x, void* device_y, const cspt_allocator* mr, void* stream,
  uint32_t** out_point_indices, cspt_quadtree* out_tree, void* out_ordered_xy)
{
  return guarded([&] {
    CSPT_EXPECTS(out_point_indices && out_tree, "output pointers must not be null");
    *out_point_indices = nullptr;
    *out_tree          = cspt_quadtree{nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    check_dtype(dtype);
    if (num_points == 0) return;  // point_quadtree.cu:167-177
    CSPT_EXPECTS(host_x && host_y && device_x && device_y,
                 "x and y columns must have the same length");
    size_t const vec = dtype == CSPT_FLOAT64 ? 16 : 8;
    CSPT_EXPECTS(out_ordered_xy && reinterpret_cast<uintptr_t>(out_ordered_xy) % vec == 0,
                 "the ordered points must start on a " + std::to_string(vec) +
                   "-byte boundary");
    Allocator alloc(mr, as_stream(stream));
    quadtree_on_points_from_host(host_x, host_y, device_x, device_y, num_points, dtype, x_min,
                                 x_max, y_min, y_max, scale, max_depth, max_size, alloc,
                                 out_point_indices, out_tree, out_ordered_xy);
  });
}

cspt_status cspt_points_in_quadtree_order(const uint32_t* point_indices,
                                          size_t num_point_indices, const void* x, const void* y,
                                          size_t num_points, cspt_dtype dtype, void* out_xy,
                                          void* stream)
{
  return guarded([&] {
    check_dtype(dtype);
    if (num_point_indices == 0) return;
    CSPT_EXPECTS(point_indices && x && y && out_xy, "input and output arrays must not be null");
    size_t const vec = dtype == CSPT_FLOAT64 ? 16 : 8;
    CSPT_EXPECTS(reinterpret_cast<uintptr_t>(out_xy) % vec == 0,
                 "the ordered points must start on a " + std::to_string(vec) +
                   "-byte boundary");
    points_in_quadtree_order(point_indices, num_point_indices, x, y, num_points, dtype, out_xy,
                             as_stream(stream));
  });
}

cspt_status cspt_polygon_bounding_boxes(const uint32_t* poly_offsets, size_t num_poly_offsets,
                                        const uint32_t* ring_offsets, size_t num_ring_offsets,
                                        const void* x, const void* y, size_t num_vertices,
                                        cspt_dtype dtype, double expansion_radius,
                                        void* out_min_x, void* out_min_y, void* out_max_x,
                                        void* out_max_y, void* stream)
{
  return guarded([&] {
    check_dtype(dtype);
    size_t const np = num_poly_offsets > 0 ? num_poly_offsets - 1 : 0;
    if (np == 0) return;  // polygon_bounding_boxes.cu:147-155
    // CUSPATIAL_EXPECTS_VALID_POLYGON_SIZES (detail/utility/validation.hpp:87-92)
    CSPT_EXPECTS(num_poly_offsets > 0, "Polygon offsets must contain at least one (1) value");
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    if (num_ring_offsets < 2 || num_vertices == 0) {
      // bounding_boxes.cuh:166: no rings or no vertices -> nothing written
      return;
    }
    Allocator alloc(nullptr, as_stream(stream));
    polygon_bounding_boxes(poly_offsets, num_poly_offsets, ring_offsets, num_ring_offsets, x, y,
                           num_vertices, dtype, expansion_radius, out_min_x, out_min_y,
                           out_max_x, out_max_y, alloc);
  });
}

cspt_status cspt_linestring_bounding_boxes(const uint32_t* linestring_offsets,
                                           size_t num_linestring_offsets, const void* x,
                                           const void* y, size_t num_vertices, cspt_dtype dtype,
                                           double expansion_radius, void* out_min_x,
                                           void* out_min_y, void* out_max_x, void* out_max_y,
                                           void* stream)
{
  return guarded([&] {
    check_dtype(dtype);
    size_t const nl = num_linestring_offsets > 0 ? num_linestring_offsets - 1 : 0;
    // linestring_bounding_boxes.cu:135-141
    CSPT_EXPECTS(expansion_radius >= 0, "expansion radius must be greater or equal than 0");
    CSPT_EXPECTS(num_vertices >= 2 * nl, "all linestrings must have at least 2 vertices");
    if (num_linestring_offsets == 0 || num_vertices == 0 || nl == 0) return;
    Allocator alloc(nullptr, as_stream(stream));
    linestring_bounding_boxes(linestring_offsets, num_linestring_offsets, x, y, num_vertices,
                              dtype, expansion_radius, out_min_x, out_min_y, out_max_x,
                              out_max_y, alloc);
  });
}

cspt_status cspt_join_quadtree_and_bounding_boxes(
  const cspt_quadtree* tree, const void* bbox_min_x, const void* bbox_min_y,
  const void* bbox_max_x, const void* bbox_max_y, size_t num_bboxes, cspt_dtype dtype,
  double x_min, double x_max, double y_min, double y_max, double scale, int8_t max_depth,
  const cspt_allocator* mr, void* stream, uint32_t** out_bbox_offset,
  uint32_t** out_quad_offset, size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_bbox_offset && out_quad_offset && out_num_pairs,
                 "output pointers must not be null");
    *out_bbox_offset = nullptr;
    *out_quad_offset = nullptr;
    *out_num_pairs   = 0;
    CSPT_EXPECTS(tree, "quadtree table must have 5 columns");
    check_dtype(dtype);
    // quadtree_bbox_filtering.cu:100-106
    CSPT_EXPECTS(scale > 0, "scale must be positive");
    CSPT_EXPECTS(x_min < x_max && y_min < y_max,
                 "invalid bounding box (x_min, x_max, y_min, y_max)");
    CSPT_EXPECTS(max_depth > 0 && max_depth < 16,
                 "maximum depth must be positive and less than 16");
    if (tree->num_nodes == 0 || num_bboxes == 0) return;  // :108-114
    Allocator alloc(mr, as_stream(stream));
    join_quadtree_and_bounding_boxes(tree, bbox_min_x, bbox_min_y, bbox_max_x, bbox_max_y,
                                     num_bboxes, dtype, x_min, y_min, scale, max_depth, alloc,
                                     out_bbox_offset, out_quad_offset, out_num_pairs);
  });
}

cspt_status cspt_quadtree_point_in_polygon(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* poly_offsets,
  size_t num_poly_offsets, const uint32_t* ring_offsets, size_t num_ring_offsets,
  const void* poly_x, const void* poly_y, size_t num_poly_vertices, cspt_dtype dtype,
  cspt_method method, const cspt_allocator* mr, void* stream, uint32_t** out_polygon_index,
  uint32_t** out_point_index, size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_polygon_index && out_point_index && out_num_pairs,
                 "output pointers must not be null");
    *out_polygon_index = nullptr;
    *out_point_index   = nullptr;
    *out_num_pairs     = 0;
    t_last_refined     = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    // quadtree_point_in_polygon.cu:154-169
    CSPT_EXPECTS(num_point_indices == num_points,
                 "number of points must be the same for both x and y columns");
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    // :171-178
    if (num_pairs == 0 || tree->num_nodes == 0 || num_point_indices == 0 ||
        num_poly_offsets == 0)
      return;
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    Allocator alloc(mr, as_stream(stream));
    uint64_t refined = 0;
    quadtree_point_in_polygon(pair_polygon, pair_quad, num_pairs, tree, point_indices,
                              num_point_indices, x, y, poly_offsets, num_poly_offsets,
                              ring_offsets, num_ring_offsets, poly_x, poly_y, num_poly_vertices,
                              dtype, method, alloc, out_polygon_index, out_point_index,
                              out_num_pairs, &refined);
    t_last_refined = refined;
  });
}

cspt_status cspt_quadtree_point_in_polygon_host(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* poly_offsets,
  size_t num_poly_offsets, const uint32_t* ring_offsets, size_t num_ring_offsets,
  const void* poly_x, const void* poly_y, size_t num_poly_vertices, cspt_dtype dtype,
  cspt_method method, const cspt_allocator* mr, void* stream, uint32_t* host_polygon_index,
  uint32_t* host_point_index, size_t host_capacity, size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_num_pairs, "output pointers must not be null");
    *out_num_pairs = 0;
    t_last_refined = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    // quadtree_point_in_polygon.cu:154-169
    CSPT_EXPECTS(num_point_indices == num_points,
                 "number of points must be the same for both x and y columns");
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    CSPT_EXPECTS(host_capacity == 0 || (host_polygon_index && host_point_index),
                 "host output arrays must not be null");
    // :171-178
    if (num_pairs == 0 || tree->num_nodes == 0 || num_point_indices == 0 ||
        num_poly_offsets == 0)
      return;
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    Allocator alloc(mr, as_stream(stream));
    uint64_t refined = 0;
    HostRows const host{host_polygon_index, host_point_index, host_capacity};
    quadtree_point_in_polygon(pair_polygon, pair_quad, num_pairs, tree, point_indices,
                              num_point_indices, x, y, poly_offsets, num_poly_offsets,
                              ring_offsets, num_ring_offsets, poly_x, poly_y, num_poly_vertices,
                              dtype, method, alloc, nullptr, nullptr, out_num_pairs, &refined,
                              &host);
    t_last_refined = refined;
  });
}

cspt_status cspt_point_in_polygon_join_host(
  const void* host_x, const void* host_y, size_t num_points, cspt_dtype dtype, double x_min,
  double x_max, double y_min, double y_max, double scale, int8_t max_depth, int32_t max_size,
  const uint32_t* host_poly_offsets, size_t num_poly_offsets, const uint32_t* host_ring_offsets,
  size_t num_ring_offsets, const void* host_poly_x, const void* host_poly_y,
  size_t num_poly_vertices, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* host_polygon_index, uint32_t* host_point_index, size_t host_capacity,
  size_t* out_num_rows)
{
  return guarded([&] {
    CSPT_EXPECTS(out_num_rows, "output pointers must not be null");
    *out_num_rows  = 0;
    t_last_refined = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    CSPT_EXPECTS(host_capacity == 0 || (host_polygon_index && host_point_index),
                 "host output arrays must not be null");
    // join.py:163-180: corners ordered, scale clamped to the tree's minimum;
    // then quadtree_bbox_filtering.cu:100-106
    double const x0 = x_min < x_max ? x_min : x_max, x1 = x_min < x_max ? x_max : x_min;
    double const y0 = y_min < y_max ? y_min : y_max, y1 = y_min < y_max ? y_max : y_min;
    CSPT_EXPECTS(max_depth > 0 && max_depth < 16,
                 "maximum depth must be positive and less than 16");
    double const span      = (x1 - x0) > (y1 - y0) ? (x1 - x0) : (y1 - y0);
    double const min_scale = span / static_cast<double>((1 << max_depth) + 2);
    double const sc        = scale > min_scale ? scale : min_scale;
    CSPT_EXPECTS(sc > 0, "scale must be positive");
    CSPT_EXPECTS(x0 < x1 && y0 < y1, "invalid bounding box (x_min, x_max, y_min, y_max)");
    if (num_points == 0 || num_poly_offsets < 2 || num_ring_offsets < 2 ||
        num_poly_vertices == 0)
      return;
    CSPT_EXPECTS(host_x && host_y && host_poly_offsets && host_ring_offsets && host_poly_x &&
                   host_poly_y,
                 "input columns must not be null");
    uint64_t refined = 0;
    HostRows const host{host_polygon_index, host_point_index, host_capacity};
    point_in_polygon_join_host(host_x, host_y, num_points, dtype, x0, x1, y0, y1, sc, max_depth,
                               max_size, host_poly_offsets, num_poly_offsets, host_ring_offsets,
                               num_ring_offsets, host_poly_x, host_poly_y, num_poly_vertices,
                               method, mr, as_stream(stream), host, out_num_rows, &refined);
    t_last_refined = refined;
  });
}

cspt_status cspt_quadtree_point_to_nearest_linestring(
  const uint32_t* pair_linestring, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const uint32_t* point_indices, size_t num_point_indices,
  const void* x, const void* y, size_t num_points, const uint32_t* linestring_offsets,
  size_t num_linestring_offsets, const void* ls_x, const void* ls_y, size_t num_ls_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* out_point_index, uint32_t* out_linestring_index, void* out_distance,
  size_t* out_num_rows)
{
  return guarded([&] {
    (void)num_ls_vertices;
    CSPT_EXPECTS(out_num_rows, "output pointers must not be null");
    *out_num_rows = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    // quadtree_point_to_nearest_linestring.cu:153-165
    CSPT_EXPECTS(num_point_indices == num_points,
                 "number of points must be the same for both x and y columns");
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown nearest-linestring method");
    // :167-175
    if (num_pairs == 0 || tree->num_nodes == 0 || num_point_indices == 0 ||
        num_linestring_offsets == 0)
      return;
    CSPT_EXPECTS(out_point_index && out_linestring_index && out_distance,
                 "output pointers must not be null");
    Allocator alloc(mr, as_stream(stream));
    quadtree_point_to_nearest_linestring(pair_linestring, pair_quad, num_pairs, tree,
                                         point_indices, num_point_indices, x, y,
                                         linestring_offsets, num_linestring_offsets, ls_x, ls_y,
                                         dtype, method, alloc, out_point_index,
                                         out_linestring_index, out_distance);
    *out_num_rows = num_point_indices;
  });
}

// Points in quadtree order (cspt_points_in_quadtree_order) given instead of
// point_indices, x and y: present, aligned for one vector load per point.
static void check_ordered(void const* ordered_xy, cspt_dtype dtype)
{
  size_t const vec = dtype == CSPT_FLOAT64 ? 16 : 8;
  CSPT_EXPECTS(ordered_xy, "the ordered points must not be null");
  CSPT_EXPECTS(reinterpret_cast<uintptr_t>(ordered_xy) % vec == 0,
               "the ordered points must start on a " + std::to_string(vec) + "-byte boundary");
}

cspt_status cspt_quadtree_point_in_polygon_ordered(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* poly_x, const void* poly_y, size_t num_poly_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t** out_polygon_index, uint32_t** out_point_index, size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_polygon_index && out_point_index && out_num_pairs,
                 "output pointers must not be null");
    *out_polygon_index = nullptr;
    *out_point_index   = nullptr;
    *out_num_pairs     = 0;
    t_last_refined     = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    if (num_pairs == 0 || tree->num_nodes == 0 || num_points == 0 || num_poly_offsets == 0)
      return;
    check_ordered(ordered_xy, dtype);
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    Allocator alloc(mr, as_stream(stream));
    uint64_t refined = 0;
    quadtree_point_in_polygon(pair_polygon, pair_quad, num_pairs, tree, nullptr, num_points,
                              nullptr, nullptr, poly_offsets, num_poly_offsets, ring_offsets,
                              num_ring_offsets, poly_x, poly_y, num_poly_vertices, dtype, method,
                              alloc, out_polygon_index, out_point_index, out_num_pairs, &refined,
                              nullptr, ordered_xy);
    t_last_refined = refined;
  });
}

cspt_status cspt_quadtree_point_in_polygon_host_ordered(
  const uint32_t* pair_polygon, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* poly_offsets, size_t num_poly_offsets, const uint32_t* ring_offsets,
  size_t num_ring_offsets, const void* poly_x, const void* poly_y, size_t num_poly_vertices,
  cspt_dtype dtype, cspt_method method, const cspt_allocator* mr, void* stream,
  uint32_t* host_polygon_index, uint32_t* host_point_index, size_t host_capacity,
  size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_num_pairs, "output pointers must not be null");
    *out_num_pairs = 0;
    t_last_refined = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    CSPT_EXPECTS(host_capacity == 0 || (host_polygon_index && host_point_index),
                 "host output arrays must not be null");
    if (num_pairs == 0 || tree->num_nodes == 0 || num_points == 0 || num_poly_offsets == 0)
      return;
    check_ordered(ordered_xy, dtype);
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    Allocator alloc(mr, as_stream(stream));
    uint64_t refined = 0;
    HostRows const host{host_polygon_index, host_point_index, host_capacity};
    quadtree_point_in_polygon(pair_polygon, pair_quad, num_pairs, tree, nullptr, num_points,
                              nullptr, nullptr, poly_offsets, num_poly_offsets, ring_offsets,
                              num_ring_offsets, poly_x, poly_y, num_poly_vertices, dtype, method,
                              alloc, nullptr, nullptr, out_num_pairs, &refined, &host,
                              ordered_xy);
    t_last_refined = refined;
  });
}

cspt_status cspt_quadtree_point_to_nearest_linestring_ordered(
  const uint32_t* pair_linestring, const uint32_t* pair_quad, size_t num_pairs,
  const cspt_quadtree* tree, const void* ordered_xy, size_t num_points,
  const uint32_t* linestring_offsets, size_t num_linestring_offsets, const void* ls_x,
  const void* ls_y, size_t num_ls_vertices, cspt_dtype dtype, cspt_method method,
  const cspt_allocator* mr, void* stream, uint32_t* out_point_index,
  uint32_t* out_linestring_index, void* out_distance, size_t* out_num_rows)
{
  return guarded([&] {
    (void)num_ls_vertices;
    CSPT_EXPECTS(out_num_rows, "output pointers must not be null");
    *out_num_rows = 0;
    CSPT_EXPECTS(tree, "a quadtree table must have 5 columns");
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown nearest-linestring method");
    if (num_pairs == 0 || tree->num_nodes == 0 || num_points == 0 ||
        num_linestring_offsets == 0)
      return;
    check_ordered(ordered_xy, dtype);
    CSPT_EXPECTS(out_point_index && out_linestring_index && out_distance,
                 "output pointers must not be null");
    Allocator alloc(mr, as_stream(stream));
    quadtree_point_to_nearest_linestring(pair_linestring, pair_quad, num_pairs, tree, nullptr,
                                         num_points, nullptr, nullptr, linestring_offsets,
                                         num_linestring_offsets, ls_x, ls_y, dtype, method,
                                         alloc, out_point_index, out_linestring_index,
                                         out_distance, ordered_xy);
    *out_num_rows = num_points;
  });
}

cspt_status cspt_point_in_polygon(const void* x, const void* y, size_t num_points,
                                  const uint32_t* poly_offsets, size_t num_poly_offsets,
                                  const uint32_t* ring_offsets, size_t num_ring_offsets,
                                  const void* poly_x, const void* poly_y,
                                  size_t num_poly_vertices, cspt_dtype dtype, cspt_method method,
                                  const cspt_allocator* mr, void* stream, int32_t* out)
{
  return guarded([&] {
    t_last_refined = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    // point_in_polygon.cu:64-66: an empty point column returns before the
    // polygon count is checked
    if (num_points == 0) return;
    size_t const npoly = num_poly_offsets > 0 ? num_poly_offsets - 1 : 0;
    // detail/point_in_polygon.cuh:93-94
    CSPT_EXPECTS(npoly <= 31, "Number of polygons cannot exceed 31");
    CSPT_EXPECTS(out, "output pointers must not be null");
    Allocator alloc(mr, as_stream(stream));
    if (npoly == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(out, 0, num_points * sizeof(int32_t), as_stream(stream)));
      return;
    }
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    uint64_t refined = 0;
    point_in_polygon(x, y, num_points, poly_offsets, num_poly_offsets, ring_offsets,
                     num_ring_offsets, poly_x, poly_y, num_poly_vertices, dtype, method, alloc,
                     out, &refined);
    t_last_refined = refined;
  });
}

cspt_status cspt_pairwise_point_in_polygon(const void* x, const void* y, size_t num_points,
                                           const uint32_t* poly_offsets, size_t num_poly_offsets,
                                           const uint32_t* ring_offsets, size_t num_ring_offsets,
                                           const void* poly_x, const void* poly_y,
                                           size_t num_poly_vertices, cspt_dtype dtype,
                                           cspt_method method, const cspt_allocator* mr,
                                           void* stream, uint8_t* out)
{
  return guarded([&] {
    t_last_refined = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    // point_in_polygon.cu:133-136
    size_t const npoly = num_poly_offsets > 0 ? num_poly_offsets - 1 : 0;
    CSPT_EXPECTS(num_points == npoly, "Must pass in the same number of points as polygons.");
    if (num_points == 0) return;
    CSPT_EXPECTS(out, "output pointers must not be null");
    CSPT_EXPECTS(num_ring_offsets > 0,
                 "Polygon ring offsets must contain at least one (1) value");
    Allocator alloc(mr, as_stream(stream));
    uint64_t refined = 0;
    pairwise_point_in_polygon(x, y, num_points, poly_offsets, ring_offsets, poly_x, poly_y,
                              num_poly_vertices, dtype, method, alloc, out, &refined);
    t_last_refined = refined;
  });
}

cspt_status cspt_quadtree_contains_properly(
  const void* x, const void* y, size_t num_points, const uint32_t* geometry_offsets,
  size_t num_geometry_offsets, const uint32_t* part_offsets, size_t num_part_offsets,
  const uint32_t* ring_offsets, size_t num_ring_offsets, const void* poly_x, const void* poly_y,
  size_t num_poly_vertices, cspt_dtype dtype, cspt_method method, const cspt_allocator* mr,
  void* stream, uint32_t** out_point_index, uint32_t** out_part_index,
  uint32_t** out_geometry_index, size_t* out_num_pairs)
{
  return guarded([&] {
    CSPT_EXPECTS(out_point_index && out_part_index && out_geometry_index && out_num_pairs,
                 "output pointers must not be null");
    *out_point_index    = nullptr;
    *out_part_index     = nullptr;
    *out_geometry_index = nullptr;
    *out_num_pairs      = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    // contains.py:46-47: no polygons, no rows
    if (num_part_offsets < 2 || num_poly_vertices == 0) return;
    quadtree_contains_properly(x, y, num_points, geometry_offsets, num_geometry_offsets,
                               part_offsets, num_part_offsets, ring_offsets, num_ring_offsets,
                               poly_x, poly_y, num_poly_vertices, dtype, method, mr, stream,
                               out_point_index, out_part_index, out_geometry_index,
                               out_num_pairs);
  });
}

cspt_status cspt_pairwise_point_linestring_distance(
  const uint32_t* point_geometry_offsets, size_t num_point_geometry_offsets, const void* x,
  const void* y, size_t num_points, const uint32_t* linestring_geometry_offsets,
  size_t num_linestring_geometry_offsets, const uint32_t* linestring_part_offsets,
  size_t num_linestring_part_offsets, const void* ls_x, const void* ls_y,
  size_t num_ls_vertices, cspt_dtype dtype, cspt_method method, void* stream,
  void* out_distance)
{
  return guarded([&] {
    t_last_refined = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown distance method");
    PlPairs const pr = pl_pairs(point_geometry_offsets, num_point_geometry_offsets, num_points,
                                linestring_geometry_offsets, num_linestring_geometry_offsets,
                                num_linestring_part_offsets);
    // point_linestring_distance.cu:92-93
    CSPT_EXPECTS(pr.points == pr.linestrings,
                 "Inputs should have the same number of geometries.");
    if (pr.points == 0) return;
    CSPT_EXPECTS(out_distance, "output pointers must not be null");
    Allocator alloc(nullptr, as_stream(stream));
    uint64_t refined = 0;
    pairwise_point_linestring(pr.points, point_geometry_offsets, num_point_geometry_offsets, x,
                              y, num_points, linestring_geometry_offsets,
                              num_linestring_geometry_offsets, linestring_part_offsets,
                              num_linestring_part_offsets, ls_x, ls_y, num_ls_vertices, dtype,
                              method, alloc, out_distance, nullptr, nullptr, nullptr, nullptr,
                              &refined);
    t_last_refined = refined;
  });
}

cspt_status cspt_pairwise_point_linestring_nearest_points(
  const uint32_t* point_geometry_offsets, size_t num_point_geometry_offsets, const void* x,
  const void* y, size_t num_points, const uint32_t* linestring_geometry_offsets,
  size_t num_linestring_geometry_offsets, const uint32_t* linestring_part_offsets,
  size_t num_linestring_part_offsets, const void* ls_x, const void* ls_y,
  size_t num_ls_vertices, cspt_dtype dtype, cspt_method method, void* stream,
  int32_t* out_point_geometry_id, int32_t* out_linestring_geometry_id, int32_t* out_segment_id,
  void* out_nearest_xy)
{
  return guarded([&] {
    t_last_refined = 0;
    check_dtype(dtype);
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown distance method");
    PlPairs const pr = pl_pairs(point_geometry_offsets, num_point_geometry_offsets, num_points,
                                linestring_geometry_offsets, num_linestring_geometry_offsets,
                                num_linestring_part_offsets);
    // point_linestring_nearest_points.cu:225-236
    CSPT_EXPECTS(pr.points == pr.linestrings,
                 "Mismatch number of (multi)points and (multi)linestrings.");
    if (pr.points == 0) return;
    CSPT_EXPECTS(out_segment_id && out_nearest_xy, "output pointers must not be null");
    Allocator alloc(nullptr, as_stream(stream));
    uint64_t refined = 0;
    pairwise_point_linestring(pr.points, point_geometry_offsets, num_point_geometry_offsets, x,
                              y, num_points, linestring_geometry_offsets,
                              num_linestring_geometry_offsets, linestring_part_offsets,
                              num_linestring_part_offsets, ls_x, ls_y, num_ls_vertices, dtype,
                              method, alloc, nullptr, out_point_geometry_id,
                              out_linestring_geometry_id, out_segment_id, out_nearest_xy,
                              &refined);
    t_last_refined = refined;
  });
}

}  // extern "C"
