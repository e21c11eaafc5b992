// Batched point-in-polygon join: many independent instances (each its own
// points, polygons and quadtree parameters) planned together and evaluated by
// one pass of the same kernels, with the evaluation captured into a CUDA
// graph.  Every instance's outputs equal what the single-instance calls
//   quadtree_on_points -> polygon_bounding_boxes ->
//   join_quadtree_and_bounding_boxes -> quadtree_point_in_polygon
// return for that instance alone (the reference has no batched form; its
// single-instance semantics are cpp/include/cuspatial/detail/
// point_quadtree.cuh:237-272, quadtree_bbox_filtering.cuh:35-188 and
// quadtree_point_in_polygon.cuh:104-235).
//
// Instance i owns points [pt_begin_i, pt_end_i) of the concatenated x/y
// columns and polygons [poly_begin_i, poly_end_i) of the concatenated
// polygon column (whose ring and vertex offsets are global).  The trees are
// one Forest (forest.cuh); each polygon's box walks its instance's tree with
// the shared join kernel; the pairs of all instances, sorted by global point
// position, are instance-major and in each instance's reference order.  Rows
// of instance i land at [row_offsets_i, row_offsets_{i+1}) with
// instance-local polygon and point indices.
#include <memory>
#include <vector>

#include "forest.cuh"
#include "polygon_index.cuh"

namespace cspt {

void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);

namespace {

// the instance of polygon b
struct PolygonInstance {
  uint32_t const* poly_begin;
  uint32_t ni;
  __device__ uint32_t operator()(size_t b) const
  {
    return find_instance(poly_begin, ni, static_cast<uint32_t>(b));
  }
};

// first pair of each instance: pairs are sorted by global point position
__global__ void pair_begin_kernel(uint32_t const* __restrict__ skey, size_t k,
                                  Inst const* __restrict__ inst, uint32_t ni,
                                  uint32_t* __restrict__ pair_begin)
{
  CSPT_GRID_STRIDE(i, static_cast<size_t>(ni) + 1)
  {
    if (i == ni) {
      pair_begin[i] = static_cast<uint32_t>(k);
      continue;
    }
    uint32_t const v = inst[i].pt_begin;
    size_t lo = 0, hi = k;
    while (lo < hi) {
      size_t const mid = (lo + hi) >> 1;
      if (skey[mid] < v)
        lo = mid + 1;
      else
        hi = mid;
    }
    pair_begin[i] = static_cast<uint32_t>(lo);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// the plan
// ---------------------------------------------------------------------------
class BatchedPip {
 public:
  BatchedPip(size_t ni, uint64_t const* h_pt_off, double const* x, double const* y,
             uint64_t const* h_poly_off, uint32_t const* po, size_t npo, uint32_t const* ro,
             size_t nro, double const* vx, double const* vy, size_t nv,
             cspt_instance_params const* params, cspt_method method, bool ordered, int block,
             cspt_allocator const* mr, cudaStream_t stream)
    : mr_copy_(mr ? *mr : cspt_allocator{}), alloc_(mr ? &mr_copy_ : nullptr, stream),
      palloc_(mr ? &mr_copy_ : nullptr, nullptr), ni_(ni), f_(alloc_)
  {
    try {
      plan(h_pt_off, x, y, h_poly_off, po, npo, ro, nro, vx, vy, nv, params, method, ordered,
           block);
    } catch (...) {
      release();
      throw;
    }
  }
  ~BatchedPip() { release(); }

  void run(bool use_graph, cudaStream_t s)
  {
    if (!pip_) return;
    KernelTimer timer("batched_pip", s);
    if (evaluated_) {
      // the plan's sizing evaluation already holds this batch's bits and
      // row offsets: the first run only writes the rows
      evaluated_ = false;
      finish(s);
      return;
    }
    if (use_graph) {
      if (!exec_) capture();
      CSPT_CUDA_TRY(cudaGraphLaunch(exec_, s));
      count_launches(kernels_per_run_);
    } else {
      execute(s);
    }
  }

  void info(cspt_batched_pip_info* o) const
  {
    o->num_instances   = ni_;
    o->num_points      = f_.n_;
    o->num_polygons    = np_;
    o->num_nodes       = f_.q_;
    o->num_pairs       = k_;
    o->num_rows        = m_;
    o->kernels_per_run = kernels_per_run_;
    o->polygon_index   = op_.data();
    o->point_index     = oq_.data();
    o->row_offsets     = row_off_.data();
    o->point_indices   = f_.pidx_.data();
    o->tree            = f_.tree();
    o->node_offsets    = f_.node_off_.data();
  }

  uint64_t refined(cudaStream_t s) const
  {
    return pip_ ? read_back(pip_->refined(), s) : 0u;
  }

 private:
  void execute(cudaStream_t s)
  {
    pip_->evaluate(s);
    finish(s);
  }

  // rows, per-instance row offsets and instance-local indices from the
  // evaluated bits
  void finish(cudaStream_t s)
  {
    pip_->expand(s, op_.data(), oq_.data(), m_);
    unsigned const g1 = grid_for(ni_ + 1, kBlk, grid_cap());
    row_offsets_kernel<<<g1, kBlk, 0, s>>>(pair_begin_.data(), pip_->pair_out_offsets(),
                                            static_cast<uint32_t>(ni_), row_off_.data());
    CSPT_CHECK_LAUNCH();
    if (m_) {
      localize_kernel<<<grid_for(m_, kBlk, grid_cap()), kBlk, 0, s>>>(
        op_.data(), oq_.data(), m_, f_.pt_begin_.data(), f_.tile_inst_.data(), f_.inst_.data(),
        true);
      CSPT_CHECK_LAUNCH();
    }
  }

  // Records execute() once into a graph on a private stream (capture only;
  // nothing runs there) and instantiates it.
  void capture()
  {
    if (!capture_stream_)
      CSPT_CUDA_TRY(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking));
    uint64_t const before = cspt_launch_count();
    CSPT_CUDA_TRY(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal));
    try {
      execute(capture_stream_);
    } catch (...) {
      cudaGraph_t g = nullptr;
      (void)cudaStreamEndCapture(capture_stream_, &g);
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      throw;
    }
    CSPT_CUDA_TRY(cudaStreamEndCapture(capture_stream_, &graph_));
    kernels_per_run_ = cspt_launch_count() - before;
    uncount_launches(kernels_per_run_);  // recorded, not run
    CSPT_CUDA_TRY(cudaGraphInstantiate(&exec_, graph_, 0));
  }

  // Frees the polygon-side buffers on their stream once the plan's stream
  // has caught up, then the graph and its stream.
  void release()
  {
    if (poly_stream_) {
      StreamJoin after(poly_stream_, alloc_.stream());
      after.join();
    }
    pip_.reset();
    index_.reset();
    bminx_.reset();
    bminy_.reset();
    bmaxx_.reset();
    bmaxy_.reset();
    poly_stream_ = nullptr;
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
    exec_           = nullptr;
    graph_          = nullptr;
    capture_stream_ = nullptr;
  }

  void plan(uint64_t const* h_pt_off, double const* x, double const* y,
            uint64_t const* h_poly_off, uint32_t const* po, size_t npo, uint32_t const* ro,
            size_t nro, double const* vx, double const* vy, size_t nv,
            cspt_instance_params const* params, cspt_method method, bool ordered, int block)
  {
    cudaStream_t const s = alloc_.stream();
    Allocator const& a   = alloc_;
    np_                  = h_poly_off[ni_];
    CSPT_EXPECTS(np_ + 1 <= npo, "polygon offsets do not cover the instances' polygons");
    f_.setup(ni_, h_pt_off, params, h_poly_off);
    uint32_t const ni = static_cast<uint32_t>(ni_);
    row_off_          = Buffer<uint64_t>(a, ni_ + 1);
    bool const filtered = method == CSPT_METHOD_FILTERED;
    // the ordered index's windows serve small blocks; the one-shot index's
    // quadrant fast path keeps per-warp lists sized for blocks of 256
    bool const order_slabs = filtered && ordered;

    // The boxes and the polygon index need only the polygons: they are built
    // on a private stream beside the forest build (which is bound by memory
    // and short launches; the index by the float64 pipe), from memory
    // ordered on that stream, and the plan's stream waits for them before
    // the join.  Every polygon must have vertices so that the rows stay
    // aligned with the polygons (empty geometries shift rows).
    if (np_ > 0) {
      poly_stream_ = library_stream();
      palloc_      = Allocator(alloc_.resource(), poly_stream_);
      stream_wait(poly_stream_, s);  // the polygon columns were written on s
      Allocator const& pa = palloc_;
      bminx_              = Buffer<double>(pa, np_);
      bminy_              = Buffer<double>(pa, np_);
      bmaxx_              = Buffer<double>(pa, np_);
      bmaxy_              = Buffer<double>(pa, np_);
      polygon_bounding_boxes(po, np_ + 1, ro, nro, vx, vy, nv, CSPT_FLOAT64, 0.0, bminx_.data(),
                             bminy_.data(), bmaxx_.data(), bmaxy_.data(), pa);
      index_.reset(new PolygonIndex<double>(po, np_ + 1, ro, nro, vx, vy, nv, filtered, pa,
                                            order_slabs));
    }
    {
      KernelTimer timer("batched_tree", s);
      f_.build(x, y);
    }
    if (poly_stream_) stream_wait(s, poly_stream_);
    if (f_.n_ == 0 || np_ == 0 || f_.q_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni_ + 1) * 8, s));
      return;
    }
    double const last = read_back(bminx_.data() + np_ - 1, s);
    CSPT_EXPECTS(!(last != last),
                 "the batched form requires every polygon to have at least one vertex");
    {
      KernelTimer timer("batched_join", s);
      join(ni);
    }
    if (k_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni_ + 1) * 8, s));
      return;
    }
    unsigned const pair_block = order_slabs || !filtered ? static_cast<unsigned>(block) : 256u;
    pip_.reset(new PipExec(pair_poly_.data(), pair_quad_.data(), k_, f_.length_.data(),
                           f_.goff_.data(), f_.sidx_.data(), f_.n_, x, y, index_->view(),
                           filtered, pair_block, a));
    // one evaluation sizes the outputs
    pip_->evaluate(s);
    m_  = read_back(pip_->total(), s);
    op_ = Buffer<uint32_t>(a, m_);
    oq_ = Buffer<uint32_t>(a, m_);
    evaluated_ = true;
  }

  void join(uint32_t ni)
  {
    Allocator const& a   = alloc_;
    cudaStream_t const s = a.stream();
    size_t const nb      = np_;
    TreeView const tv = f_.view();
    ForestTrees<PolygonInstance> const trees{PolygonInstance{f_.poly_begin_.data(), ni},
                                             f_.inst_.data()};
    Buffer<uint32_t> counts(a, nb + 1);
    Buffer<uint32_t> status(a, 2);
    CSPT_CUDA_TRY(cudaMemsetAsync(status.data(), 0, 2 * sizeof(uint32_t), s));
    int* err           = reinterpret_cast<int*>(status.data() + 1);
    unsigned const blk = kJoinWarps * 32;
    unsigned const grd = grid_for(nb * 32, blk, grid_cap());
    join_warp_kernel<double, false><<<grd, blk, 0, s>>>(
      tv, trees, bminx_.data(), bminy_.data(), bmaxx_.data(), bmaxy_.data(), nb, counts.data(),
      status.data(), nullptr, nullptr, nullptr, nullptr, err);
    CSPT_CHECK_LAUNCH();
    exclusive_scan<uint32_t>(counts.data(), counts.data(), nb, counts.data() + nb, a);
    uint32_t host[3];
    CSPT_CUDA_TRY(
      cudaMemcpyAsync(host, counts.data() + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(
      cudaMemcpyAsync(host + 1, status.data(), 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    CSPT_EXPECTS(host[2] == 0, "batched quadtree is malformed");
    k_ = host[0];
    pair_begin_ = Buffer<uint32_t>(a, ni_ + 1);
    if (k_ == 0) return;
    int key_bits = 1;
    while (key_bits < 32 && (host[1] >> key_bits) != 0) ++key_bits;
    Buffer<uint32_t> key(a, k_), key_alt(a, k_), node(a, k_), box(a, k_), perm(a, k_),
      perm_alt(a, k_);
    join_warp_kernel<double, true><<<grd, blk, 0, s>>>(
      tv, trees, bminx_.data(), bminy_.data(), bmaxx_.data(), bmaxy_.data(), nb, nullptr,
      nullptr, counts.data(), key.data(), node.data(), box.data(), err);
    CSPT_CHECK_LAUNCH();
    bool const alt = radix_sort_pairs<uint32_t>(key.data(), perm.data(), key_alt.data(),
                                                perm_alt.data(), k_, 0, key_bits, true, a);
    pair_poly_ = Buffer<uint32_t>(a, k_);
    pair_quad_ = Buffer<uint32_t>(a, k_);
    gather_pairs_kernel<<<grid_for(k_, kBlk, grid_cap()), kBlk, 0, s>>>(
      alt ? perm_alt.data() : perm.data(), node.data(), box.data(), k_, pair_poly_.data(),
      pair_quad_.data());
    CSPT_CHECK_LAUNCH();
    pair_begin_kernel<<<grid_for(ni_ + 1, kBlk, grid_cap()), kBlk, 0, s>>>(
      alt ? key_alt.data() : key.data(), k_, f_.inst_.data(), ni, pair_begin_.data());
    CSPT_CHECK_LAUNCH();
  }

  cspt_allocator mr_copy_;
  Allocator alloc_;
  Allocator palloc_;  // the polygon side's memory, ordered on poly_stream_
  cudaStream_t poly_stream_ = nullptr;  // library_stream(), not owned
  size_t ni_;
  Forest f_;
  size_t np_ = 0, k_ = 0, m_ = 0;
  Buffer<uint64_t> row_off_;
  Buffer<double> bminx_, bminy_, bmaxx_, bmaxy_;
  Buffer<uint32_t> pair_poly_, pair_quad_, pair_begin_;
  std::unique_ptr<PolygonIndex<double>> index_;
  std::unique_ptr<PipExec> pip_;
  Buffer<uint32_t> op_, oq_;
  cudaStream_t capture_stream_ = nullptr;
  cudaGraph_t graph_           = nullptr;
  cudaGraphExec_t exec_        = nullptr;
  uint64_t kernels_per_run_    = 0;
  bool evaluated_              = false;  // no run since the plan's evaluation
};

}  // namespace cspt

using namespace cspt;

extern "C" {

cspt_status cspt_batched_pip_plan(size_t num_instances, const uint64_t* point_offsets,
                                  const void* x, const void* y, const uint64_t* polygon_offsets,
                                  const uint32_t* poly_offsets, size_t num_poly_offsets,
                                  const uint32_t* ring_offsets, size_t num_ring_offsets,
                                  const void* poly_x, const void* poly_y,
                                  size_t num_poly_vertices, const cspt_instance_params* params,
                                  cspt_dtype dtype, cspt_method method, int ordered_index,
                                  int block_threads, const cspt_allocator* mr, void* stream,
                                  cspt_batched_pip** out_plan)
{
  return guarded([&] {
    CSPT_EXPECTS(out_plan, "output pointers must not be null");
    *out_plan = nullptr;
    if (dtype != CSPT_FLOAT32 && dtype != CSPT_FLOAT64)
      throw Error{CSPT_UNSUPPORTED, "Only floating-point types are supported"};
    if (dtype != CSPT_FLOAT64)
      throw Error{CSPT_UNSUPPORTED, "the batched form supports float64 coordinates"};
    CSPT_EXPECTS(num_instances > 0 && num_instances < (size_t{1} << 20),
                 "the batched form takes between 1 and 2^20 - 1 instances");
    CSPT_EXPECTS(point_offsets && polygon_offsets && params,
                 "instance offsets and parameters must not be null");
    CSPT_EXPECTS(method == CSPT_METHOD_EXACT || method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    CSPT_EXPECTS(block_threads >= 32 && block_threads <= 256 && block_threads % 32 == 0,
                 "block_threads must be a multiple of 32 in [32, 256]");
    CSPT_EXPECTS(point_offsets[0] == 0 && polygon_offsets[0] == 0,
                 "instance offsets must start at 0");
    *out_plan = reinterpret_cast<cspt_batched_pip*>(new BatchedPip(
      num_instances, point_offsets, static_cast<double const*>(x),
      static_cast<double const*>(y), polygon_offsets, poly_offsets, num_poly_offsets,
      ring_offsets, num_ring_offsets, static_cast<double const*>(poly_x),
      static_cast<double const*>(poly_y), num_poly_vertices, params, method, ordered_index != 0,
      block_threads, mr,
      static_cast<cudaStream_t>(stream)));
  });
}

cspt_status cspt_batched_pip_run(cspt_batched_pip* plan, int use_graph, void* stream)
{
  return guarded([&] {
    CSPT_EXPECTS(plan, "plan must not be null");
    reinterpret_cast<BatchedPip*>(plan)->run(use_graph != 0, static_cast<cudaStream_t>(stream));
  });
}

cspt_status cspt_batched_pip_get_info(const cspt_batched_pip* plan, cspt_batched_pip_info* out)
{
  return guarded([&] {
    CSPT_EXPECTS(plan && out, "plan and output must not be null");
    reinterpret_cast<BatchedPip const*>(plan)->info(out);
  });
}

cspt_status cspt_batched_pip_refined_count(const cspt_batched_pip* plan, void* stream,
                                           uint64_t* out)
{
  return guarded([&] {
    CSPT_EXPECTS(plan && out, "plan and output must not be null");
    *out = reinterpret_cast<BatchedPip const*>(plan)->refined(static_cast<cudaStream_t>(stream));
  });
}

void cspt_batched_pip_free(cspt_batched_pip* plan)
{
  delete reinterpret_cast<BatchedPip*>(plan);
}

}  // extern "C"
