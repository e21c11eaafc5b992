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
// Layout.  Instance i owns points [pt_begin_i, pt_end_i) of the concatenated
// x/y columns and polygons [poly_begin_i, poly_end_i) of the concatenated
// polygon column (whose ring and vertex offsets are global).  Outputs are
// concatenations of the per-instance outputs, with instance offsets:
//   * point_indices: instance i's sorted point order at [pt_begin_i,
//     pt_end_i), values local to the instance;
//   * quadtree: instance i's nodes at [node_offsets_i, node_offsets_{i+1}),
//     child and point offsets local to the instance;
//   * (polygon_index, point_index) rows of instance i at [row_offsets_i,
//     row_offsets_{i+1}), both local to the instance.
//
// Tree.  Points are sorted once by the composite key (instance << kb) |
// morton key, which keeps instances contiguous and each instance's points
// in its own stable Morton order.  The single-tree construction (quadtree.cu)
// carries over level by level with three changes: a sorted position starts a
// node at every level when it is the first point of its instance, a level-l
// node exists only for instances with max_depth > l, and node ends are
// clipped to the instance's last point.  Kept nodes are then laid out
// instance-major, level-major within the instance.
#include <algorithm>
#include <memory>
#include <vector>

#include "join_kernel.cuh"
#include "polygon_index.cuh"
#include "radix_sort.cuh"
#include "scan.cuh"

namespace cspt {

void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);

namespace {

constexpr int kLevels       = 16;
constexpr uint8_t kNoStart  = 0xFF;
constexpr unsigned kBlk     = 256;
constexpr unsigned kGridCap = 152u * 16u;

struct Inst {
  double minx, miny, maxx, maxy, scale;
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

#define GRID_STRIDE(i, n)                                                           \
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < (n); \
       i += static_cast<size_t>(gridDim.x) * blockDim.x)

// phase_1.cuh:73-85 per instance, tagged with the instance
__global__ void keys_kernel(double const* __restrict__ x, double const* __restrict__ y, size_t n,
                            uint32_t const* __restrict__ pt_begin, uint32_t ni,
                            Inst const* __restrict__ inst, int kb, uint64_t* __restrict__ keys)
{
  GRID_STRIDE(i, n)
  {
    uint32_t const k = find_instance(pt_begin, ni, static_cast<uint32_t>(i));
    Inst const& I    = inst[k];
    double const px = x[i], py = y[i];
    uint32_t key;
    if (px < I.minx || px > I.maxx || py < I.miny || py > I.maxy) {
      key = (1u << (2 * I.d)) - 1u;
    } else {
      uint16_t const cx = static_cast<uint16_t>((px - I.minx) / I.scale);
      uint16_t const cy = static_cast<uint16_t>((py - I.miny) / I.scale);
      key               = (spread16(cy) << 1) | spread16(cx);
    }
    keys[i] = (static_cast<uint64_t>(k) << kb) | key;
  }
}

__global__ void start_level_kernel(uint64_t const* __restrict__ sk, size_t n, int kb,
                                   Inst const* __restrict__ inst, uint8_t* __restrict__ lvl,
                                   uint8_t* __restrict__ lim)
{
  uint64_t const mask = (uint64_t{1} << kb) - 1u;
  GRID_STRIDE(i, n)
  {
    uint64_t const c = sk[i];
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

struct StartFlag {
  uint8_t const* lvl;
  uint8_t const* lim;
  int l;
  __device__ uint32_t operator()(size_t i) const
  {
    return (static_cast<int>(lvl[i]) <= l && l < static_cast<int>(lim[i])) ? 1u : 0u;
  }
};
struct RankStore {
  uint32_t* rank;
  uint32_t* starts;
  __device__ void operator()(size_t i, uint32_t e, uint32_t f) const
  {
    rank[i] = e;
    if (f) starts[e] = static_cast<uint32_t>(i);
  }
};

__device__ inline uint32_t node_end(uint32_t const* starts, size_t nl, size_t k, uint32_t iend)
{
  uint32_t const e = (k + 1 < nl) ? starts[k + 1] : iend;
  return e < iend ? e : iend;
}

// point counts and instances of one level's nodes
__global__ void count_kernel(uint32_t const* __restrict__ starts, size_t nl,
                             uint64_t const* __restrict__ sk, int kb,
                             Inst const* __restrict__ inst, uint32_t* __restrict__ count,
                             uint32_t* __restrict__ ninst)
{
  GRID_STRIDE(k, nl)
  {
    uint32_t const s = starts[k];
    uint32_t const i = static_cast<uint32_t>(sk[s] >> kb);
    count[k]         = node_end(starts, nl, k, inst[i].pt_end) - s;
    ninst[k]         = i;
  }
}

__global__ void child_count_kernel(uint32_t const* __restrict__ prev_starts, size_t nprev,
                                   uint32_t const* __restrict__ prev_inst,
                                   Inst const* __restrict__ inst,
                                   uint32_t const* __restrict__ rank_cur,
                                   uint32_t* __restrict__ child)
{
  GRID_STRIDE(p, nprev)
  {
    uint32_t const e = node_end(prev_starts, nprev, p, inst[prev_inst[p]].pt_end);
    child[p]         = rank_cur[e] - rank_cur[prev_starts[p]];
  }
}

// phase_2.cuh:206-236 with the instance's max_size
__global__ void keep_kernel(uint32_t const* __restrict__ starts, size_t nl,
                            uint32_t const* __restrict__ ninst, uint8_t const* __restrict__ lvl,
                            int prev_level, uint32_t const* __restrict__ rank_prev,
                            uint32_t const* __restrict__ count_prev,
                            Inst const* __restrict__ inst, uint8_t* __restrict__ keep)
{
  GRID_STRIDE(k, nl)
  {
    uint32_t const i      = starts[k];
    uint32_t const is_beg = static_cast<int>(lvl[i]) <= prev_level ? 1u : 0u;
    uint32_t const parent = rank_prev[i] + is_beg - 1u;
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

__global__ void compact_level_kernel(size_t nl, uint8_t const* __restrict__ kp,
                                     uint32_t const* __restrict__ ps,
                                     uint32_t const* __restrict__ starts,
                                     uint32_t const* __restrict__ cnt,
                                     uint32_t const* __restrict__ child,
                                     uint32_t const* __restrict__ ninst,
                                     uint64_t const* __restrict__ sk, int kb,
                                     Inst const* __restrict__ inst, int level,
                                     uint32_t* __restrict__ okey, uint32_t* __restrict__ ocount,
                                     uint32_t* __restrict__ ochild, uint32_t* __restrict__ ostart,
                                     uint32_t* __restrict__ oinst)
{
  uint64_t const mask = (uint64_t{1} << kb) - 1u;
  GRID_STRIDE(k, nl)
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

// first / one-past-last compacted index of each instance within a level
__global__ void level_span_kernel(uint32_t const* __restrict__ oinst, size_t m, int level,
                                  uint32_t* __restrict__ first, uint32_t* __restrict__ end)
{
  GRID_STRIDE(k, m)
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
  GRID_STRIDE(k, m)
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
  GRID_STRIDE(o, q)
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

__global__ void local_indices_kernel(uint32_t const* __restrict__ sidx,
                                     uint64_t const* __restrict__ sk, int kb,
                                     Inst const* __restrict__ inst, size_t n,
                                     uint32_t* __restrict__ out)
{
  GRID_STRIDE(i, n) { out[i] = sidx[i] - inst[sk[i] >> kb].pt_begin; }
}

// the tree a polygon's box walks: its instance's
struct InstanceTrees {
  uint32_t const* poly_begin;
  uint32_t ni;
  Inst const* inst;
  __device__ BoxTree<double> operator()(size_t b) const
  {
    Inst const& I = inst[find_instance(poly_begin, ni, static_cast<uint32_t>(b))];
    return BoxTree<double>{I.node_base, I.nq,     I.L0,    I.pt_begin,
                           I.minx,      I.miny,   I.scale, static_cast<int>(I.d)};
  }
};

// first pair of each instance: pairs are sorted by global point position
__global__ void pair_begin_kernel(uint32_t const* __restrict__ skey, size_t k,
                                  Inst const* __restrict__ inst, uint32_t ni,
                                  uint32_t* __restrict__ pair_begin)
{
  GRID_STRIDE(i, static_cast<size_t>(ni) + 1)
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

__global__ void row_offsets_kernel(uint32_t const* __restrict__ pair_begin,
                                   uint64_t const* __restrict__ pair_out, uint32_t ni,
                                   uint64_t* __restrict__ row_offsets)
{
  GRID_STRIDE(i, static_cast<size_t>(ni) + 1) { row_offsets[i] = pair_out[pair_begin[i]]; }
}

__global__ void localize_kernel(uint32_t* __restrict__ op, uint32_t* __restrict__ oq, size_t m,
                                uint32_t const* __restrict__ pt_begin, uint32_t ni,
                                Inst const* __restrict__ inst)
{
  GRID_STRIDE(j, m)
  {
    uint32_t const pos = oq[j];
    Inst const& I      = inst[find_instance(pt_begin, ni, pos)];
    oq[j]              = pos - I.pt_begin;
    op[j]              = op[j] - I.poly_begin;
  }
}

#undef GRID_STRIDE

}  // namespace

// ---------------------------------------------------------------------------
// the plan
// ---------------------------------------------------------------------------
class BatchedPip {
 public:
  BatchedPip(size_t ni, uint64_t const* h_pt_off, double const* x, double const* y,
             uint64_t const* h_poly_off, uint32_t const* po, size_t npo, uint32_t const* ro,
             size_t nro, double const* vx, double const* vy, size_t nv,
             cspt_instance_params const* params, cspt_method method, int block,
             cspt_allocator const* mr, cudaStream_t stream)
    : mr_copy_(mr ? *mr : cspt_allocator{}), alloc_(mr ? &mr_copy_ : nullptr, stream), ni_(ni)
  {
    plan(h_pt_off, x, y, h_poly_off, po, npo, ro, nro, vx, vy, nv, params, method, block);
  }
  ~BatchedPip()
  {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
  }

  void run(bool use_graph, cudaStream_t s)
  {
    if (!pip_) return;
    KernelTimer timer("batched_pip", s);
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
    o->num_points      = n_;
    o->num_polygons    = np_;
    o->num_nodes       = q_;
    o->num_pairs       = k_;
    o->num_rows        = m_;
    o->kernels_per_run = kernels_per_run_;
    o->polygon_index   = op_.data();
    o->point_index     = oq_.data();
    o->row_offsets     = row_off_.data();
    o->point_indices   = pidx_.data();
    o->tree = cspt_quadtree{key_.data(), level_.data(), internal_.data(), length_.data(),
                            offset_.data(), q_};
    o->node_offsets = node_off_.data();
  }

  uint64_t refined(cudaStream_t s) const
  {
    return pip_ ? read_back(pip_->refined(), s) : 0u;
  }

 private:
  void execute(cudaStream_t s)
  {
    pip_->execute(s, op_.data(), oq_.data(), m_);
    unsigned const g1 = grid_for(ni_ + 1, kBlk, kGridCap);
    row_offsets_kernel<<<g1, kBlk, 0, s>>>(pair_begin_.data(), pip_->pair_out_offsets(),
                                            static_cast<uint32_t>(ni_), row_off_.data());
    CSPT_CHECK_LAUNCH();
    if (m_) {
      localize_kernel<<<grid_for(m_, kBlk, kGridCap), kBlk, 0, s>>>(
        op_.data(), oq_.data(), m_, pt_begin_.data(), static_cast<uint32_t>(ni_), inst_.data());
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

  void plan(uint64_t const* h_pt_off, double const* x, double const* y,
            uint64_t const* h_poly_off, uint32_t const* po, size_t npo, uint32_t const* ro,
            size_t nro, double const* vx, double const* vy, size_t nv,
            cspt_instance_params const* params, cspt_method method, int block)
  {
    cudaStream_t const s = alloc_.stream();
    Allocator const& a   = alloc_;
    n_                   = h_pt_off[ni_];
    np_                  = h_poly_off[ni_];
    CSPT_EXPECTS(n_ < (size_t{1} << 32), "the batched form supports fewer than 2^32 points");
    CSPT_EXPECTS(np_ + 1 <= npo, "polygon offsets do not cover the instances' polygons");
    // host instance table (clamps of detail/point_quadtree.cuh:258-268)
    std::vector<Inst> hi(ni_);
    std::vector<uint32_t> h_ptb(ni_ + 1), h_pob(ni_ + 1);
    int dmax = 1;
    for (size_t i = 0; i < ni_; ++i) {
      cspt_instance_params const& p = params[i];
      CSPT_EXPECTS(h_pt_off[i] <= h_pt_off[i + 1] && h_poly_off[i] <= h_poly_off[i + 1],
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
      I.max_size        = static_cast<uint32_t>(p.max_size < 1 ? 1 : p.max_size);
      I.pt_begin        = static_cast<uint32_t>(h_pt_off[i]);
      I.pt_end          = static_cast<uint32_t>(h_pt_off[i + 1]);
      I.poly_begin      = static_cast<uint32_t>(h_poly_off[i]);
      I.poly_end        = static_cast<uint32_t>(h_poly_off[i + 1]);
      I.node_base = I.nq = I.L0 = 0;
      h_ptb[i]                  = I.pt_begin;
      h_pob[i]                  = I.poly_begin;
      dmax                      = std::max(dmax, p.max_depth);
    }
    h_ptb[ni_] = static_cast<uint32_t>(n_);
    h_pob[ni_] = static_cast<uint32_t>(np_);
    inst_      = Buffer<Inst>(a, ni_);
    pt_begin_  = Buffer<uint32_t>(a, ni_ + 1);
    poly_begin_ = Buffer<uint32_t>(a, ni_ + 1);
    CSPT_CUDA_TRY(cudaMemcpyAsync(inst_.data(), hi.data(), ni_ * sizeof(Inst),
                                  cudaMemcpyHostToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(pt_begin_.data(), h_ptb.data(), (ni_ + 1) * 4,
                                  cudaMemcpyHostToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(poly_begin_.data(), h_pob.data(), (ni_ + 1) * 4,
                                  cudaMemcpyHostToDevice, s));
    // the host arrays above must outlive the copies
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    uint32_t const ni = static_cast<uint32_t>(ni_);

    node_off_ = Buffer<uint64_t>(a, ni_ + 1);
    row_off_  = Buffer<uint64_t>(a, ni_ + 1);
    if (n_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(node_off_.data(), 0, (ni_ + 1) * 8, s));
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni_ + 1) * 8, s));
      return;
    }
    {
      KernelTimer timer("batched_tree", s);
      build_tree(x, y, dmax);
    }
    if (np_ == 0 || q_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni_ + 1) * 8, s));
      return;
    }

    // boxes of all polygons; every polygon must have vertices so that the
    // rows stay aligned with the polygons (empty geometries shift rows)
    bminx_ = Buffer<double>(a, np_);
    bminy_ = Buffer<double>(a, np_);
    bmaxx_ = Buffer<double>(a, np_);
    bmaxy_ = Buffer<double>(a, np_);
    polygon_bounding_boxes(po, np_ + 1, ro, nro, vx, vy, nv, CSPT_FLOAT64, 0.0, bminx_.data(),
                           bminy_.data(), bmaxx_.data(), bmaxy_.data(), a);
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
    bool const filtered = method == CSPT_METHOD_FILTERED;
    index_.reset(new PolygonIndex<double>(po, np_ + 1, ro, nro, vx, vy, nv, filtered, a));
    pip_.reset(new PipExec(pair_poly_.data(), pair_quad_.data(), k_, length_.data(),
                           goff_.data(), sidx_.data(), n_, x, y, index_->view(), filtered,
                           static_cast<unsigned>(block), a));
    // one evaluation sizes the outputs
    pip_->execute(s, nullptr, nullptr, 0);
    m_  = read_back(pip_->total(), s);
    op_ = Buffer<uint32_t>(a, m_);
    oq_ = Buffer<uint32_t>(a, m_);
  }

  void build_tree(double const* x, double const* y, int dmax)
  {
    Allocator const& a   = alloc_;
    cudaStream_t const s = a.stream();
    uint32_t const ni    = static_cast<uint32_t>(ni_);
    size_t const n       = n_;
    unsigned const grd   = grid_for(n, kBlk, kGridCap);
    int const kb         = dmax >= 2 ? 2 * dmax + 2 : 2 * dmax + 4;
    int ib               = 0;
    while ((uint64_t{1} << ib) < ni_) ++ib;

    Buffer<uint64_t> keys(a, n), keys_alt(a, n);
    Buffer<uint32_t> idx(a, n), idx_alt(a, n);
    keys_kernel<<<grd, kBlk, 0, s>>>(x, y, n, pt_begin_.data(), ni, inst_.data(), kb,
                                     keys.data());
    CSPT_CHECK_LAUNCH();
    bool const alt = radix_sort_pairs<uint64_t>(keys.data(), idx.data(), keys_alt.data(),
                                                idx_alt.data(), n, 0, kb + ib, true, a);
    Buffer<uint64_t>& sk = alt ? keys_alt : keys;
    sidx_                = std::move(alt ? idx_alt : idx);
    (alt ? keys : keys_alt).reset();
    (alt ? idx : idx_alt).reset();

    Buffer<uint8_t> lvl(a, n), lim(a, n);
    start_level_kernel<<<grd, kBlk, 0, s>>>(sk.data(), n, kb, inst_.data(), lvl.data(),
                                            lim.data());
    CSPT_CHECK_LAUNCH();
    pidx_ = Buffer<uint32_t>(a, n);
    local_indices_kernel<<<grd, kBlk, 0, s>>>(sidx_.data(), sk.data(), kb, inst_.data(), n,
                                              pidx_.data());
    CSPT_CHECK_LAUNCH();

    struct Level {
      Buffer<uint32_t> key, count, child, start, inst;
      size_t size = 0;
    };
    std::vector<Level> levels(dmax);
    Buffer<uint32_t> first(a, ni_ * kLevels), end(a, ni_ * kLevels);
    CSPT_CUDA_TRY(cudaMemsetAsync(first.data(), 0, ni_ * kLevels * 4, s));
    CSPT_CUDA_TRY(cudaMemsetAsync(end.data(), 0, ni_ * kLevels * 4, s));
    Buffer<uint32_t> total(a, 1);
    Buffer<uint32_t> rank_prev(a, n + 1), rank_cur(a, n + 1);
    Buffer<uint32_t> starts_prev, starts_cur, count_prev, count_cur, inst_prev, inst_cur;
    Buffer<uint8_t> keep_prev, keep_cur;
    size_t n_prev = 0;

    auto emit = [&](int lv, Buffer<uint32_t>& starts, Buffer<uint32_t>& counts,
                    Buffer<uint32_t>* childs, Buffer<uint32_t>& ninst, Buffer<uint8_t>* keep,
                    size_t nl) {
      Level& L          = levels[lv];
      uint8_t const* kp = keep ? keep->data() : nullptr;
      Buffer<uint32_t> pos(a, nl);
      scan_apply<uint32_t>(KeepIn{kp}, PosOut{pos.data()}, nl, total.data(), a);
      size_t const m = read_back(total.data(), s);
      L.size         = m;
      L.key          = Buffer<uint32_t>(a, m);
      L.count        = Buffer<uint32_t>(a, m);
      L.child        = Buffer<uint32_t>(a, m);
      L.start        = Buffer<uint32_t>(a, m);
      L.inst         = Buffer<uint32_t>(a, m);
      if (nl) {
        compact_level_kernel<<<grid_for(nl, kBlk, kGridCap), kBlk, 0, s>>>(
          nl, kp, pos.data(), starts.data(), counts.data(), childs ? childs->data() : nullptr,
          ninst.data(), sk.data(), kb, inst_.data(), lv, L.key.data(), L.count.data(),
          L.child.data(), L.start.data(), L.inst.data());
        CSPT_CHECK_LAUNCH();
      }
      if (m) {
        level_span_kernel<<<grid_for(m, kBlk, kGridCap), kBlk, 0, s>>>(L.inst.data(), m, lv,
                                                                       first.data(), end.data());
        CSPT_CHECK_LAUNCH();
      }
    };

    for (int l = 0; l < dmax; ++l) {
      starts_cur = Buffer<uint32_t>(a, n);
      scan_apply<uint32_t>(StartFlag{lvl.data(), lim.data(), l},
                           RankStore{rank_cur.data(), starts_cur.data()}, n,
                           rank_cur.data() + n, a);
      size_t const nl = read_back(rank_cur.data() + n, s);
      count_cur       = Buffer<uint32_t>(a, nl);
      inst_cur        = Buffer<uint32_t>(a, nl);
      keep_cur        = Buffer<uint8_t>(a, nl);
      unsigned const g = grid_for(nl, kBlk, kGridCap);
      if (nl) {
        count_kernel<<<g, kBlk, 0, s>>>(starts_cur.data(), nl, sk.data(), kb, inst_.data(),
                                        count_cur.data(), inst_cur.data());
        CSPT_CHECK_LAUNCH();
      }
      if (l == 0) {
        if (nl) CSPT_CUDA_TRY(cudaMemsetAsync(keep_cur.data(), 1, nl, s));
      } else {
        if (nl) {
          keep_kernel<<<g, kBlk, 0, s>>>(starts_cur.data(), nl, inst_cur.data(), lvl.data(),
                                         l - 1, rank_prev.data(), count_prev.data(),
                                         inst_.data(), keep_cur.data());
          CSPT_CHECK_LAUNCH();
        }
        Buffer<uint32_t> child_prev(a, n_prev);
        if (n_prev) {
          child_count_kernel<<<grid_for(n_prev, kBlk, kGridCap), kBlk, 0, s>>>(
            starts_prev.data(), n_prev, inst_prev.data(), inst_.data(), rank_cur.data(),
            child_prev.data());
          CSPT_CHECK_LAUNCH();
        }
        emit(l - 1, starts_prev, count_prev, &child_prev, inst_prev,
             l - 1 == 0 ? nullptr : &keep_prev, n_prev);
      }
      std::swap(rank_prev, rank_cur);
      starts_prev = std::move(starts_cur);
      count_prev  = std::move(count_cur);
      inst_prev   = std::move(inst_cur);
      keep_prev   = std::move(keep_cur);
      n_prev      = nl;
    }
    emit(dmax - 1, starts_prev, count_prev, nullptr, inst_prev, dmax - 1 == 0 ? nullptr : &keep_prev,
         n_prev);
    starts_prev.reset();
    count_prev.reset();
    inst_prev.reset();
    keep_prev.reset();
    rank_prev.reset();
    rank_cur.reset();
    lvl.reset();
    lim.reset();
    sk.reset();

    Buffer<long long> shift(a, ni_ * kLevels);
    Buffer<int> err(a, 1);
    CSPT_CUDA_TRY(cudaMemsetAsync(err.data(), 0, sizeof(int), s));
    layout_kernel<<<1, 1024, 0, s>>>(first.data(), end.data(), ni, inst_.data(), shift.data(),
                                     node_off_.data(), err.data());
    CSPT_CHECK_LAUNCH();
    size_t q = 0;
    for (auto& L : levels) q += L.size;
    CSPT_EXPECTS(read_back(err.data(), s) == 0,
                 "an instance's quadtree has too many nodes for the batched form");
    q_        = q;
    key_      = Buffer<uint32_t>(a, q);
    length_   = Buffer<uint32_t>(a, q);
    offset_   = Buffer<uint32_t>(a, q);
    goff_     = Buffer<uint32_t>(a, q);
    level_    = Buffer<uint8_t>(a, q);
    internal_ = Buffer<uint8_t>(a, q);
    if (q == 0) return;
    Buffer<uint32_t> ichild(a, q), node_inst(a, q);
    for (int l = 0; l < dmax; ++l) {
      Level& L = levels[l];
      if (L.size) {
        assemble_kernel<<<grid_for(L.size, kBlk, kGridCap), kBlk, 0, s>>>(
          L.key.data(), L.count.data(), L.child.data(), L.start.data(), L.inst.data(), L.size,
          l, inst_.data(), shift.data(), key_.data(), level_.data(), internal_.data(),
          length_.data(), offset_.data(), ichild.data(), node_inst.data());
        CSPT_CHECK_LAUNCH();
      }
      L = Level{};
    }
    exclusive_scan<uint32_t>(ichild.data(), ichild.data(), q, static_cast<uint32_t*>(nullptr), a);
    offsets_kernel<<<grid_for(q, kBlk, kGridCap), kBlk, 0, s>>>(
      internal_.data(), ichild.data(), node_inst.data(), inst_.data(), q, offset_.data(),
      goff_.data());
    CSPT_CHECK_LAUNCH();
  }

  void join(uint32_t ni)
  {
    Allocator const& a   = alloc_;
    cudaStream_t const s = a.stream();
    size_t const nb      = np_;
    TreeView const tv{key_.data(), level_.data(), internal_.data(), length_.data(),
                      offset_.data(), q_};
    InstanceTrees const trees{poly_begin_.data(), ni, inst_.data()};
    Buffer<uint32_t> counts(a, nb + 1);
    Buffer<uint32_t> status(a, 2);
    CSPT_CUDA_TRY(cudaMemsetAsync(status.data(), 0, 2 * sizeof(uint32_t), s));
    int* err           = reinterpret_cast<int*>(status.data() + 1);
    unsigned const blk = kJoinWarps * 32;
    unsigned const grd = grid_for(nb * 32, blk, kGridCap);
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
    gather_pairs_kernel<<<grid_for(k_, kBlk, kGridCap), kBlk, 0, s>>>(
      alt ? perm_alt.data() : perm.data(), node.data(), box.data(), k_, pair_poly_.data(),
      pair_quad_.data());
    CSPT_CHECK_LAUNCH();
    pair_begin_kernel<<<grid_for(ni_ + 1, kBlk, kGridCap), kBlk, 0, s>>>(
      alt ? key_alt.data() : key.data(), k_, inst_.data(), ni, pair_begin_.data());
    CSPT_CHECK_LAUNCH();
  }

  cspt_allocator mr_copy_;
  Allocator alloc_;
  size_t ni_;
  size_t n_ = 0, np_ = 0, q_ = 0, k_ = 0, m_ = 0;
  Buffer<Inst> inst_;
  Buffer<uint32_t> pt_begin_, poly_begin_;
  Buffer<uint32_t> sidx_, pidx_;
  Buffer<uint32_t> key_, length_, offset_, goff_;
  Buffer<uint8_t> level_, internal_;
  Buffer<uint64_t> node_off_, row_off_;
  Buffer<double> bminx_, bminy_, bmaxx_, bmaxy_;
  Buffer<uint32_t> pair_poly_, pair_quad_, pair_begin_;
  std::unique_ptr<PolygonIndex<double>> index_;
  std::unique_ptr<PipExec> pip_;
  Buffer<uint32_t> op_, oq_;
  cudaStream_t capture_stream_ = nullptr;
  cudaGraph_t graph_           = nullptr;
  cudaGraphExec_t exec_        = nullptr;
  uint64_t kernels_per_run_    = 0;
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
                                  cspt_dtype dtype, cspt_method method, int block_threads,
                                  const cspt_allocator* mr, void* stream,
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
      static_cast<double const*>(poly_y), num_poly_vertices, params, method, block_threads, mr,
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
