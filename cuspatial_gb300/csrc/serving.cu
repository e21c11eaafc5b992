// Serving form: a device-resident polygon set answering point-in-polygon
// requests of any size, batched as they arrive.
//
// A request is a set of points with its own quadtree parameters; its answer
// is exactly what the single-instance calls return for it against the whole
// polygon set:
//   quadtree_on_points(points, params) -> polygon_bounding_boxes(set) ->
//   join_quadtree_and_bounding_boxes -> quadtree_point_in_polygon
// (reference: cpp/include/cuspatial/detail/point_quadtree.cuh:237-272,
// quadtree_bbox_filtering.cuh:35-188, quadtree_point_in_polygon.cuh:104-235).
//
// Join from the leaf side.  The reference's traversal emits a (box, leaf)
// pair exactly when the box meets the leaf's extent: child extents are
// v_min + k * scale * 2^s computed with one rounding, and a parent's corners
// coincide bit for bit with its outer children's, so a box meeting a leaf
// meets every ancestor.  The resident set keeps its polygon boxes in a
// uniform cell grid; every (leaf, covered cell) is one work item that keeps
// a polygon of the cell when the reference's closed-interval overlap test
// holds, counting it only in the first cell (in both axes) that the leaf's
// and the box's cell ranges share.  The cell of a coordinate is floor((v - v0) / w) clamped to
// the grid, a monotone function of v, so any common point of box and extent
// lies in a cell of both ranges and every pair is found exactly once.  Pairs
// are then sorted by (leaf first position, polygon), the reference's order.
//
// Serving.  Requests are queued on submit; worker threads (one CUDA stream
// each) take batches off the queue as device memory and workers free up,
// admitting requests in arrival order while the estimated working memory of
// all batches in flight stays within the budget.  All device memory of a
// batch comes from a byte-budget allocator; a batch that still runs out is
// split and its requests retried one by one.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "forest.cuh"
#include "polygon_index.cuh"

namespace cspt {

void polygon_bounding_boxes(uint32_t const* poly_offsets, size_t npo,
                            uint32_t const* ring_offsets, size_t nro, void const* x,
                            void const* y, size_t nv, cspt_dtype dtype, double r, void* ominx,
                            void* ominy, void* omaxx, void* omaxy, Allocator const& alloc);

namespace {

constexpr int kGridMax = 4096;

struct GridView {
  double x0, y0, cw, ch;
  int gx, gy;
  uint32_t const* cell_start;  // gx * gy + 1
  uint32_t const* cell_poly;
  int2 const* poly_cell;       // first cell (x, y) of each polygon's box
  double const *bminx, *bminy, *bmaxx, *bmaxy;
};

// monotone in v: clamp(floor((v - v0) / w), 0, g - 1)
__device__ inline int cell_of(double v, double v0, double w, int g)
{
  double const f = floor((v - v0) / w);
  if (!(f > 0.0)) return 0;
  if (f >= static_cast<double>(g - 1)) return g - 1;
  return static_cast<int>(f);
}

__global__ void __launch_bounds__(1024)
  domain_kernel(double const* __restrict__ bminx, double const* __restrict__ bminy,
                double const* __restrict__ bmaxx, double const* __restrict__ bmaxy, size_t np,
                double* __restrict__ out)
{
  double a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
  for (size_t i = threadIdx.x; i < np; i += blockDim.x) {
    a = fmin(a, bminx[i]);
    b = fmin(b, bminy[i]);
    c = fmax(c, bmaxx[i]);
    d = fmax(d, bmaxy[i]);
  }
  __shared__ double s[4][32];
  for (int off = 16; off > 0; off >>= 1) {
    a = fmin(a, __shfl_xor_sync(0xFFFFFFFFu, a, off));
    b = fmin(b, __shfl_xor_sync(0xFFFFFFFFu, b, off));
    c = fmax(c, __shfl_xor_sync(0xFFFFFFFFu, c, off));
    d = fmax(d, __shfl_xor_sync(0xFFFFFFFFu, d, off));
  }
  int const w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s[0][w] = a;
    s[1][w] = b;
    s[2][w] = c;
    s[3][w] = d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int const nw = (blockDim.x + 31) >> 5;
    for (int k = 1; k < nw; ++k) {
      s[0][0] = fmin(s[0][0], s[0][k]);
      s[1][0] = fmin(s[1][0], s[1][k]);
      s[2][0] = fmax(s[2][0], s[2][k]);
      s[3][0] = fmax(s[3][0], s[3][k]);
    }
    for (int k = 0; k < 4; ++k) out[k] = s[k][0];
  }
}

__global__ void grid_count_kernel(GridView g, size_t np, uint32_t* __restrict__ counts,
                                  int2* __restrict__ poly_cell)
{
  CSPT_GRID_STRIDE(p, np)
  {
    int const cx0 = cell_of(g.bminx[p], g.x0, g.cw, g.gx);
    int const cx1 = cell_of(g.bmaxx[p], g.x0, g.cw, g.gx);
    int const cy0 = cell_of(g.bminy[p], g.y0, g.ch, g.gy);
    int const cy1 = cell_of(g.bmaxy[p], g.y0, g.ch, g.gy);
    poly_cell[p]  = make_int2(cx0, cy0);
    for (int cy = cy0; cy <= cy1; ++cy)
      for (int cx = cx0; cx <= cx1; ++cx) atomicAdd(&counts[cy * g.gx + cx], 1u);
  }
}

__global__ void grid_fill_kernel(GridView g, size_t np, uint32_t* __restrict__ cursor,
                                 uint32_t* __restrict__ cell_poly)
{
  CSPT_GRID_STRIDE(p, np)
  {
    int const cx0 = cell_of(g.bminx[p], g.x0, g.cw, g.gx);
    int const cx1 = cell_of(g.bmaxx[p], g.x0, g.cw, g.gx);
    int const cy0 = cell_of(g.bminy[p], g.y0, g.ch, g.gy);
    int const cy1 = cell_of(g.bmaxy[p], g.y0, g.ch, g.gy);
    for (int cy = cy0; cy <= cy1; ++cy)
      for (int cx = cx0; cx <= cx1; ++cx) {
        int const c                           = cy * g.gx + cx;
        cell_poly[g.cell_start[c] + atomicAdd(&cursor[c], 1u)] = static_cast<uint32_t>(p);
      }
  }
}

// instance of a node: node_off has ni + 1 entries
__device__ inline uint32_t node_instance(uint64_t const* __restrict__ node_off, uint32_t ni,
                                         uint64_t g)
{
  uint32_t lo = 0, hi = ni;
  while (hi - lo > 1) {
    uint32_t const mid = (lo + hi) >> 1;
    if (node_off[mid] <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The cells a leaf's extent covers, one work item per (leaf, cell), so a
// large leaf (a sparse request's leaves can cover thousands of cells) is
// spread over the whole GPU.
struct LeafCells {
  double x0, y0, x1, y1;  // leaf extent (intersection.cuh:104-128)
  int cx0, cy0, ncx;
  uint32_t ncells;
};

__global__ void leaf_cells_kernel(TreeView t, uint64_t const* __restrict__ node_off, uint32_t ni,
                                  Inst const* __restrict__ inst, GridView g,
                                  LeafCells* __restrict__ lc, uint32_t* __restrict__ ncells)
{
  CSPT_GRID_STRIDE(n, t.nq)
  {
    LeafCells c{0.0, 0.0, -1.0, -1.0, 0, 0, 0, 0u};
    if (!t.internal[n]) {
      Inst const& I      = inst[node_instance(node_off, ni, n)];
      uint32_t const key = t.key[n];
      int const sh       = static_cast<int>(I.d) - 1 - static_cast<int>(t.level[n]);
      if (sh >= 0) {
        double const kx = static_cast<double>(gather16(key));
        double const ky = static_cast<double>(gather16(key >> 1));
        double const ls = I.scale * static_cast<double>(1 << sh);
        c.x0            = fma_rn(kx, ls, I.minx);
        c.y0            = fma_rn(ky, ls, I.miny);
        c.x1            = fma_rn(kx + 1.0, ls, I.minx);
        c.y1            = fma_rn(ky + 1.0, ls, I.miny);
        c.cx0           = cell_of(c.x0, g.x0, g.cw, g.gx);
        c.cy0           = cell_of(c.y0, g.y0, g.ch, g.gy);
        c.ncx           = cell_of(c.x1, g.x0, g.cw, g.gx) - c.cx0 + 1;
        c.ncells =
          static_cast<uint32_t>(c.ncx * (cell_of(c.y1, g.y0, g.ch, g.gy) - c.cy0 + 1));
      }
    }
    lc[n]     = c;
    ncells[n] = c.ncells;
  }
}

// One thread per (leaf, cell): the polygons of the cell whose box meets the
// leaf's extent, counted only in the first cell both cell ranges share.
template <bool Write>
__global__ void leaf_cell_join_kernel(LeafCells const* __restrict__ lc,
                                      uint32_t const* __restrict__ cell_off, size_t q,
                                      size_t nitems, GridView g, uint32_t const* __restrict__ goff,
                                      uint32_t* __restrict__ counts,
                                      uint32_t const* __restrict__ pos, int pbits,
                                      uint64_t* __restrict__ okey, uint32_t* __restrict__ opoly,
                                      uint32_t* __restrict__ onode)
{
  CSPT_GRID_STRIDE(i, nitems)
  {
    // the node whose cell range holds item i: cell_off[n] <= i < cell_off[n + 1]
    size_t lo = 0, hi = q;
    while (hi - lo > 1) {
      size_t const mid = (lo + hi) >> 1;
      if (cell_off[mid] <= i)
        lo = mid;
      else
        hi = mid;
    }
    size_t const n  = lo;
    LeafCells const c = lc[n];
    uint32_t const k  = static_cast<uint32_t>(i - cell_off[n]);
    int const cx = c.cx0 + static_cast<int>(k % static_cast<uint32_t>(c.ncx));
    int const cy = c.cy0 + static_cast<int>(k / static_cast<uint32_t>(c.ncx));
    int const cell = cy * g.gx + cx;
    uint32_t found = 0;
    uint32_t const base = Write ? pos[i] : 0u;
    for (uint32_t j = g.cell_start[cell]; j < g.cell_start[cell + 1]; ++j) {
      uint32_t const p = g.cell_poly[j];
      int2 const pc    = g.poly_cell[p];
      if (max(pc.x, c.cx0) != cx || max(pc.y, c.cy0) != cy) continue;
      if (c.x0 > g.bmaxx[p] || c.x1 < g.bminx[p] || c.y0 > g.bmaxy[p] || c.y1 < g.bminy[p])
        continue;
      if (Write) {
        uint32_t const d = base + found;
        okey[d]          = (static_cast<uint64_t>(goff[n]) << pbits) | p;
        opoly[d]         = p;
        onode[d]         = static_cast<uint32_t>(n);
      }
      ++found;
    }
    if (!Write) counts[i] = found;
  }
}

__global__ void gather_sorted_pairs_kernel(uint32_t const* __restrict__ perm,
                                           uint32_t const* __restrict__ poly,
                                           uint32_t const* __restrict__ node, size_t k,
                                           uint32_t* __restrict__ opoly,
                                           uint32_t* __restrict__ onode)
{
  CSPT_GRID_STRIDE(i, k)
  {
    uint32_t const j = perm[i];
    opoly[i]         = poly[j];
    onode[i]         = node[j];
  }
}

// first pair of each instance (keys hold the leaf's first global position
// above pbits)
__global__ void pair_begin64_kernel(uint64_t const* __restrict__ skey, size_t k, int pbits,
                                    Inst const* __restrict__ inst, uint32_t ni,
                                    uint32_t* __restrict__ pair_begin)
{
  CSPT_GRID_STRIDE(i, static_cast<size_t>(ni) + 1)
  {
    if (i == ni) {
      pair_begin[i] = static_cast<uint32_t>(k);
      continue;
    }
    uint64_t const v = inst[i].pt_begin;
    size_t lo = 0, hi = k;
    while (lo < hi) {
      size_t const mid = (lo + hi) >> 1;
      if ((skey[mid] >> pbits) < v)
        lo = mid + 1;
      else
        hi = mid;
    }
    pair_begin[i] = static_cast<uint32_t>(lo);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// the resident polygon set
// ---------------------------------------------------------------------------
class PolygonSet {
 public:
  PolygonSet(uint32_t const* po, size_t npo, uint32_t const* ro, size_t nro, double const* vx,
             double const* vy, size_t nv, cspt_allocator const* mr, cudaStream_t s)
    : mr_copy_(mr ? *mr : cspt_allocator{}), alloc_(mr ? &mr_copy_ : nullptr, s)
  {
    Allocator const& a = alloc_;
    np_                = npo ? npo - 1 : 0;
    CSPT_EXPECTS(np_ > 0 && np_ < (size_t{1} << 31), "the polygon set must not be empty");
    // own copies of the columns (the set stays resident)
    po_ = Buffer<uint32_t>(a, npo);
    ro_ = Buffer<uint32_t>(a, nro);
    vx_ = Buffer<double>(a, nv);
    vy_ = Buffer<double>(a, nv);
    CSPT_CUDA_TRY(cudaMemcpyAsync(po_.data(), po, npo * 4, cudaMemcpyDeviceToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(ro_.data(), ro, nro * 4, cudaMemcpyDeviceToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(vx_.data(), vx, nv * 8, cudaMemcpyDeviceToDevice, s));
    CSPT_CUDA_TRY(cudaMemcpyAsync(vy_.data(), vy, nv * 8, cudaMemcpyDeviceToDevice, s));
    nro_ = nro;
    nv_  = nv;
    bminx_ = Buffer<double>(a, np_);
    bminy_ = Buffer<double>(a, np_);
    bmaxx_ = Buffer<double>(a, np_);
    bmaxy_ = Buffer<double>(a, np_);
    polygon_bounding_boxes(po_.data(), npo, ro_.data(), nro, vx_.data(), vy_.data(), nv,
                           CSPT_FLOAT64, 0.0, bminx_.data(), bminy_.data(), bmaxx_.data(),
                           bmaxy_.data(), a);
    index_.reset(new PolygonIndex<double>(po_.data(), npo, ro_.data(), nro, vx_.data(),
                                          vy_.data(), nv, true, a, /*order_slabs=*/true));
    // cell grid over the boxes
    Buffer<double> dom(a, 4);
    domain_kernel<<<1, 1024, 0, s>>>(bminx_.data(), bminy_.data(), bmaxx_.data(),
                                     bmaxy_.data(), np_, dom.data());
    CSPT_CHECK_LAUNCH();
    double d[4];
    CSPT_CUDA_TRY(cudaMemcpyAsync(d, dom.data(), sizeof d, cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    CSPT_EXPECTS(d[0] <= d[2] && d[1] <= d[3],
                 "every polygon of the set must have at least one vertex");
    int const side = static_cast<int>(std::min<double>(kGridMax, std::ceil(std::sqrt(np_))));
    g_.gx = g_.gy = std::max(side, 1);
    g_.x0         = d[0];
    g_.y0         = d[1];
    g_.cw         = (d[2] > d[0]) ? (d[2] - d[0]) / g_.gx : 1.0;
    g_.ch         = (d[3] > d[1]) ? (d[3] - d[1]) / g_.gy : 1.0;
    g_.bminx      = bminx_.data();
    g_.bminy      = bminy_.data();
    g_.bmaxx      = bmaxx_.data();
    g_.bmaxy      = bmaxy_.data();
    size_t const ncell = static_cast<size_t>(g_.gx) * g_.gy;
    cell_start_        = Buffer<uint32_t>(a, ncell + 1);
    poly_cell_         = Buffer<int2>(a, np_);
    Buffer<uint32_t> cursor(a, ncell);
    CSPT_CUDA_TRY(cudaMemsetAsync(cell_start_.data(), 0, (ncell + 1) * 4, s));
    CSPT_CUDA_TRY(cudaMemsetAsync(cursor.data(), 0, ncell * 4, s));
    unsigned const grd = grid_for(np_, 256, sm_grid(16u));
    grid_count_kernel<<<grd, 256, 0, s>>>(g_, np_, cell_start_.data(), poly_cell_.data());
    CSPT_CHECK_LAUNCH();
    exclusive_scan<uint32_t>(cell_start_.data(), cell_start_.data(), ncell,
                             cell_start_.data() + ncell, a);
    size_t const entries = read_back(cell_start_.data() + ncell, s);
    cell_poly_           = Buffer<uint32_t>(a, entries);
    g_.cell_start        = cell_start_.data();
    g_.cell_poly         = cell_poly_.data();
    g_.poly_cell         = poly_cell_.data();
    grid_fill_kernel<<<grd, 256, 0, s>>>(g_, np_, cursor.data(), cell_poly_.data());
    CSPT_CHECK_LAUNCH();
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    pbits_ = 1;
    while ((size_t{1} << pbits_) < np_) ++pbits_;
    entries_ = entries;
  }

  GridView grid() const { return g_; }
  PolygonIndexView<double> index() const { return index_->view(); }
  size_t num_polygons() const { return np_; }
  int pbits() const { return pbits_; }
  size_t entries() const { return entries_; }

 private:
  cspt_allocator mr_copy_;
  Allocator alloc_;
  size_t np_ = 0, nro_ = 0, nv_ = 0, entries_ = 0;
  int pbits_ = 1;
  Buffer<uint32_t> po_, ro_;
  Buffer<double> vx_, vy_;
  Buffer<double> bminx_, bminy_, bmaxx_, bmaxy_;
  std::unique_ptr<PolygonIndex<double>> index_;
  Buffer<uint32_t> cell_start_, cell_poly_;
  Buffer<int2> poly_cell_;
  GridView g_{};
};

// ---------------------------------------------------------------------------
// one batch of requests against the resident set
// ---------------------------------------------------------------------------
class ServingBatch {
 public:
  ServingBatch(PolygonSet const& set, size_t ni, uint64_t const* h_pt_off, double const* x,
               double const* y, cspt_instance_params const* params, cspt_method method,
               int block, Allocator const& a)
    : f_(a)
  {
    cudaStream_t const s = a.stream();
    f_.setup(ni, h_pt_off, params, nullptr);
    f_.build(x, y);
    row_off_ = Buffer<uint64_t>(a, ni + 1);
    if (f_.n_ == 0 || f_.q_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni + 1) * 8, s));
      return;
    }
    uint32_t const ni32 = static_cast<uint32_t>(ni);
    size_t const q      = f_.q_;
    GridView const g    = set.grid();
    int const pbits     = set.pbits();
    unsigned const blk = 256;
    Buffer<LeafCells> lc(a, q);
    Buffer<uint32_t> cell_off(a, q + 1);
    Buffer<uint32_t> counts;
    size_t nitems = 0;
    {
      KernelTimer timer("serving_join", s);
      leaf_cells_kernel<<<grid_for(q, blk, sm_grid(16u)), blk, 0, s>>>(
        f_.view(), f_.node_off_.data(), ni32, f_.inst_.data(), g, lc.data(), cell_off.data());
      CSPT_CHECK_LAUNCH();
      exclusive_scan<uint32_t>(cell_off.data(), cell_off.data(), q, cell_off.data() + q, a);
      nitems = read_back(cell_off.data() + q, s);
      counts = Buffer<uint32_t>(a, nitems + 1);
      if (nitems) {
        leaf_cell_join_kernel<false><<<grid_for(nitems, blk, sm_grid(16u)), blk, 0, s>>>(
          lc.data(), cell_off.data(), q, nitems, g, f_.goff_.data(), counts.data(), nullptr,
          pbits, nullptr, nullptr, nullptr);
        CSPT_CHECK_LAUNCH();
      }
      exclusive_scan<uint32_t>(counts.data(), counts.data(), nitems, counts.data() + nitems, a);
    }
    k_ = read_back(counts.data() + nitems, s);
    pair_begin_ = Buffer<uint32_t>(a, ni + 1);
    if (k_ == 0) {
      CSPT_CUDA_TRY(cudaMemsetAsync(row_off_.data(), 0, (ni + 1) * 8, s));
      return;
    }
    {
      Buffer<uint64_t> key(a, k_), key_alt(a, k_);
      Buffer<uint32_t> poly(a, k_), node(a, k_), perm(a, k_), perm_alt(a, k_);
      leaf_cell_join_kernel<true><<<grid_for(nitems, blk, sm_grid(16u)), blk, 0, s>>>(
        lc.data(), cell_off.data(), q, nitems, g, f_.goff_.data(), nullptr, counts.data(), pbits,
        key.data(), poly.data(), node.data());
      CSPT_CHECK_LAUNCH();
      int const bits = 32 + pbits;
      KernelTimer timer("serving_sort", s);
      bool const alt = radix_sort_pairs<uint64_t>(key.data(), perm.data(), key_alt.data(),
                                                  perm_alt.data(), k_, 0, bits, true, a);
      pair_poly_ = Buffer<uint32_t>(a, k_);
      pair_quad_ = Buffer<uint32_t>(a, k_);
      gather_sorted_pairs_kernel<<<grid_for(k_, 256, sm_grid(16u)), 256, 0, s>>>(
        alt ? perm_alt.data() : perm.data(), poly.data(), node.data(), k_, pair_poly_.data(),
        pair_quad_.data());
      CSPT_CHECK_LAUNCH();
      pair_begin64_kernel<<<grid_for(ni + 1, 256, sm_grid(16u)), 256, 0, s>>>(
        alt ? key_alt.data() : key.data(), k_, pbits, f_.inst_.data(), ni32,
        pair_begin_.data());
      CSPT_CHECK_LAUNCH();
    }
    PipExec pip(pair_poly_.data(), pair_quad_.data(), k_, f_.length_.data(), f_.goff_.data(),
                f_.sidx_.data(), f_.n_, x, y, set.index(), method == CSPT_METHOD_FILTERED,
                static_cast<unsigned>(block), a);
    {
      KernelTimer timer("serving_pip", s);
      pip.evaluate(s);
    }
    m_  = read_back(pip.total(), s);
    op_ = Buffer<uint32_t>(a, m_);
    oq_ = Buffer<uint32_t>(a, m_);
    pip.expand(s, op_.data(), oq_.data(), m_);
    row_offsets_kernel<<<grid_for(ni + 1, 256, sm_grid(16u)), 256, 0, s>>>(
      pair_begin_.data(), pip.pair_out_offsets(), ni32, row_off_.data());
    CSPT_CHECK_LAUNCH();
    if (m_) {
      localize_kernel<<<grid_for(m_, 256, sm_grid(16u)), 256, 0, s>>>(
        op_.data(), oq_.data(), m_, f_.pt_begin_.data(), f_.tile_inst_.data(), f_.inst_.data(),
        false);
      CSPT_CHECK_LAUNCH();
    }
    refined_ = read_back(pip.refined(), s);
  }

  Forest f_;
  size_t k_ = 0, m_ = 0;
  uint64_t refined_ = 0;
  Buffer<uint64_t> row_off_;
  Buffer<uint32_t> pair_poly_, pair_quad_, pair_begin_, op_, oq_;
};

// ---------------------------------------------------------------------------
// device-memory budget shared by a server's workers
// ---------------------------------------------------------------------------
struct Budget {
  size_t limit;
  std::atomic<size_t> in_use{0};
  std::atomic<size_t> peak{0};
  static void* allocate(void* ctx, size_t bytes, void* stream)
  {
    auto* b      = static_cast<Budget*>(ctx);
    size_t const now = b->in_use.fetch_add(bytes) + bytes;
    if (now > b->limit) {
      b->in_use.fetch_sub(bytes);
      return nullptr;
    }
    size_t p = b->peak.load();
    while (now > p && !b->peak.compare_exchange_weak(p, now)) {
    }
    void* ptr = nullptr;
    if (cudaMallocFromPoolAsync(&ptr, bytes, library_pool(), static_cast<cudaStream_t>(stream)) !=
        cudaSuccess) {
      (void)cudaGetLastError();
      b->in_use.fetch_sub(bytes);
      return nullptr;
    }
    return ptr;
  }
  static void deallocate(void* ctx, void* ptr, size_t bytes, void* stream)
  {
    auto* b = static_cast<Budget*>(ctx);
    (void)cudaFreeAsync(ptr, static_cast<cudaStream_t>(stream));
    b->in_use.fetch_sub(bytes);
  }
};

// ---------------------------------------------------------------------------
// the server
// ---------------------------------------------------------------------------
class Server {
 public:
  struct Request {
    uint64_t id;
    double const* hx;
    double const* hy;
    size_t n;
    cspt_instance_params params;
    size_t estimate;
    double submit_s = 0, admit_s = 0, done_s = 0;
    uint64_t batch         = 0;
    uint32_t batch_size    = 0;
    cspt_status status     = CSPT_OK;
    bool solo              = false;  // retried alone after a batch ran out of memory
    std::string error;
    std::vector<uint32_t> poly, point, point_indices;
  };

  Server(PolygonSet const* set, cspt_server_options const& o)
    : set_(set), opt_(o), t0_(std::chrono::steady_clock::now())
  {
    budget_.limit = o.memory_budget_bytes;
    CSPT_CUDA_TRY(cudaGetDevice(&device_));
    int const nw = std::max(1, o.num_streams);
    // every worker's stream exists before any worker starts: a failure is
    // reported here, to the caller creating the server
    streams_.resize(nw, nullptr);
    for (int w = 0; w < nw; ++w) {
      cudaError_t const e = cudaStreamCreateWithFlags(&streams_[w], cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        for (int v = 0; v < w; ++v) cudaStreamDestroy(streams_[v]);
        throw Error{CSPT_CUDA_ERROR, std::string("cannot create a serving stream: ") +
                                       cudaGetErrorString(e)};
      }
    }
    for (int w = 0; w < nw; ++w) workers_.emplace_back([this, w] { worker(streams_[w]); });
  }

  ~Server()
  {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
    for (cudaStream_t st : streams_) cudaStreamDestroy(st);
  }

  double now() const
  {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }

  // working memory of a request: sort, level and tree arrays of its points
  // plus a fixed part (instance table, scans, pairs of small requests)
  static size_t estimate(size_t n) { return n * 256 + (size_t{1} << 20); }

  void submit(uint64_t id, double const* hx, double const* hy, size_t n,
              cspt_instance_params const& p)
  {
    CSPT_EXPECTS(p.scale > 0, "scale must be positive");
    CSPT_EXPECTS(p.x_min < p.x_max && p.y_min < p.y_max,
                 "invalid bounding box (x_min, x_max, y_min, y_max)");
    CSPT_EXPECTS(p.max_depth > 0 && p.max_depth < 16,
                 "maximum depth must be positive and less than 16");
    CSPT_EXPECTS(n == 0 || (hx && hy), "request points must not be null");
    CSPT_EXPECTS(n < (size_t{1} << 31), "a request holds fewer than 2^31 points");
    auto r       = std::make_unique<Request>();
    r->id        = id;
    r->hx        = hx;
    r->hy        = hy;
    r->n         = n;
    r->params    = p;
    r->estimate  = estimate(n);
    r->submit_s  = now();
    {
      std::lock_guard<std::mutex> lk(mu_);
      CSPT_EXPECTS(all_.find(id) == all_.end(), "request id already in use");
      Request* raw = r.get();
      all_.emplace(id, std::move(r));
      queue_.push_back(raw);
      ++submitted_;
    }
    cv_.notify_all();
  }

  size_t poll(uint64_t* ids, size_t max_ids, double timeout_s)
  {
    std::unique_lock<std::mutex> lk(mu_);
    if (done_.empty() && timeout_s > 0)
      done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s),
                        [this] { return !done_.empty(); });
    size_t k = 0;
    while (k < max_ids && !done_.empty()) {
      ids[k++] = done_.front();
      done_.pop_front();
    }
    return k;
  }

  Request const* find(uint64_t id)
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = all_.find(id);
    return (it == all_.end() || !it->second->done_s) ? nullptr : it->second.get();
  }

  void release(uint64_t id)
  {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = all_.find(id);
    if (it != all_.end() && it->second->done_s) all_.erase(it);
  }

  void stats(cspt_server_stats* o)
  {
    std::lock_guard<std::mutex> lk(mu_);
    o->submitted   = submitted_;
    o->completed   = completed_;
    o->failed      = failed_;
    o->batches     = batches_;
    o->split_batches = splits_;
    o->queued      = queue_.size();
    o->reserved_bytes = reserved_;
    o->peak_device_bytes = budget_.peak.load();
    o->memory_budget_bytes = budget_.limit;
    o->max_batch_requests_seen = max_batch_seen_;
  }

 private:
  // Takes the next batch off the queue: requests in arrival order while the
  // points, request count and reserved memory stay within the limits.
  std::vector<Request*> next_batch()
  {
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      if (stop_ && queue_.empty()) return {};
      if (!queue_.empty()) {
        Request* head = queue_.front();
        if (head->estimate > budget_.limit) {
          queue_.pop_front();
          fail_locked(head, CSPT_OUT_OF_MEMORY,
                      "request needs about " + std::to_string(head->estimate) +
                        " bytes of device memory, above the memory budget");
          continue;
        }
        if (reserved_ + head->estimate <= budget_.limit) {
          std::vector<Request*> b;
          size_t pts = 0, mem = 0;
          bool const solo = head->solo;
          while (!queue_.empty()) {
            Request* r = queue_.front();
            if (!b.empty() && (solo || r->solo || b.size() >= opt_.max_batch_requests ||
                               pts + r->n > opt_.max_batch_points ||
                               reserved_ + mem + r->estimate > budget_.limit))
              break;
            queue_.pop_front();
            b.push_back(r);
            pts += r->n;
            mem += r->estimate;
          }
          reserved_ += mem;
          double const t = now();
          for (Request* r : b) r->admit_s = t;
          max_batch_seen_ = std::max<uint64_t>(max_batch_seen_, b.size());
          return b;
        }
      }
      cv_.wait(lk);
    }
  }

  void fail_locked(Request* r, cspt_status st, std::string const& msg)
  {
    r->status = st;
    r->error  = msg;
    r->done_s = now();
    ++failed_;
    done_.push_back(r->id);
    done_cv_.notify_all();
  }

  void worker(cudaStream_t s)
  {
    cudaSetDevice(device_);
    cspt_allocator mr{&budget_, &Budget::allocate, &Budget::deallocate};
    Allocator alloc(&mr, s);
    for (;;) {
      std::vector<Request*> b = next_batch();
      if (b.empty()) break;
      size_t mem = 0;
      for (Request* r : b) mem += r->estimate;
      cspt_status st = CSPT_OK;
      std::string msg;
      uint64_t batch_id;
      {
        std::lock_guard<std::mutex> lk(mu_);
        batch_id = ++batches_;
      }
      try {
        run_batch(b, alloc, s, batch_id);
      } catch (Error const& e) {
        st  = e.status;
        msg = e.message;
      } catch (std::exception const& e) {
        st  = CSPT_CUDA_ERROR;
        msg = e.what();
      }
      if (st != CSPT_OK) {
        (void)cudaStreamSynchronize(s);
        (void)cudaGetLastError();
      }
      {
        std::lock_guard<std::mutex> lk(mu_);
        reserved_ -= mem;
        if (st == CSPT_OUT_OF_MEMORY && b.size() > 1) {
          // retry the requests one by one, ahead of later arrivals
          ++splits_;
          for (auto it = b.rbegin(); it != b.rend(); ++it) {
            (*it)->solo = true;
            queue_.push_front(*it);
          }
        } else if (st != CSPT_OK) {
          for (Request* r : b) fail_locked(r, st, msg);
        } else {
          double const t = now();
          for (Request* r : b) {
            r->done_s = t;
            ++completed_;
            done_.push_back(r->id);
          }
          done_cv_.notify_all();
        }
      }
      cv_.notify_all();
    }
  }

  void run_batch(std::vector<Request*>& b, Allocator const& alloc, cudaStream_t s,
                 uint64_t batch_id)
  {
    size_t const ni = b.size();
    std::vector<uint64_t> off(ni + 1, 0);
    std::vector<cspt_instance_params> params(ni);
    for (size_t i = 0; i < ni; ++i) {
      off[i + 1] = off[i] + b[i]->n;
      params[i]  = b[i]->params;
    }
    size_t const n = off[ni];
    Buffer<double> dx(alloc, n), dy(alloc, n);
    for (size_t i = 0; i < ni; ++i) {
      if (!b[i]->n) continue;
      CSPT_CUDA_TRY(cudaMemcpyAsync(dx.data() + off[i], b[i]->hx, b[i]->n * 8,
                                    cudaMemcpyHostToDevice, s));
      CSPT_CUDA_TRY(cudaMemcpyAsync(dy.data() + off[i], b[i]->hy, b[i]->n * 8,
                                    cudaMemcpyHostToDevice, s));
    }
    ServingBatch sb(*set_, ni, off.data(), dx.data(), dy.data(), params.data(), opt_.method,
                    opt_.block_threads, alloc);
    std::vector<uint64_t> ro(ni + 1, 0);
    std::vector<uint32_t> poly(sb.m_), point(sb.m_), pidx(n);
    CSPT_CUDA_TRY(
      cudaMemcpyAsync(ro.data(), sb.row_off_.data(), (ni + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (sb.m_) {
      CSPT_CUDA_TRY(cudaMemcpyAsync(poly.data(), sb.op_.data(), sb.m_ * 4,
                                    cudaMemcpyDeviceToHost, s));
      CSPT_CUDA_TRY(cudaMemcpyAsync(point.data(), sb.oq_.data(), sb.m_ * 4,
                                    cudaMemcpyDeviceToHost, s));
    }
    if (n && sb.f_.pidx_.data())
      CSPT_CUDA_TRY(cudaMemcpyAsync(pidx.data(), sb.f_.pidx_.data(), n * 4,
                                    cudaMemcpyDeviceToHost, s));
    CSPT_CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i < ni; ++i) {
      Request* r = b[i];
      r->poly.assign(poly.begin() + ro[i], poly.begin() + ro[i + 1]);
      r->point.assign(point.begin() + ro[i], point.begin() + ro[i + 1]);
      r->point_indices.assign(pidx.begin() + off[i], pidx.begin() + off[i + 1]);
      r->batch      = batch_id;
      r->batch_size = static_cast<uint32_t>(ni);
      r->status     = CSPT_OK;
    }
  }

  PolygonSet const* set_;
  cspt_server_options opt_;
  std::chrono::steady_clock::time_point t0_;
  int device_ = 0;
  Budget budget_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> queue_;
  std::deque<uint64_t> done_;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> all_;
  size_t reserved_ = 0;
  uint64_t submitted_ = 0, completed_ = 0, failed_ = 0, batches_ = 0, splits_ = 0;
  uint64_t max_batch_seen_ = 0;
  bool stop_ = false;
  std::vector<std::thread> workers_;
  std::vector<cudaStream_t> streams_;
};

}  // namespace cspt

using namespace cspt;

extern "C" {

cspt_status cspt_polygon_set_create(const uint32_t* poly_offsets, size_t num_poly_offsets,
                                    const uint32_t* ring_offsets, size_t num_ring_offsets,
                                    const void* poly_x, const void* poly_y,
                                    size_t num_poly_vertices, cspt_dtype dtype,
                                    const cspt_allocator* mr, void* stream,
                                    cspt_polygon_set** out)
{
  return guarded([&] {
    CSPT_EXPECTS(out, "output pointers must not be null");
    *out = nullptr;
    if (dtype != CSPT_FLOAT32 && dtype != CSPT_FLOAT64)
      throw Error{CSPT_UNSUPPORTED, "Only floating-point types are supported"};
    if (dtype != CSPT_FLOAT64)
      throw Error{CSPT_UNSUPPORTED, "the serving form supports float64 coordinates"};
    *out = reinterpret_cast<cspt_polygon_set*>(new PolygonSet(
      poly_offsets, num_poly_offsets, ring_offsets, num_ring_offsets,
      static_cast<double const*>(poly_x), static_cast<double const*>(poly_y), num_poly_vertices,
      mr, static_cast<cudaStream_t>(stream)));
  });
}

void cspt_polygon_set_free(cspt_polygon_set* set) { delete reinterpret_cast<PolygonSet*>(set); }

cspt_status cspt_server_create(const cspt_polygon_set* set, const cspt_server_options* options,
                               cspt_server** out)
{
  return guarded([&] {
    CSPT_EXPECTS(set && options && out, "arguments must not be null");
    *out = nullptr;
    CSPT_EXPECTS(options->block_threads >= 32 && options->block_threads <= 256 &&
                   options->block_threads % 32 == 0,
                 "block_threads must be a multiple of 32 in [32, 256]");
    CSPT_EXPECTS(options->max_batch_requests >= 1 && options->max_batch_points >= 1,
                 "batch limits must be positive");
    CSPT_EXPECTS(options->method == CSPT_METHOD_EXACT || options->method == CSPT_METHOD_FILTERED,
                 "unknown point-in-polygon method");
    *out = reinterpret_cast<cspt_server*>(
      new Server(reinterpret_cast<PolygonSet const*>(set), *options));
  });
}

cspt_status cspt_server_submit(cspt_server* server, uint64_t request_id, const double* x,
                               const double* y, size_t num_points,
                               const cspt_instance_params* params)
{
  return guarded([&] {
    CSPT_EXPECTS(server && params, "arguments must not be null");
    reinterpret_cast<Server*>(server)->submit(request_id, x, y, num_points, *params);
  });
}

size_t cspt_server_poll(cspt_server* server, uint64_t* ids, size_t max_ids, double timeout_s)
{
  if (!server || !ids) return 0;
  return reinterpret_cast<Server*>(server)->poll(ids, max_ids, timeout_s);
}

cspt_status cspt_server_result(cspt_server* server, uint64_t request_id,
                               cspt_request_result* out)
{
  return guarded([&] {
    CSPT_EXPECTS(server && out, "arguments must not be null");
    auto const* r = reinterpret_cast<Server*>(server)->find(request_id);
    CSPT_EXPECTS(r, "no completed request with this id");
    out->status         = r->status;
    out->error          = r->error.c_str();
    out->polygon_index  = r->poly.data();
    out->point_index    = r->point.data();
    out->num_rows       = r->poly.size();
    out->point_indices  = r->point_indices.data();
    out->num_points     = r->point_indices.size();
    out->submit_s       = r->submit_s;
    out->admit_s        = r->admit_s;
    out->done_s         = r->done_s;
    out->batch          = r->batch;
    out->batch_requests = r->batch_size;
  });
}

void cspt_server_release(cspt_server* server, uint64_t request_id)
{
  if (server) reinterpret_cast<Server*>(server)->release(request_id);
}

double cspt_server_now(const cspt_server* server)
{
  return server ? reinterpret_cast<Server const*>(server)->now() : 0.0;
}

cspt_status cspt_server_get_stats(cspt_server* server, cspt_server_stats* out)
{
  return guarded([&] {
    CSPT_EXPECTS(server && out, "arguments must not be null");
    reinterpret_cast<Server*>(server)->stats(out);
  });
}

void cspt_server_free(cspt_server* server) { delete reinterpret_cast<Server*>(server); }

}  // extern "C"
