// CPU oracle for the quadtree spatial-join path of cuSpatial 25.06.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain C++17 restatement of the
// reference algorithm, written step by step after the reference sources cited
// on each function (paths are relative to the cuSpatial repository).  It is
// the checker for the CUDA library in cuspatial_gb300/ and the timed CPU
// baseline; nothing in the product links or calls it.
//
// Floating-point expressions follow the reference's evaluation order.  Where
// the reference's device code is compiled with nvcc's default FMA contraction
// (`a*b + c` patterns), the oracle calls std::fma explicitly; the file is built
// with -ffp-contract=off so that no other expression is contracted.
//
// The one place the oracle deliberately differs from a literal reading of the
// reference is the parent-node count of the quadtree when keys above bit 2*d
// produce several roots (reference: detail/index/construction/phase_1.cuh:
// 174-177 counts `end - num_top_quads - 1`, which assumes a single root and
// leads to an out-of-bounds scatter in phase_2.cuh:159-167 otherwise).  The
// oracle counts the nodes of levels 0..max_depth-2, which equals the
// reference's count whenever the tree has a single root.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_last_error;

template <typename T>
struct bits_of;
template <>
struct bits_of<float> {
  using type = uint32_t;
};
template <>
struct bits_of<double> {
  using type = uint64_t;
};

// detail/utility/floating_point.cuh:97-129 — ULP comparison on the biased
// integer image of the two values, at most 4 units apart, NaN never equal.
template <typename T>
bool float_equal(T a, T b)
{
  if (std::isnan(a) || std::isnan(b)) return false;
  using U = typename bits_of<T>::type;
  U ua, ub;
  std::memcpy(&ua, &a, sizeof(T));
  std::memcpy(&ub, &b, sizeof(T));
  U const sign = U{1} << (8 * sizeof(U) - 1);
  auto biased  = [sign](U s) -> U { return (s & sign) ? U(~s + 1) : U(s | sign); };
  U const ba   = biased(ua);
  U const bb   = biased(ub);
  return (ba >= bb ? ba - bb : bb - ba) <= 4u;
}

// detail/utility/z_order.cuh:69-77 — bit interleave, x in even bits, y in odd
// bits.  Computed arithmetically rather than by table.
inline uint32_t spread16(uint32_t v)
{
  v &= 0xFFFFu;
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
inline uint32_t gather16(uint32_t v)
{
  v &= 0x55555555u;
  v = (v | (v >> 1)) & 0x33333333u;
  v = (v | (v >> 2)) & 0x0F0F0F0Fu;
  v = (v | (v >> 4)) & 0x00FF00FFu;
  v = (v | (v >> 8)) & 0x0000FFFFu;
  return v;
}
inline uint32_t z_order(uint16_t x, uint16_t y) { return (spread16(y) << 1) | spread16(x); }
inline uint16_t z_order_x(uint32_t k) { return static_cast<uint16_t>(gather16(k)); }
inline uint16_t z_order_y(uint32_t k) { return static_cast<uint16_t>(gather16(k >> 1)); }

struct Tree {
  std::vector<uint32_t> point_indices;
  std::vector<uint32_t> key;
  std::vector<uint8_t> level;
  std::vector<uint8_t> is_internal;
  std::vector<uint32_t> length;
  std::vector<uint32_t> offset;
};

// point_quadtree.cuh / detail/point_quadtree.cuh:237-272 (clamps) and
// :190-233 (construct_quadtree); phase_1.cuh:60-381; phase_2.cuh:56-345;
// detail/point_quadtree.cuh:43-188 (make_quad_tree / make_leaf_tree).
template <typename T>
Tree quadtree_on_points(T const* xs, T const* ys, size_t n, T x1, T x2, T y1, T y2, T scale,
                        int max_depth_in, int32_t max_size)
{
  Tree t;
  if (n == 0) return t;
  T const minx = std::min(x1, x2), maxx = std::max(x1, x2);
  T const miny = std::min(y1, y2), maxy = std::max(y1, y2);
  max_size      = std::max(1, max_size);
  int const d   = std::max(0, std::min(15, max_depth_in));
  scale = std::max(scale, std::max(maxx - minx, maxy - miny) / static_cast<T>((1 << d) + 2));

  // phase_1.cuh:73-85 — Morton keys; points outside the box get the last
  // key of the deepest level.
  std::vector<uint32_t> keys(n);
  for (size_t i = 0; i < n; ++i) {
    T const x = xs[i], y = ys[i];
    if (x < minx || x > maxx || y < miny || y > maxy) {
      keys[i] = static_cast<uint32_t>((1 << (2 * d)) - 1);
    } else {
      keys[i] = z_order(static_cast<uint16_t>((x - minx) / scale),
                        static_cast<uint16_t>((y - miny) / scale));
    }
  }
  // phase_1.cuh:87-92 — stable sort of (key, original index).
  t.point_indices.resize(n);
  std::iota(t.point_indices.begin(), t.point_indices.end(), 0u);
  std::stable_sort(t.point_indices.begin(), t.point_indices.end(),
                   [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  std::vector<uint32_t> sorted_keys(n);
  for (size_t i = 0; i < n; ++i) sorted_keys[i] = keys[t.point_indices[i]];

  // phase_1.cuh:274-285 — bottom quadrants: one node per distinct key.
  std::vector<uint32_t> qkey, qpts, qchild;
  for (size_t i = 0; i < n; ++i) {
    if (i == 0 || sorted_keys[i] != sorted_keys[i - 1]) {
      qkey.push_back(sorted_keys[i]);
      qpts.push_back(1);
    } else {
      ++qpts.back();
    }
  }
  size_t const nb = qkey.size();
  qchild.assign(nb, 0);

  // phase_1.cuh:130-157 — reduce each level into its parents (key >> 2),
  // appending levels bottom-up; remember where each level lives.
  std::vector<size_t> begin_pos(d), end_pos(d);
  size_t begin = 0, end = nb;
  for (int level = d - 1; level >= 0; --level) {
    size_t produced = 0;
    for (size_t i = begin; i < end; ++i) {
      uint32_t const pk = qkey[i] >> 2;
      if (i == begin || pk != (qkey[i - 1] >> 2)) {
        qkey.push_back(pk);
        qpts.push_back(qpts[i]);
        qchild.push_back(1);
        ++produced;
      } else {
        qpts.back() += qpts[i];
        qchild.back() += 1;
      }
    }
    end_pos[level]   = end;
    begin_pos[level] = begin;
    begin            = end;
    end              = end + produced;
  }

  // Parent-node count: nodes of levels 0..d-2 (see the file header).
  int64_t num_parent_nodes = 0;
  for (int level = 0; level + 1 < d; ++level)
    num_parent_nodes += static_cast<int64_t>(end_pos[level] - begin_pos[level]);

  if (num_parent_nodes <= 0) {
    // detail/point_quadtree.cuh:155-188 — leaf-only tree of the bottom quads.
    t.key.assign(qkey.begin(), qkey.begin() + nb);
    t.length.assign(qpts.begin(), qpts.begin() + nb);
    t.level.assign(nb, 0);
    t.is_internal.assign(nb, 0);
    t.offset.resize(nb);
    uint32_t acc = 0;
    for (size_t i = 0; i < nb; ++i) {
      t.offset[i] = acc;
      acc += t.length[i];
    }
    return t;
  }

  // phase_1.cuh:185-232 — reverse the level order (root excluded).
  std::vector<uint32_t> keys_r, pts_r, child_r;
  std::vector<uint8_t> lev_r;
  for (int level = 0; level < d; ++level) {
    for (size_t i = begin_pos[level]; i < end_pos[level]; ++i) {
      keys_r.push_back(qkey[i]);
      pts_r.push_back(qpts[i]);
      child_r.push_back(qchild[i]);
      lev_r.push_back(static_cast<uint8_t>(level));
    }
  }
  size_t const level_1_size = end_pos[0] - begin_pos[0];
  size_t const np           = static_cast<size_t>(num_parent_nodes);

  // detail/point_quadtree.cuh:55-57 — number of child nodes.
  size_t num_child_nodes = 0;
  for (size_t i = 0; i < np; ++i) num_child_nodes += child_r[i];

  // phase_2.cuh:143-177 — parent position of every child node.
  std::vector<uint32_t> parent_pos(num_child_nodes, 0);
  {
    size_t acc = 0;
    for (size_t i = 0; i < np; ++i) {
      if (acc < num_child_nodes) parent_pos[acc] = static_cast<uint32_t>(i);
      acc += child_r[i];
    }
    for (size_t j = 1; j < num_child_nodes; ++j)
      parent_pos[j] = std::max(parent_pos[j], parent_pos[j - 1]);
  }
  // phase_2.cuh:206-236 — drop children whose parent holds <= max_size points
  // (level-0 nodes are always kept).
  size_t num_invalid = 0;
  for (size_t j = 0; j + level_1_size < np; ++j)
    if (pts_r[parent_pos[j]] <= static_cast<uint32_t>(max_size)) ++num_invalid;
  {
    std::vector<char> drop(num_child_nodes);
    for (size_t j = 0; j < num_child_nodes; ++j)
      drop[j] = pts_r[parent_pos[j]] <= static_cast<uint32_t>(max_size);
    size_t w = level_1_size;
    for (size_t j = 0; j < num_child_nodes; ++j) {
      if (drop[j]) continue;
      size_t const r = level_1_size + j;
      keys_r[w]      = keys_r[r];
      pts_r[w]       = pts_r[r];
      child_r[w]     = child_r[r];
      lev_r[w]       = lev_r[r];
      ++w;
    }
    keys_r.resize(w);
    pts_r.resize(w);
    child_r.resize(w);
    lev_r.resize(w);
  }
  size_t const num_valid = keys_r.size();
  size_t const np2       = np - num_invalid;

  // phase_2.cuh:275-311 — internal flag and zeroed point counts of parents.
  std::vector<uint8_t> internal(num_valid, 0);
  for (size_t i = 0; i < np2; ++i) {
    internal[i] = pts_r[i] > static_cast<uint32_t>(max_size);
    if (internal[i]) pts_r[i] = 0;
  }

  // phase_2.cuh:71-141 — first point position of every leaf, via the leaves
  // ordered by their keys flattened to the bottom level.
  std::vector<uint32_t> point_pos(num_valid, 0);
  {
    std::vector<uint32_t> flat(num_valid), order(num_valid);
    for (size_t i = 0; i < num_valid; ++i)
      flat[i] = internal[i] ? 0xFFFFFFFFu : (keys_r[i] << (2 * (d - 1 - lev_r[i])));
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(
      order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return flat[a] < flat[b]; });
    std::vector<uint32_t> counts_sorted;
    for (size_t k = 0; k < num_valid; ++k)
      if (pts_r[order[k]] != 0) counts_sorted.push_back(pts_r[order[k]]);
    std::vector<uint32_t> leaf_idx;
    for (size_t i = 0; i < num_valid; ++i)
      if (!internal[i]) leaf_idx.push_back(static_cast<uint32_t>(i));
    size_t const nl = leaf_idx.size();
    // initial indices of the first nl sorted entries, with their exclusive
    // point-count scan, sorted back by node index and scattered to the leaves
    std::vector<std::pair<uint32_t, std::pair<uint32_t, uint32_t>>> rows(nl);
    uint32_t acc = 0;
    for (size_t k = 0; k < nl; ++k) {
      uint32_t const c = k < counts_sorted.size() ? counts_sorted[k] : 0;
      rows[k]          = {order[k], {c, acc}};
      acc += c;
    }
    std::stable_sort(rows.begin(), rows.end(),
                     [](auto const& a, auto const& b) { return a.first < b.first; });
    for (size_t k = 0; k < nl; ++k) {
      pts_r[leaf_idx[k]]     = rows[k].second.first;
      point_pos[leaf_idx[k]] = rows[k].second.second;
    }
  }
  // detail/point_quadtree.cuh:82-131 — child offsets scan from level_1_size,
  // then select (length, offset) by the internal flag.
  t.key.resize(num_valid);
  t.level.resize(num_valid);
  t.is_internal.resize(num_valid);
  t.length.resize(num_valid);
  t.offset.resize(num_valid);
  uint32_t child_acc = static_cast<uint32_t>(level_1_size);
  for (size_t i = 0; i < num_valid; ++i) {
    uint32_t const cc = internal[i] ? child_r[i] : 0;
    t.key[i]          = keys_r[i];
    t.level[i]        = lev_r[i];
    t.is_internal[i]  = internal[i];
    t.length[i]       = internal[i] ? cc : pts_r[i];
    t.offset[i]       = internal[i] ? child_acc : point_pos[i];
    child_acc += cc;
  }
  return t;
}

// detail/bounding_boxes.cuh:37-58, 139-184 — per-geometry min/max of every
// vertex expanded by +-r, reduced by geometry id.  A geometry without
// vertices produces no row, so later rows move up (reduce_by_key semantics);
// the rows left over at the end are filled with NaN here.
template <typename T>
void bounding_boxes(std::vector<int64_t> const& vert_begin, std::vector<int64_t> const& vert_end,
                    T const* x, T const* y, T r, T* ominx, T* ominy, T* omaxx, T* omaxy)
{
  size_t const ng = vert_begin.size();
  size_t row      = 0;
  for (size_t g = 0; g < ng; ++g) {
    if (vert_end[g] <= vert_begin[g]) continue;
    T mnx = x[vert_begin[g]] - r, mny = y[vert_begin[g]] - r;
    T mxx = x[vert_begin[g]] + r, mxy = y[vert_begin[g]] + r;
    for (int64_t v = vert_begin[g] + 1; v < vert_end[g]; ++v) {
      mnx = std::min(mnx, x[v] - r);
      mny = std::min(mny, y[v] - r);
      mxx = std::max(mxx, x[v] + r);
      mxy = std::max(mxy, y[v] + r);
    }
    ominx[row] = mnx;
    ominy[row] = mny;
    omaxx[row] = mxx;
    omaxy[row] = mxy;
    ++row;
  }
  for (; row < ng; ++row)
    ominx[row] = ominy[row] = omaxx[row] = omaxy[row] = std::numeric_limits<T>::quiet_NaN();
}

inline float fma_t(float a, float b, float c) { return std::fma(a, b, c); }
inline double fma_t(double a, double b, double c) { return std::fma(a, b, c); }

// quadtree_bbox_filtering.cuh:35-188, intersection.cuh:79-136,
// traversal.cuh:57-145 — level-synchronous descent, then a stable sort of
// the (bbox, leaf) pairs by the leaf's first-point offset.
template <typename T>
void join_quadtree_and_bboxes(uint32_t const* key, uint8_t const* level, uint8_t const* internal,
                              uint32_t const* length, uint32_t const* offset, size_t nq,
                              T const* bminx, T const* bminy, T const* bmaxx, T const* bmaxy,
                              size_t nb, T vminx, T vminy, T scale, int max_depth,
                              std::vector<uint32_t>& out_bbox, std::vector<uint32_t>& out_quad)
{
  out_bbox.clear();
  out_quad.clear();
  size_t L0 = 0;
  for (size_t i = 0; i < nq; ++i) L0 += level[i] == 0;
  struct P {
    uint32_t node, bbox;
  };
  std::vector<P> cur;
  cur.reserve(L0 * nb);
  for (size_t i = 0; i < L0 * nb; ++i)
    cur.push_back({static_cast<uint32_t>(i % L0), static_cast<uint32_t>(i / L0)});

  // intersection.cuh:94-128
  auto classify = [&](P const& p) -> int {  // 0 leaf, 1 quad, 2 none
    uint32_t const k   = key[p.node];
    uint8_t const lev  = level[p.node];
    T const kx         = static_cast<T>(z_order_x(k));
    T const ky         = static_cast<T>(z_order_y(k));
    T const ls         = scale * static_cast<T>(1 << (max_depth - 1 - lev));
    T const nxmin      = fma_t(kx + T{0}, ls, vminx);
    T const nymin      = fma_t(ky + T{0}, ls, vminy);
    T const nxmax      = fma_t(kx + T{1}, ls, vminx);
    T const nymax      = fma_t(ky + T{1}, ls, vminy);
    if (nxmin > bmaxx[p.bbox] || nxmax < bminx[p.bbox] || nymin > bmaxy[p.bbox] ||
        nymax < bminy[p.bbox])
      return 2;
    return internal[p.node] ? 1 : 0;
  };
  std::vector<P> leaves;
  auto step = [&](std::vector<P> const& in) {
    std::vector<P> parents;
    for (auto const& p : in) {
      int const c = classify(p);
      if (c == 0) leaves.push_back(p);
      if (c == 1) parents.push_back(p);
    }
    return parents;
  };
  std::vector<P> parents = step(cur);
  for (int lev = 1; lev < max_depth && !parents.empty(); ++lev) {
    std::vector<P> next;
    for (auto const& p : parents)
      for (uint32_t c = 0; c < length[p.node]; ++c) next.push_back({offset[p.node] + c, p.bbox});
    parents = step(next);
  }
  std::stable_sort(leaves.begin(), leaves.end(), [&](P const& a, P const& b) {
    return offset[a.node] < offset[b.node];
  });
  out_bbox.reserve(leaves.size());
  out_quad.reserve(leaves.size());
  for (auto const& p : leaves) {
    out_bbox.push_back(p.bbox);
    out_quad.push_back(p.node);
  }
}

// detail/algorithm/is_point_in_polygon.cuh:45-100 — crossing test over every
// ring, false on an edge.  Polygon = rings [ring_begin, ring_end).
template <typename T, typename Off>
bool is_point_in_polygon(T px, T py, Off const* ring_offsets, int64_t ring_begin,
                         int64_t ring_end, T const* vx, T const* vy)
{
  bool within  = false;
  bool on_edge = false;
  for (int64_t r = ring_begin; r < ring_end; ++r) {
    int64_t const v0 = ring_offsets[r];
    int64_t const v1 = ring_offsets[r + 1];
    // last segment's second point = the ring's last vertex
    T bx       = vx[v1 - 1];
    T by       = vy[v1 - 1];
    bool y0    = by > py;
    bool y1    = false;
    for (int64_t v = v0; v < v1; ++v) {
      T const ax   = vx[v];
      T const ay   = vy[v];
      T const run  = bx - ax;
      T const rise = by - ay;
      if (float_equal(run, T{0}) && float_equal(rise, T{0})) continue;
      T const rise_to_point = py - ay;
      T const run_to_point  = px - ax;
      bool const collinear  = float_equal(run * rise_to_point, run_to_point * rise);
      if (collinear) {
        T mn = ax, mx = bx;
        if (mn > mx) std::swap(mn, mx);
        if (mn <= px && px <= mx) {
          on_edge = true;
          break;
        }
      }
      y1 = ay > py;
      if (y1 != y0) {
        T const lhs = (px - ax) * rise;
        T const rhs = run * rise_to_point;
        if ((lhs < rhs) != y1) within = !within;
      }
      bx = ax;
      by = ay;
      y0 = y1;
    }
    if (on_edge) {
      within = false;
      break;
    }
  }
  return within;
}

// quadtree_point_in_polygon.cuh:104-235 with
// get_quad_and_local_point_indices.cuh:26-45 — every point of every paired
// quadrant is tested against the paired polygon; output in pair order, then
// point position.  point_index is a position in point_indices.
template <typename T, typename Off>
void quadtree_point_in_polygon(uint32_t const* pair_poly, uint32_t const* pair_quad, size_t np,
                               uint32_t const* length, uint32_t const* offset,
                               uint32_t const* point_indices, size_t npi, T const* x, T const* y,
                               Off const* poly_offsets, Off const* ring_offsets, T const* vx,
                               T const* vy, std::vector<uint32_t>& out_poly,
                               std::vector<uint32_t>& out_point)
{
  out_poly.clear();
  out_point.clear();
  // blocks of consecutive pairs, handed out dynamically (pairs differ widely
  // in cost); each block's rows are kept apart and concatenated in block
  // order, which keeps the output order
  size_t const kBlock  = 64;
  size_t const nblocks = (np + kBlock - 1) / kBlock;
  std::vector<std::vector<uint32_t>> tp(nblocks), tq(nblocks);
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t b = 0; b < nblocks; ++b) {
    size_t const lo = b * kBlock, hi = std::min(np, lo + kBlock);
    std::vector<uint32_t>& bp = tp[b];
    std::vector<uint32_t>& bq = tq[b];
    for (size_t k = lo; k < hi; ++k) {
      uint32_t const poly = pair_poly[k];
      uint32_t const quad = pair_quad[k];
      uint64_t const len  = length[quad];
      for (uint64_t lp = 0; lp < len; ++lp) {
        uint64_t const pos = static_cast<uint64_t>(offset[quad]) + lp;
        if (pos >= npi) continue;
        uint32_t const pi = point_indices[pos];
        if (is_point_in_polygon<T, Off>(x[pi], y[pi], ring_offsets, poly_offsets[poly],
                                        poly_offsets[poly + 1], vx, vy)) {
          bp.push_back(poly);
          bq.push_back(static_cast<uint32_t>(pos));
        }
      }
    }
  }
  size_t total = 0;
  for (auto const& v : tp) total += v.size();
  out_poly.reserve(total);
  out_point.reserve(total);
  for (size_t b = 0; b < nblocks; ++b) {
    out_poly.insert(out_poly.end(), tp[b].begin(), tp[b].end());
    out_point.insert(out_point.end(), tq[b].begin(), tq[b].end());
  }
}

// detail/algorithm/point_linestring_distance.cuh:26-51; dot() is
// geometry/vec_2d.hpp:167 (a.x*b.x + a.y*b.y, contracted to one FMA).
template <typename T>
inline T dot2(T ax, T ay, T bx, T by)
{
  return fma_t(ax, bx, ay * by);
}
template <typename T>
T point_linestring_distance(T px, T py, T const* lx, T const* ly, int64_t v0, int64_t v1)
{
  T ds = std::numeric_limits<T>::max();
  for (int64_t s = v0; s + 1 < v1; ++s) {
    T const ax = lx[s], ay = ly[s], bx = lx[s + 1], by = ly[s + 1];
    T const v1px = px - ax, v1py = py - ay;
    T const v2px = px - bx, v2py = py - by;
    T const d0   = dot2(v1px, v1py, v1px, v1py);
    T const d1   = dot2(v2px, v2py, v2px, v2py);
    T const ex = bx - ax, ey = by - ay;
    T const d2   = dot2(ex, ey, ex, ey);
    T const d3   = dot2(px - ax, py - ay, ex, ey);
    T const r    = d3 * d3 / d2;
    T const d    = (d3 <= 0 || r >= d2) ? std::fmin(d0, d1) : d0 - r;
    ds           = std::fmin(ds, d);
  }
  return std::sqrt(ds);
}

// quadtree_point_to_nearest_linestring.cuh:143-312 — candidates of one
// quadrant are enumerated point-major (the transposed order at :63-89), the
// per-point minimum uses the reduction rule at :279-294 and results are
// scattered to the point's position.  Rows without a candidate keep
// (position, 0xFFFFFFFF, 0).
template <typename T>
void quadtree_point_to_nearest_linestring(uint32_t const* pair_ls, uint32_t const* pair_quad,
                                          size_t np, uint32_t const* length,
                                          uint32_t const* offset, uint32_t const* point_indices,
                                          size_t npi, T const* x, T const* y,
                                          uint32_t const* ls_offsets, T const* lx, T const* ly,
                                          uint32_t* out_point, uint32_t* out_ls, T* out_dist)
{
  for (size_t i = 0; i < npi; ++i) {
    out_point[i] = static_cast<uint32_t>(i);
    out_ls[i]    = 0xFFFFFFFFu;
    out_dist[i]  = T{0};
  }
  // groups of consecutive pairs that share a quadrant offset
  std::vector<size_t> gstart;
  for (size_t k = 0; k < np; ++k)
    if (k == 0 || offset[pair_quad[k]] != offset[pair_quad[k - 1]]) gstart.push_back(k);
  gstart.push_back(np);
  size_t const ng = gstart.size() - 1;
#pragma omp parallel for schedule(dynamic, 4)
  for (size_t g = 0; g < ng; ++g) {
    size_t const k0    = gstart[g], k1 = gstart[g + 1];
    uint32_t const q   = pair_quad[k0];
    uint64_t const len = length[q];
    for (uint64_t lp = 0; lp < len; ++lp) {
      uint64_t const pos = static_cast<uint64_t>(offset[q]) + lp;
      if (pos >= npi) continue;
      uint32_t const pi = point_indices[pos];
      bool have         = false;
      uint32_t best_id  = 0;
      T best_d          = 0;
      for (size_t k = k0; k < k1; ++k) {
        uint32_t const lid = pair_ls[k];
        T const d =
          point_linestring_distance<T>(x[pi], y[pi], lx, ly, ls_offsets[lid], ls_offsets[lid + 1]);
        if (!have) {
          have    = true;
          best_id = lid;
          best_d  = d;
          continue;
        }
        // lhs = running value, rhs = new candidate
        bool take_rhs;
        if (best_d == T{0}) {
          take_rhs = true;
        } else if (d == T{0}) {
          take_rhs = false;
        } else if (best_d == d) {
          take_rhs = !(best_id < lid);
        } else {
          take_rhs = !(best_d < d);
        }
        if (take_rhs) {
          best_id = lid;
          best_d  = d;
        }
      }
      if (have) {
        out_point[pos] = static_cast<uint32_t>(pos);
        out_ls[pos]    = best_id;
        out_dist[pos]  = best_d;
      }
    }
  }
}

// detail/utility/linestring.cuh:56-75 — squared distance from c to segment
// ab and the nearest point on it.  The reference's build contracts each dot
// product x1*x2 + y1*y2 into fma(x1, x2, y1*y2) and a + t*ab into
// fma(t, ab, a); the oracle writes those fmas out.
template <typename T>
T segment_nearest(T cx, T cy, T ax, T ay, T bx, T by, T& nx, T& ny)
{
  T const abx = bx - ax, aby = by - ay;
  T const acx = cx - ax, acy = cy - ay;
  T const l2  = std::fma(abx, abx, aby * aby);
  if (float_equal(l2, T{0})) {
    nx = ax;
    ny = ay;
    return std::fma(acx, acx, acy * acy);
  }
  T const r   = std::fma(acx, abx, acy * aby);
  T const bcx = cx - bx, bcy = cy - by;
  if (r <= 0 || r >= l2) {
    T const dac = std::fma(acx, acx, acy * acy);
    T const dbc = std::fma(bcx, bcx, bcy * bcy);
    if (dac < dbc) {
      nx = ax;
      ny = ay;
      return dac;
    }
    nx = bx;
    ny = by;
    return dbc;
  }
  T const t   = r / l2;
  T const px  = std::fma(t, abx, ax);
  T const py  = std::fma(t, aby, ay);
  T const pcx = cx - px, pcy = cy - py;
  nx          = px;
  ny          = py;
  return std::fma(pcx, pcx, pcy * pcy);
}

// detail/kernel/pairwise_distance.cuh:94-131 with
// detail/distance/point_linestring_distance.cuh:37-60: per segment the
// smallest squared distance over the multipoint (device min = fmin, from
// T max), its square root, and the smallest of those over the segments
// (from T max).  pgo / lgo: geometry offsets (null: one point / one
// linestring per pair); lpo: linestring part offsets.
template <typename T>
void pairwise_point_linestring_distance(size_t n, uint32_t const* pgo, T const* x, T const* y,
                                        uint32_t const* lgo, uint32_t const* lpo, size_t nparts,
                                        T const* lx, T const* ly, T* out)
{
  T const big = std::numeric_limits<T>::max();
  for (size_t g = 0; g < n; ++g) {
    size_t const p0 = pgo ? pgo[g] : g, p1 = pgo ? pgo[g + 1] : g + 1;
    // parts named beyond the last part offset do not exist (the reference
    // maps each vertex to its part, pairwise_distance.cuh:115-121)
    size_t const l1 = std::min<size_t>(lgo ? lgo[g + 1] : g + 1, nparts);
    size_t const l0 = std::min<size_t>(lgo ? lgo[g] : g, l1);
    T d = big;
    for (size_t part = l0; part < l1; ++part) {
      for (size_t v = lpo[part]; v + 1 < lpo[part + 1]; ++v) {
        T m = big;
        for (size_t p = p0; p < p1; ++p) {
          T nx, ny;
          m = std::fmin(m, segment_nearest<T>(x[p], y[p], lx[v], ly[v], lx[v + 1], ly[v + 1],
                                              nx, ny));
        }
        d = std::fmin(d, std::sqrt(m));
      }
    }
    out[g] = d;
  }
}

// detail/point_linestring_nearest_points.cuh:55-110: the first strictly
// smaller squared distance over (point, part, segment) in order; ids local
// to the pair.  Pairs without a segment keep (0, 0, 0, (0, 0)).
template <typename T>
void pairwise_point_linestring_nearest_points(size_t n, uint32_t const* pgo, T const* x,
                                              T const* y, uint32_t const* lgo,
                                              uint32_t const* lpo, size_t nparts, T const* lx,
                                              T const* ly, int32_t* opt, int32_t* ols,
                                              int32_t* oseg, T* oxy)
{
  for (size_t g = 0; g < n; ++g) {
    size_t const p0 = pgo ? pgo[g] : g, p1 = pgo ? pgo[g + 1] : g + 1;
    size_t const l1 = std::min<size_t>(lgo ? lgo[g + 1] : g + 1, nparts);
    size_t const l0 = std::min<size_t>(lgo ? lgo[g] : g, l1);
    T best           = std::numeric_limits<T>::max();
    int32_t bp = 0, bl = 0, bs = 0;
    T bx = 0, by = 0;
    for (size_t p = p0; p < p1; ++p) {
      for (size_t part = l0; part < l1; ++part) {
        size_t const s0 = lpo[part];
        for (size_t v = s0; v + 1 < lpo[part + 1]; ++v) {
          T nx, ny;
          T const d =
            segment_nearest<T>(x[p], y[p], lx[v], ly[v], lx[v + 1], ly[v + 1], nx, ny);
          if (d < best) {
            best = d;
            bp   = static_cast<int32_t>(p - p0);
            bl   = static_cast<int32_t>(part - l0);
            bs   = static_cast<int32_t>(v - s0);
            bx   = nx;
            by   = ny;
          }
        }
      }
    }
    opt[g]         = bp;
    ols[g]         = bl;
    oseg[g]        = bs;
    oxy[2 * g]     = bx;
    oxy[2 * g + 1] = by;
  }
}

template <typename T>
void* dup_vec(std::vector<T> const& v)
{
  if (v.empty()) return nullptr;
  void* p = std::malloc(v.size() * sizeof(T));
  std::memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

}  // namespace

// ---------------------------------------------------------------------------
// C interface used by the tests and the CPU baseline (host pointers).
// dtype: 0 = float32, 1 = float64.  Arrays returned through `void**` are
// malloc'd; release them with oracle_free.
// ---------------------------------------------------------------------------
extern "C" {

const char* oracle_last_error() { return g_last_error.c_str(); }
void oracle_free(void* p) { std::free(p); }

int oracle_num_threads()
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void oracle_set_num_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int oracle_quadtree_on_points(void const* x, void const* y, size_t n, int dtype, double x_min,
                              double x_max, double y_min, double y_max, double scale,
                              int max_depth, int32_t max_size, void** point_indices,
                              void** key, void** level, void** internal, void** length,
                              void** offset, size_t* num_nodes)
{
  Tree t;
  if (dtype == 1) {
    t = quadtree_on_points<double>(static_cast<double const*>(x), static_cast<double const*>(y), n,
                                   x_min, x_max, y_min, y_max, scale, max_depth, max_size);
  } else {
    t = quadtree_on_points<float>(static_cast<float const*>(x), static_cast<float const*>(y), n,
                                  static_cast<float>(x_min), static_cast<float>(x_max),
                                  static_cast<float>(y_min), static_cast<float>(y_max),
                                  static_cast<float>(scale), max_depth, max_size);
  }
  *point_indices = dup_vec(t.point_indices);
  *key           = dup_vec(t.key);
  *level         = dup_vec(t.level);
  *internal      = dup_vec(t.is_internal);
  *length        = dup_vec(t.length);
  *offset        = dup_vec(t.offset);
  *num_nodes     = t.key.size();
  return 0;
}

// Polygon boxes: polygon p owns rings [poly_offsets[p], poly_offsets[p+1]);
// ring r owns vertices [ring_offsets[r], ring_offsets[r+1]).
int oracle_polygon_bounding_boxes(uint32_t const* poly_offsets, size_t n_poly_offsets,
                                  uint32_t const* ring_offsets, size_t n_ring_offsets,
                                  void const* x, void const* y, size_t nv, int dtype,
                                  double expansion_radius, void* ominx, void* ominy, void* omaxx,
                                  void* omaxy)
{
  (void)n_ring_offsets;
  (void)nv;
  size_t const np = n_poly_offsets ? n_poly_offsets - 1 : 0;
  std::vector<int64_t> vb(np), ve(np);
  for (size_t p = 0; p < np; ++p) {
    vb[p] = ring_offsets[poly_offsets[p]];
    ve[p] = ring_offsets[poly_offsets[p + 1]];
  }
  if (dtype == 1)
    bounding_boxes<double>(vb, ve, static_cast<double const*>(x), static_cast<double const*>(y),
                           expansion_radius, static_cast<double*>(ominx),
                           static_cast<double*>(ominy), static_cast<double*>(omaxx),
                           static_cast<double*>(omaxy));
  else
    bounding_boxes<float>(vb, ve, static_cast<float const*>(x), static_cast<float const*>(y),
                          static_cast<float>(expansion_radius), static_cast<float*>(ominx),
                          static_cast<float*>(ominy), static_cast<float*>(omaxx),
                          static_cast<float*>(omaxy));
  return 0;
}

int oracle_linestring_bounding_boxes(uint32_t const* ls_offsets, size_t n_ls_offsets,
                                     void const* x, void const* y, size_t nv, int dtype,
                                     double expansion_radius, void* ominx, void* ominy,
                                     void* omaxx, void* omaxy)
{
  (void)nv;
  size_t const nl = n_ls_offsets ? n_ls_offsets - 1 : 0;
  std::vector<int64_t> vb(nl), ve(nl);
  for (size_t p = 0; p < nl; ++p) {
    vb[p] = ls_offsets[p];
    ve[p] = ls_offsets[p + 1];
  }
  if (dtype == 1)
    bounding_boxes<double>(vb, ve, static_cast<double const*>(x), static_cast<double const*>(y),
                           expansion_radius, static_cast<double*>(ominx),
                           static_cast<double*>(ominy), static_cast<double*>(omaxx),
                           static_cast<double*>(omaxy));
  else
    bounding_boxes<float>(vb, ve, static_cast<float const*>(x), static_cast<float const*>(y),
                          static_cast<float>(expansion_radius), static_cast<float*>(ominx),
                          static_cast<float*>(ominy), static_cast<float*>(omaxx),
                          static_cast<float*>(omaxy));
  return 0;
}

int oracle_join_quadtree_and_bounding_boxes(uint32_t const* key, uint8_t const* level,
                                            uint8_t const* internal, uint32_t const* length,
                                            uint32_t const* offset, size_t nq, void const* bminx,
                                            void const* bminy, void const* bmaxx,
                                            void const* bmaxy, size_t nb, int dtype,
                                            double x_min, double x_max, double y_min,
                                            double y_max, double scale, int max_depth,
                                            void** out_bbox, void** out_quad, size_t* n_out)
{
  std::vector<uint32_t> ob, oq;
  double const vminx = std::min(x_min, x_max), vminy = std::min(y_min, y_max);
  if (nq > 0 && nb > 0) {
    if (dtype == 1)
      join_quadtree_and_bboxes<double>(key, level, internal, length, offset, nq,
                                       static_cast<double const*>(bminx),
                                       static_cast<double const*>(bminy),
                                       static_cast<double const*>(bmaxx),
                                       static_cast<double const*>(bmaxy), nb, vminx, vminy, scale,
                                       max_depth, ob, oq);
    else
      join_quadtree_and_bboxes<float>(
        key, level, internal, length, offset, nq, static_cast<float const*>(bminx),
        static_cast<float const*>(bminy), static_cast<float const*>(bmaxx),
        static_cast<float const*>(bmaxy), nb, static_cast<float>(vminx),
        static_cast<float>(vminy), static_cast<float>(scale), max_depth, ob, oq);
  }
  *out_bbox = dup_vec(ob);
  *out_quad = dup_vec(oq);
  *n_out    = ob.size();
  return 0;
}

int oracle_quadtree_point_in_polygon(uint32_t const* pair_poly, uint32_t const* pair_quad,
                                     size_t np, uint32_t const* length, uint32_t const* offset,
                                     uint32_t const* point_indices, size_t npi, void const* x,
                                     void const* y, uint32_t const* poly_offsets,
                                     uint32_t const* ring_offsets, void const* vx, void const* vy,
                                     int dtype, void** out_poly, void** out_point, size_t* n_out)
{
  std::vector<uint32_t> op, oq;
  if (dtype == 1)
    quadtree_point_in_polygon<double, uint32_t>(
      pair_poly, pair_quad, np, length, offset, point_indices, npi, static_cast<double const*>(x),
      static_cast<double const*>(y), poly_offsets, ring_offsets, static_cast<double const*>(vx),
      static_cast<double const*>(vy), op, oq);
  else
    quadtree_point_in_polygon<float, uint32_t>(
      pair_poly, pair_quad, np, length, offset, point_indices, npi, static_cast<float const*>(x),
      static_cast<float const*>(y), poly_offsets, ring_offsets, static_cast<float const*>(vx),
      static_cast<float const*>(vy), op, oq);
  *out_poly  = dup_vec(op);
  *out_point = dup_vec(oq);
  *n_out     = op.size();
  return 0;
}

// Single (point, polygon) test, exposed for boundary-rule known-answer tests.
int oracle_is_point_in_polygon(double px, double py, uint32_t const* ring_offsets,
                               int64_t ring_begin, int64_t ring_end, double const* vx,
                               double const* vy)
{
  return is_point_in_polygon<double, uint32_t>(px, py, ring_offsets, ring_begin, ring_end, vx, vy)
           ? 1
           : 0;
}

// detail/point_in_polygon.cuh:41-66 (pip_functor) — bit p of out[i] is point i
// inside polygon p, for at most 31 polygons; detail/point_in_polygon.cuh:
// 112-140 — pairwise form, point i against polygon i.
int oracle_point_in_polygon(void const* x, void const* y, size_t n, uint32_t const* poly_offsets,
                            size_t npoly, uint32_t const* ring_offsets, void const* vx,
                            void const* vy, int dtype, int pairwise, void* out)
{
  for (size_t i = 0; i < n; ++i) {
    size_t const p0 = pairwise ? i : 0;
    size_t const p1 = pairwise ? i + 1 : npoly;
    int32_t mask    = 0;
    for (size_t p = p0; p < p1; ++p) {
      bool hit;
      if (dtype == 1)
        hit = is_point_in_polygon<double, uint32_t>(
          static_cast<double const*>(x)[i], static_cast<double const*>(y)[i], ring_offsets,
          poly_offsets[p], poly_offsets[p + 1], static_cast<double const*>(vx),
          static_cast<double const*>(vy));
      else
        hit = is_point_in_polygon<float, uint32_t>(
          static_cast<float const*>(x)[i], static_cast<float const*>(y)[i], ring_offsets,
          poly_offsets[p], poly_offsets[p + 1], static_cast<float const*>(vx),
          static_cast<float const*>(vy));
      if (hit) mask |= pairwise ? 1 : (1 << p);
    }
    if (pairwise)
      static_cast<uint8_t*>(out)[i] = static_cast<uint8_t>(mask);
    else
      static_cast<int32_t*>(out)[i] = mask;
  }
  return 0;
}

int oracle_pairwise_point_linestring(size_t n, uint32_t const* pgo, void const* x,
                                     void const* y, uint32_t const* lgo, uint32_t const* lpo,
                                     size_t nparts, void const* lx, void const* ly, int dtype,
                                     void* out_dist, int32_t* opt, int32_t* ols, int32_t* oseg,
                                     void* oxy)
{
  if (dtype == 1) {
    auto X = static_cast<double const*>(x), Y = static_cast<double const*>(y);
    auto LX = static_cast<double const*>(lx), LY = static_cast<double const*>(ly);
    pairwise_point_linestring_distance<double>(n, pgo, X, Y, lgo, lpo, nparts, LX, LY,
                                               static_cast<double*>(out_dist));
    pairwise_point_linestring_nearest_points<double>(n, pgo, X, Y, lgo, lpo, nparts, LX, LY,
                                                     opt, ols, oseg, static_cast<double*>(oxy));
  } else {
    auto X = static_cast<float const*>(x), Y = static_cast<float const*>(y);
    auto LX = static_cast<float const*>(lx), LY = static_cast<float const*>(ly);
    pairwise_point_linestring_distance<float>(n, pgo, X, Y, lgo, lpo, nparts, LX, LY,
                                              static_cast<float*>(out_dist));
    pairwise_point_linestring_nearest_points<float>(n, pgo, X, Y, lgo, lpo, nparts, LX, LY,
                                                    opt, ols, oseg, static_cast<float*>(oxy));
  }
  return 0;
}

int oracle_quadtree_point_to_nearest_linestring(uint32_t const* pair_ls,
                                                uint32_t const* pair_quad, size_t np,
                                                uint32_t const* length, uint32_t const* offset,
                                                uint32_t const* point_indices, size_t npi,
                                                void const* x, void const* y,
                                                uint32_t const* ls_offsets, void const* lx,
                                                void const* ly, int dtype, uint32_t* out_point,
                                                uint32_t* out_ls, void* out_dist)
{
  if (dtype == 1)
    quadtree_point_to_nearest_linestring<double>(
      pair_ls, pair_quad, np, length, offset, point_indices, npi, static_cast<double const*>(x),
      static_cast<double const*>(y), ls_offsets, static_cast<double const*>(lx),
      static_cast<double const*>(ly), out_point, out_ls, static_cast<double*>(out_dist));
  else
    quadtree_point_to_nearest_linestring<float>(
      pair_ls, pair_quad, np, length, offset, point_indices, npi, static_cast<float const*>(x),
      static_cast<float const*>(y), ls_offsets, static_cast<float const*>(lx),
      static_cast<float const*>(ly), out_point, out_ls, static_cast<float*>(out_dist));
  return 0;
}

}  // extern "C"
