// The quadrant / bounding-box join kernel, shared by the single-tree join
// and the batched form.  Each box walks one tree, described by a BoxTree
// that a lookup functor returns for the box: the single-tree join returns
// the same tree for every box, the batched form the tree of the box's
// instance inside the concatenated node arrays.
//
// Reference: cpp/include/cuspatial/detail/join/quadtree_bbox_filtering.cuh:
// 35-188, intersection.cuh:79-136 and traversal.cuh:57-145.
#pragma once

#include "common.cuh"
#include "scan.cuh"

namespace cspt {
namespace {

constexpr int kStack = 64;

struct TreeView {
  uint32_t const* key;
  uint8_t const* level;
  uint8_t const* internal;
  uint32_t const* length;
  uint32_t const* offset;
  size_t nq;
};

// The tree one box walks: nodes [base, base + nq) of the node arrays, whose
// child offsets count from base; its leaf offsets plus pt_base are the
// positions in the (concatenated) point order.
template <typename T>
struct BoxTree {
  uint32_t base;
  uint32_t nq;
  uint32_t L0;  // level-0 nodes
  uint32_t pt_base;
  T vminx, vminy, scale;
  int max_depth;
};

// every box walks the same tree
template <typename T>
struct OneTree {
  uint32_t const* L0p;
  uint32_t nq;
  T vminx, vminy, scale;
  int max_depth;
  __device__ BoxTree<T> operator()(size_t) const
  {
    return BoxTree<T>{0u, nq, *L0p, 0u, vminx, vminy, scale, max_depth};
  }
};

// intersection.cuh:104-128; the node corners are v_min + k * level_scale,
// which the reference's build contracts into one FMA.
template <typename T>
__device__ inline int classify(TreeView const& t, uint32_t node, T bminx, T bminy, T bmaxx,
                               T bmaxy, T vminx, T vminy, T scale, int max_depth)
{
  uint32_t const key = t.key[node];
  int const lev      = t.level[node];
  int const sh       = max_depth - 1 - lev;
  if (sh < 0) return 2;
  T const kx  = static_cast<T>(gather16(key));
  T const ky  = static_cast<T>(gather16(key >> 1));
  T const ls  = scale * static_cast<T>(1 << sh);
  T const x0  = fma_rn(kx + T{0}, ls, vminx);
  T const y0  = fma_rn(ky + T{0}, ls, vminy);
  T const x1  = fma_rn(kx + T{1}, ls, vminx);
  T const y1  = fma_rn(ky + T{1}, ls, vminy);
  if (x0 > bmaxx || x1 < bminx || y0 > bmaxy || y1 < bminy) return 2;
  return t.internal[node] ? 1 : 0;
}

// float32 pre-classification of a node for float64 trees.  The reference's
// corner fl64(fma(k, s 2^sh, v_min)) and the float32 fmaf(k, fl32(s) 2^sh,
// fl32(v_min)) both lie within u32 (|k s 2^sh| + |v_min| + |corner|) of the
// exact value, so within eps = 2^-20 M of each other for
// M = max(|v_min|) + s 2^(max_depth+1); a box side rounded to float32 lies
// within its own margin eb.  Each of the reference's four comparisons is
// decided when the float32 values are farther apart than both margins (and
// the float32 rounding of the compared sums, covered by the factor 2 in
// eps); otherwise the float64 expression decides.
struct FloatBox {
  float x0, y0, x1, y1;      // box sides, rounded to float32
  float ex0, ey0, ex1, ey1;  // their margins
  float vx, vy, s, eps;      // tree origin and scale in float32, corner margin
};

__device__ inline float side_margin(float v)
{
  return fmaf(fabsf(v), 4.76837158203125e-07f, 1.17549435e-38f);  // 2^-21 |v|
}

template <typename T>
__device__ inline FloatBox float_box(T x0, T y0, T x1, T y1, T vminx, T vminy, T scale,
                                     int max_depth)
{
  FloatBox f;
  f.x0  = static_cast<float>(x0);
  f.y0  = static_cast<float>(y0);
  f.x1  = static_cast<float>(x1);
  f.y1  = static_cast<float>(y1);
  f.ex0 = side_margin(f.x0);
  f.ey0 = side_margin(f.y0);
  f.ex1 = side_margin(f.x1);
  f.ey1 = side_margin(f.y1);
  f.vx  = static_cast<float>(vminx);
  f.vy  = static_cast<float>(vminy);
  f.s   = static_cast<float>(scale);
  float const m = fmaxf(fabsf(f.vx), fabsf(f.vy)) + ldexpf(f.s, max_depth + 1);
  f.eps = 9.5367431640625e-07f * m;  // 2^-20 M (NaN or inf: nothing is decided)
  return f;
}

// 2 disjoint, 1 internal and overlapping, 0 overlapping leaf; -1 undecided
__device__ inline int classify_float(uint32_t key, int sh, FloatBox const& f)
{
  float const kx  = static_cast<float>(gather16(key));
  float const ky  = static_cast<float>(gather16(key >> 1));
  float const ls  = ldexpf(f.s, sh);
  float const ax0 = fmaf(kx, ls, f.vx), ax1 = fmaf(kx + 1.0f, ls, f.vx);
  float const ay0 = fmaf(ky, ls, f.vy), ay1 = fmaf(ky + 1.0f, ls, f.vy);
  float const e   = f.eps;
  // intersection.cuh:123-126: x0 > bmaxx || x1 < bminx || y0 > bmaxy || y1 < bminy
  if (ax0 - e > f.x1 + f.ex1 || ax1 + e < f.x0 - f.ex0 || ay0 - e > f.y1 + f.ey1 ||
      ay1 + e < f.y0 - f.ey0)
    return 2;
  if (ax0 + e < f.x1 - f.ex1 && ax1 - e > f.x0 + f.ex0 && ay0 + e < f.y1 - f.ey1 &&
      ay1 - e > f.y0 + f.ey0)
    return 1;  // overlapping: internal or leaf decided by the caller
  return -1;
}

template <typename T>
__device__ inline int classify_filtered(TreeView const& t, uint32_t node, FloatBox const& f,
                                        T bminx, T bminy, T bmaxx, T bmaxy, T vminx, T vminy,
                                        T scale, int max_depth)
{
  if constexpr (std::is_same<T, double>::value) {
    uint32_t const key = t.key[node];
    int const sh       = max_depth - 1 - t.level[node];
    if (sh < 0) return 2;
    int const c = classify_float(key, sh, f);
    if (c == 2) return 2;
    if (c == 1) return t.internal[node] ? 1 : 0;
  }
  return classify<T>(t, node, bminx, bminy, bmaxx, bmaxy, vminx, vminy, scale, max_depth);
}

// Walks the tree for box b; calls emit(node) for every intersecting leaf.
// Returns false when the private stack would overflow (malformed tree).
template <typename T, typename Emit>
__device__ inline bool walk(TreeView const& t, BoxTree<T> const& bt, T bminx, T bminy, T bmaxx,
                            T bmaxy, Emit&& emit)
{
  uint32_t stack[kStack];
  int sp = 0;
  for (uint32_t seed = 0; seed < bt.L0; ++seed) {
    stack[sp++] = seed << 4;  // tree-local node index << 4 | depth
    while (sp > 0) {
      uint32_t const top  = stack[--sp];
      uint32_t const node = top >> 4;
      int const depth     = top & 15;
      if (node >= bt.nq) return false;
      uint32_t const g = bt.base + node;
      int const c      = classify<T>(t, g, bminx, bminy, bmaxx, bmaxy, bt.vminx, bt.vminy,
                                bt.scale, bt.max_depth);
      if (c == 0) {
        emit(g);
      } else if (c == 1 && depth + 1 < bt.max_depth) {
        uint32_t const first = t.offset[g];
        uint32_t const len   = t.length[g];
        if (sp + static_cast<int>(len) > kStack) return false;
        for (uint32_t k = len; k-- > 0;) stack[sp++] = ((first + k) << 4) | (depth + 1);
      }
    }
  }
  return true;
}

constexpr int kJoinWarps = 4;       // warps per block
constexpr int kWarpStack = 2048;    // stack entries per warp (shared memory)

// Where the count pass appends each (node, box) it finds, in any order, while
// fewer than `cap` have been found (`n` counts them all, also past cap).
struct JoinAppend {
  uint32_t* node;
  uint32_t* box;
  unsigned long long* n;
  size_t cap;
};

// One warp per box.  Each round pops up to 32 entries (node << 4 | depth)
// from the warp's shared stack, one per lane, classifies them, counts or
// writes the leaves with a ballot, and pushes the children of internal nodes
// (warp scan of the child counts).  If the stack would overflow the warp
// restarts the box on lane 0 with the private-stack walk above.  Seeds (the
// level-0 nodes) are fed 32 at a time whenever the stack runs empty.
template <typename T, bool Write, typename Trees>
__global__ void __launch_bounds__(kJoinWarps * 32)
  join_warp_kernel(TreeView t, Trees trees, T const* __restrict__ bminx,
                   T const* __restrict__ bminy, T const* __restrict__ bmaxx,
                   T const* __restrict__ bmaxy, size_t nb, uint32_t* __restrict__ counts,
                   uint32_t* __restrict__ maxkey,
                   uint32_t const* __restrict__ pos, uint32_t* __restrict__ okey,
                   uint32_t* __restrict__ onode, uint32_t* __restrict__ obox,
                   int* __restrict__ error, JoinAppend app = JoinAppend{nullptr, nullptr, nullptr, 0})
{
  __shared__ uint32_t stack_s[kJoinWarps][kWarpStack];
  uint32_t* stack      = stack_s[threadIdx.x >> 5];
  int const lane       = threadIdx.x & 31;
  unsigned const lt    = (1u << lane) - 1u;
  size_t const nwarps  = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t local_max   = 0;
  for (size_t b = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; b < nb;
       b += nwarps) {
    T const x0 = bminx[b], y0 = bminy[b], x1 = bmaxx[b], y1 = bmaxy[b];
    BoxTree<T> const bt = trees(b);
    FloatBox const fbox = float_box<T>(x0, y0, x1, y1, bt.vminx, bt.vminy, bt.scale,
                                       bt.max_depth);
    uint32_t const L0   = bt.L0;
    uint32_t found      = 0;
    uint32_t p     = Write ? pos[b] : 0u;
    int sp         = 0;
    uint32_t seed  = 0;
    bool overflow  = false;
    bool bad       = false;
    while (sp > 0 || seed < L0) {
      uint32_t e     = 0;
      bool have      = false;
      int const take = sp > 0 ? (sp < 32 ? sp : 32) : 0;
      if (take > 0) {
        if (lane < take) {
          e    = stack[sp - 1 - lane];
          have = true;
        }
        sp -= take;
      } else {
        uint32_t const s = seed + lane;
        if (s < L0) {
          e    = s << 4;
          have = true;
        }
        seed += 32;
      }
      __syncwarp();
      uint32_t const node = e >> 4;
      int const depth     = e & 15;
      int c               = 2;
      uint32_t const g    = bt.base + node;
      if (have) {
        if (node >= bt.nq) {
          bad = true;
        } else {
          c = classify_filtered<T>(t, g, fbox, x0, y0, x1, y1, bt.vminx, bt.vminy, bt.scale,
                                   bt.max_depth);
        }
      }
      unsigned const leaves = __ballot_sync(0xFFFFFFFFu, c == 0);
      if (!Write && app.n && leaves) {
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(app.n, static_cast<unsigned long long>(__popc(leaves)));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        if (c == 0) {
          unsigned long long const d = at + __popc(leaves & lt);
          if (d < app.cap) {
            app.node[d] = g;
            app.box[d]  = static_cast<uint32_t>(b);
          }
        }
      }
      if (c == 0) {
        uint32_t const key = bt.pt_base + t.offset[g];
        if (Write) {
          uint32_t const d = p + __popc(leaves & lt);
          okey[d]          = key;
          onode[d]         = g;
          obox[d]          = static_cast<uint32_t>(b);
        } else {
          local_max = key > local_max ? key : local_max;
        }
      }
      p += __popc(leaves);
      found += __popc(leaves);
      uint32_t nchild = 0, first = 0;
      if (c == 1 && depth + 1 < bt.max_depth) {
        first  = t.offset[g];
        nchild = t.length[g];
      }
      uint32_t const incl  = warp_inclusive_scan(nchild);
      uint32_t const total = __shfl_sync(0xFFFFFFFFu, incl, 31);
      if (sp + static_cast<int>(total) > kWarpStack) {
        overflow = true;
        break;
      }
      uint32_t const at = sp + incl - nchild;
      for (uint32_t k = 0; k < nchild; ++k) stack[at + k] = ((first + k) << 4) | (depth + 1);
      sp += static_cast<int>(total);
      __syncwarp();
    }
    if (__any_sync(0xFFFFFFFFu, bad)) {
      if (lane == 0) atomicExch(error, 1);
      continue;
    }
    if (overflow) {
      // rare: restart the box serially on lane 0.  The box's pairs appended
      // so far would repeat, so the appended set is given up (its count is
      // pushed past any capacity) and the write pass runs instead.
      if (!Write && app.n && lane == 0) atomicAdd(app.n, 1ull << 62);
      if (lane == 0) {
        uint32_t q = Write ? pos[b] : 0u;
        found      = 0;
        bool const ok =
          walk<T>(t, bt, x0, y0, x1, y1, [&](uint32_t node) {
            uint32_t const key = bt.pt_base + t.offset[node];
            if (Write) {
              okey[q]  = key;
              onode[q] = node;
              obox[q]  = static_cast<uint32_t>(b);
            } else {
              local_max = key > local_max ? key : local_max;
            }
            ++q;
            ++found;
          });
        if (!ok) atomicExch(error, 1);
      }
      found = __shfl_sync(0xFFFFFFFFu, found, 0);
    }
    if (!Write && lane == 0) counts[b] = found;
  }
  if (!Write) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      uint32_t const o = __shfl_xor_sync(0xFFFFFFFFu, local_max, off);
      local_max        = o > local_max ? o : local_max;
    }
    if (lane == 0 && local_max) atomicMax(maxkey, local_max);
  }
}

__global__ void gather_pairs_kernel(uint32_t const* __restrict__ perm,
                                    uint32_t const* __restrict__ node,
                                    uint32_t const* __restrict__ box, size_t k,
                                    uint32_t* __restrict__ out_box, uint32_t* __restrict__ out_node)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < k;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t const j = perm[i];
    out_box[i]       = box[j];
    out_node[i]      = node[j];
  }
}

}  // namespace
}  // namespace cspt
