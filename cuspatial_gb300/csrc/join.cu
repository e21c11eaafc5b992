// Quadrant / bounding-box intersection join on sm_103a.
//
// Reference: cpp/include/cuspatial/detail/join/quadtree_bbox_filtering.cuh:
// 35-188 (seeds, level loop, final stable sort by leaf offset),
// intersection.cuh:79-136 (node extent and closed-interval overlap) and
// traversal.cuh:57-145 (descent to children).
//
// The reference walks all boxes level by level with a host synchronisation
// per level.  Here each thread owns one box and walks the tree depth-first
// with a private stack; a count pass sizes the output, a write pass emits
// (leaf first-point offset, node, box) in box-major order, and a stable radix
// sort by the leaf offset gives the reference's order (leaf offset, box).
// A node at traversal depth t is expanded only while t + 1 < max_depth, the
// reference's loop bound (quadtree_bbox_filtering.cuh:118).
#include "common.cuh"
#include "radix_sort.cuh"
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

// Walks the tree for box b; calls emit(node) for every intersecting leaf.
// Returns false when the private stack would overflow (malformed tree).
template <typename T, typename Emit>
__device__ inline bool walk(TreeView const& t, uint32_t L0, T bminx, T bminy, T bmaxx, T bmaxy,
                            T vminx, T vminy, T scale, int max_depth, Emit&& emit)
{
  uint32_t stack[kStack];
  int sp = 0;
  for (uint32_t seed = 0; seed < L0; ++seed) {
    stack[sp++] = seed << 4;  // node index << 4 | depth
    while (sp > 0) {
      uint32_t const top  = stack[--sp];
      uint32_t const node = top >> 4;
      int const depth     = top & 15;
      if (node >= t.nq) return false;
      int const c =
        classify<T>(t, node, bminx, bminy, bmaxx, bmaxy, vminx, vminy, scale, max_depth);
      if (c == 0) {
        emit(node);
      } else if (c == 1 && depth + 1 < max_depth) {
        uint32_t const first = t.offset[node];
        uint32_t const len   = t.length[node];
        if (sp + static_cast<int>(len) > kStack) return false;
        for (uint32_t k = len; k-- > 0;) stack[sp++] = ((first + k) << 4) | (depth + 1);
      }
    }
  }
  return true;
}

template <typename T>
__global__ void join_count_kernel(TreeView t, uint32_t const* __restrict__ L0p,
                                  T const* __restrict__ bminx, T const* __restrict__ bminy,
                                  T const* __restrict__ bmaxx, T const* __restrict__ bmaxy,
                                  size_t nb, T vminx, T vminy, T scale, int max_depth,
                                  uint32_t* __restrict__ counts, int* __restrict__ error)
{
  uint32_t const L0 = *L0p;
  for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; b < nb;
       b += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t c   = 0;
    bool const ok = walk<T>(t, L0, bminx[b], bminy[b], bmaxx[b], bmaxy[b], vminx, vminy, scale,
                            max_depth, [&](uint32_t) { ++c; });
    if (!ok) atomicExch(error, 1);
    counts[b] = c;
  }
}

template <typename T>
__global__ void join_write_kernel(TreeView t, uint32_t const* __restrict__ L0p,
                                  T const* __restrict__ bminx, T const* __restrict__ bminy,
                                  T const* __restrict__ bmaxx, T const* __restrict__ bmaxy,
                                  size_t nb, T vminx, T vminy, T scale, int max_depth,
                                  uint32_t const* __restrict__ pos, uint32_t* __restrict__ okey,
                                  uint32_t* __restrict__ onode, uint32_t* __restrict__ obox)
{
  uint32_t const L0 = *L0p;
  for (size_t b = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; b < nb;
       b += static_cast<size_t>(gridDim.x) * blockDim.x) {
    uint32_t p = pos[b];
    walk<T>(t, L0, bminx[b], bminy[b], bmaxx[b], bmaxy[b], vminx, vminy, scale, max_depth,
            [&](uint32_t node) {
              okey[p]  = t.offset[node];
              onode[p] = node;
              obox[p]  = static_cast<uint32_t>(b);
              ++p;
            });
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

template <typename T>
void run(cspt_quadtree const* tree, T const* bminx, T const* bminy, T const* bmaxx,
         T const* bmaxy, size_t nb, T vminx, T vminy, T scale, int max_depth,
         Allocator const& alloc, uint32_t** out_box, uint32_t** out_node, size_t* out_n)
{
  cudaStream_t const s = alloc.stream();
  TreeView tv{tree->key, tree->level, tree->is_internal_node, tree->length, tree->offset,
              tree->num_nodes};
  // seeds: the number of level-0 nodes (quadtree_bbox_filtering.cuh:53-56)
  Buffer<uint32_t> L0(alloc, 1);
  uint8_t const* lev = tree->level;
  scan_apply<uint32_t>([lev] __device__(size_t i) { return lev[i] == 0 ? 1u : 0u; },
                       [] __device__(size_t, uint32_t, uint32_t) {}, tree->num_nodes, L0.data(),
                       alloc);
  Buffer<uint32_t> counts(alloc, nb + 1);
  Buffer<int> err(alloc, 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(err.data(), 0, sizeof(int), s));
  unsigned const blk = 128;
  unsigned const grd = grid_for(nb, blk, 152u * 64u);
  {
    KernelTimer timer("join_count", s);
    join_count_kernel<T><<<grd, blk, 0, s>>>(tv, L0.data(), bminx, bminy, bmaxx, bmaxy, nb,
                                             vminx, vminy, scale, max_depth, counts.data(),
                                             err.data());
    CSPT_CHECK_LAUNCH();
  }
  exclusive_scan<uint32_t>(counts.data(), counts.data(), nb, counts.data() + nb, alloc);
  size_t const k = read_back(counts.data() + nb, s);
  CSPT_EXPECTS(read_back(err.data(), s) == 0,
               "quadtree is malformed: a node has more children than a quadtree allows");
  *out_n = k;
  if (k == 0) return;
  Buffer<uint32_t> key(alloc, k), key_alt(alloc, k), node(alloc, k), box(alloc, k),
    perm(alloc, k), perm_alt(alloc, k);
  {
    KernelTimer timer("join_write", s);
    join_write_kernel<T><<<grd, blk, 0, s>>>(tv, L0.data(), bminx, bminy, bmaxx, bmaxy, nb,
                                             vminx, vminy, scale, max_depth, counts.data(),
                                             key.data(), node.data(), box.data());
    CSPT_CHECK_LAUNCH();
  }
  bool const alt = radix_sort_pairs<uint32_t>(key.data(), perm.data(), key_alt.data(),
                                              perm_alt.data(), k, 0, 32, true, alloc);
  Buffer<uint32_t> ob(alloc, k), on(alloc, k);
  gather_pairs_kernel<<<grid_for(k, 256, 152u * 16u), 256, 0, s>>>(
    alt ? perm_alt.data() : perm.data(), node.data(), box.data(), k, ob.data(), on.data());
  CSPT_CHECK_LAUNCH();
  *out_box  = ob.release();
  *out_node = on.release();
}

}  // namespace

void join_quadtree_and_bounding_boxes(cspt_quadtree const* tree, void const* bminx,
                                      void const* bminy, void const* bmaxx, void const* bmaxy,
                                      size_t nb, cspt_dtype dtype, double x_min, double y_min,
                                      double scale, int max_depth, Allocator const& alloc,
                                      uint32_t** out_box, uint32_t** out_node, size_t* out_n)
{
  if (dtype == CSPT_FLOAT64)
    run<double>(tree, static_cast<double const*>(bminx), static_cast<double const*>(bminy),
                static_cast<double const*>(bmaxx), static_cast<double const*>(bmaxy), nb, x_min,
                y_min, scale, max_depth, alloc, out_box, out_node, out_n);
  else
    run<float>(tree, static_cast<float const*>(bminx), static_cast<float const*>(bminy),
               static_cast<float const*>(bmaxx), static_cast<float const*>(bmaxy), nb,
               static_cast<float>(x_min), static_cast<float>(y_min), static_cast<float>(scale),
               max_depth, alloc, out_box, out_node, out_n);
}

}  // namespace cspt
