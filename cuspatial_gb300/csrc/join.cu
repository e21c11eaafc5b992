// Quadrant / bounding-box intersection join on sm_103a.
//
// Reference: cpp/include/cuspatial/detail/join/quadtree_bbox_filtering.cuh:
// 35-188 (seeds, level loop, final stable sort by leaf offset),
// intersection.cuh:79-136 (node extent and closed-interval overlap) and
// traversal.cuh:57-145 (descent to children).
//
// The reference walks all boxes level by level with a host synchronisation
// per level.  Here a warp owns one box and walks the tree with a stack in
// shared memory (join_kernel.cuh).  The count pass sizes the output and
// appends every (node, box) it finds; a radix sort of the composite key
// (leaf first-point offset, box) gives the reference's order.  When the
// appended pairs would not fit, a write pass emits (leaf offset, node, box)
// in box-major order and a stable radix sort by the leaf offset gives the
// same order.
// A node at traversal depth t is expanded only while t + 1 < max_depth, the
// reference's loop bound (quadtree_bbox_filtering.cuh:118).
#include "join_kernel.cuh"
#include "radix_sort.cuh"

namespace cspt {
namespace {

// Pairs the count pass may append (node + box, 8 bytes each): 64 per box, at
// most 64 Mi pairs; a join with more runs the write pass instead.
inline size_t join_append_capacity(size_t nb)
{
  size_t const c = nb * 64;
  return c < (size_t{64} << 20) ? c : (size_t{64} << 20);
}

// (leaf first-point offset << box_bits) | box of each appended pair.
__global__ void composite_key_kernel(uint32_t const* __restrict__ node,
                                     uint32_t const* __restrict__ box, size_t k,
                                     uint32_t const* __restrict__ offset, int box_bits,
                                     uint64_t* __restrict__ key)
{
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < k;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    key[i] = (static_cast<uint64_t>(offset[node[i]]) << box_bits) | box[i];
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
  CSPT_EXPECTS(tree->num_nodes < (size_t{1} << 28), "quadtree has too many nodes");
  OneTree<T> const trees{L0.data(), static_cast<uint32_t>(tree->num_nodes), vminx, vminy, scale,
                         max_depth};
  Buffer<uint32_t> counts(alloc, nb + 1);
  Buffer<uint32_t> status(alloc, 2);  // [0] max leaf offset, [1] error flag
  CSPT_CUDA_TRY(cudaMemsetAsync(status.data(), 0, 2 * sizeof(uint32_t), s));
  int* err           = reinterpret_cast<int*>(status.data() + 1);
  unsigned const blk = kJoinWarps * 32;
  unsigned const grd = grid_for(nb * 32, blk, sm_grid(16u));
  // the count pass also appends each (node, box) it finds while they fit
  size_t const cap = join_append_capacity(nb);
  Buffer<uint32_t> app_node(alloc, cap), app_box(alloc, cap);
  Buffer<unsigned long long> app_n(alloc, 1);
  CSPT_CUDA_TRY(cudaMemsetAsync(app_n.data(), 0, sizeof(unsigned long long), s));
  {
    KernelTimer timer("join_count", s);
    join_warp_kernel<T, false><<<grd, blk, 0, s>>>(
      tv, trees, bminx, bminy, bmaxx, bmaxy, nb, counts.data(), status.data(), nullptr, nullptr,
      nullptr, nullptr, err, JoinAppend{app_node.data(), app_box.data(), app_n.data(), cap});
    CSPT_CHECK_LAUNCH();
  }
  exclusive_scan<uint32_t>(counts.data(), counts.data(), nb, counts.data() + nb, alloc);
  uint32_t host[3];
  unsigned long long appended = 0;
  CSPT_CUDA_TRY(cudaMemcpyAsync(host, counts.data() + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                s));
  CSPT_CUDA_TRY(
    cudaMemcpyAsync(host + 1, status.data(), 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaMemcpyAsync(&appended, app_n.data(), sizeof(appended),
                                cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaStreamSynchronize(s));
  size_t const k = host[0];
  CSPT_EXPECTS(host[2] == 0,
               "quadtree is malformed: a node index or child count is out of range");
  *out_n = k;
  if (k == 0) return;
  int key_bits = 1;
  while (key_bits < 32 && (host[1] >> key_bits) != 0) ++key_bits;
  Buffer<uint32_t> ob(alloc, k), on(alloc, k);
  if (appended == k && k <= cap) {
    // Every pair was appended (in no particular order): sort them by
    // (leaf offset, box), one composite key, which is the order the write
    // pass and a stable sort by leaf offset give.
    int box_bits = 1;
    while (box_bits < 32 && ((nb - 1) >> box_bits) != 0) ++box_bits;
    app_n.reset();
    Buffer<uint64_t> key(alloc, k), key_alt(alloc, k);
    Buffer<uint32_t> perm(alloc, k), perm_alt(alloc, k);
    {
      KernelTimer timer("join_write", s);
      composite_key_kernel<<<grid_for(k, 256, sm_grid(16u)), 256, 0, s>>>(
        app_node.data(), app_box.data(), k, tv.offset, box_bits, key.data());
      CSPT_CHECK_LAUNCH();
    }
    bool const alt = radix_sort_pairs<uint64_t>(key.data(), perm.data(), key_alt.data(),
                                                perm_alt.data(), k, 0, key_bits + box_bits, true,
                                                alloc);
    gather_pairs_kernel<<<grid_for(k, 256, sm_grid(16u)), 256, 0, s>>>(
      alt ? perm_alt.data() : perm.data(), app_node.data(), app_box.data(), k, ob.data(),
      on.data());
    CSPT_CHECK_LAUNCH();
  } else {
    app_node.reset();
    app_box.reset();
    Buffer<uint32_t> key(alloc, k), key_alt(alloc, k), node(alloc, k), box(alloc, k),
      perm(alloc, k), perm_alt(alloc, k);
    {
      KernelTimer timer("join_write", s);
      join_warp_kernel<T, true><<<grd, blk, 0, s>>>(tv, trees, bminx, bminy, bmaxx, bmaxy, nb,
                                                    nullptr, nullptr, counts.data(), key.data(),
                                                    node.data(), box.data(), err);
      CSPT_CHECK_LAUNCH();
    }
    bool const alt = radix_sort_pairs<uint32_t>(key.data(), perm.data(), key_alt.data(),
                                                perm_alt.data(), k, 0, key_bits, true, alloc);
    gather_pairs_kernel<<<grid_for(k, 256, sm_grid(16u)), 256, 0, s>>>(
      alt ? perm_alt.data() : perm.data(), node.data(), box.data(), k, ob.data(), on.data());
    CSPT_CHECK_LAUNCH();
  }
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
