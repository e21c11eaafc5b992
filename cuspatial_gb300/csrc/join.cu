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

constexpr int kJoinWarps = 4;       // warps per block
constexpr int kWarpStack = 2048;    // stack entries per warp (shared memory)

// One warp per box.  Each round pops up to 32 entries (node << 4 | depth)
// from the warp's shared stack, one per lane, classifies them, counts or
// writes the leaves with a ballot, and pushes the children of internal nodes
// (warp scan of the child counts).  If the stack would overflow the warp
// restarts the box on lane 0 with the private-stack walk above.  Seeds (the
// level-0 nodes) are fed 32 at a time whenever the stack runs empty.
template <typename T, bool Write>
__global__ void __launch_bounds__(kJoinWarps * 32)
  join_warp_kernel(TreeView t, uint32_t const* __restrict__ L0p, T const* __restrict__ bminx,
                   T const* __restrict__ bminy, T const* __restrict__ bmaxx,
                   T const* __restrict__ bmaxy, size_t nb, T vminx, T vminy, T scale,
                   int max_depth, uint32_t* __restrict__ counts, uint32_t* __restrict__ maxkey,
                   uint32_t const* __restrict__ pos, uint32_t* __restrict__ okey,
                   uint32_t* __restrict__ onode, uint32_t* __restrict__ obox,
                   int* __restrict__ error)
{
  __shared__ uint32_t stack_s[kJoinWarps][kWarpStack];
  uint32_t* stack      = stack_s[threadIdx.x >> 5];
  int const lane       = threadIdx.x & 31;
  unsigned const lt    = (1u << lane) - 1u;
  uint32_t const L0    = *L0p;
  size_t const nwarps  = (static_cast<size_t>(gridDim.x) * blockDim.x) >> 5;
  uint32_t local_max   = 0;
  for (size_t b = (blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5; b < nb;
       b += nwarps) {
    T const x0 = bminx[b], y0 = bminy[b], x1 = bmaxx[b], y1 = bmaxy[b];
    uint32_t found = 0;
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
      if (have) {
        if (node >= t.nq) {
          bad = true;
        } else {
          c = classify<T>(t, node, x0, y0, x1, y1, vminx, vminy, scale, max_depth);
        }
      }
      unsigned const leaves = __ballot_sync(0xFFFFFFFFu, c == 0);
      if (c == 0) {
        uint32_t const key = t.offset[node];
        if (Write) {
          uint32_t const d = p + __popc(leaves & lt);
          okey[d]          = key;
          onode[d]         = node;
          obox[d]          = static_cast<uint32_t>(b);
        } else {
          local_max = key > local_max ? key : local_max;
        }
      }
      p += __popc(leaves);
      found += __popc(leaves);
      uint32_t nchild = 0, first = 0;
      if (c == 1 && depth + 1 < max_depth) {
        first  = t.offset[node];
        nchild = t.length[node];
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
      // rare: restart the box serially on lane 0
      if (lane == 0) {
        uint32_t q = Write ? pos[b] : 0u;
        found      = 0;
        bool const ok =
          walk<T>(t, L0, x0, y0, x1, y1, vminx, vminy, scale, max_depth, [&](uint32_t node) {
            uint32_t const key = t.offset[node];
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
  Buffer<uint32_t> status(alloc, 2);  // [0] max leaf offset, [1] error flag
  CSPT_CUDA_TRY(cudaMemsetAsync(status.data(), 0, 2 * sizeof(uint32_t), s));
  int* err           = reinterpret_cast<int*>(status.data() + 1);
  unsigned const blk = kJoinWarps * 32;
  unsigned const grd = grid_for(nb * 32, blk, 152u * 16u);
  {
    KernelTimer timer("join_count", s);
    join_warp_kernel<T, false><<<grd, blk, 0, s>>>(
      tv, L0.data(), bminx, bminy, bmaxx, bmaxy, nb, vminx, vminy, scale, max_depth,
      counts.data(), status.data(), nullptr, nullptr, nullptr, nullptr, err);
    CSPT_CHECK_LAUNCH();
  }
  exclusive_scan<uint32_t>(counts.data(), counts.data(), nb, counts.data() + nb, alloc);
  uint32_t host[3];
  CSPT_CUDA_TRY(cudaMemcpyAsync(host, counts.data() + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                s));
  CSPT_CUDA_TRY(
    cudaMemcpyAsync(host + 1, status.data(), 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CSPT_CUDA_TRY(cudaStreamSynchronize(s));
  size_t const k = host[0];
  CSPT_EXPECTS(host[2] == 0,
               "quadtree is malformed: a node index or child count is out of range");
  *out_n = k;
  if (k == 0) return;
  int key_bits = 1;
  while (key_bits < 32 && (host[1] >> key_bits) != 0) ++key_bits;
  Buffer<uint32_t> key(alloc, k), key_alt(alloc, k), node(alloc, k), box(alloc, k),
    perm(alloc, k), perm_alt(alloc, k);
  {
    KernelTimer timer("join_write", s);
    join_warp_kernel<T, true><<<grd, blk, 0, s>>>(
      tv, L0.data(), bminx, bminy, bmaxx, bmaxy, nb, vminx, vminy, scale, max_depth, nullptr,
      nullptr, counts.data(), key.data(), node.data(), box.data(), err);
    CSPT_CHECK_LAUNCH();
  }
  bool const alt = radix_sort_pairs<uint32_t>(key.data(), perm.data(), key_alt.data(),
                                              perm_alt.data(), k, 0, key_bits, true, alloc);
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
