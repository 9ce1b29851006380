// Tiled subset check: for every query row c, does some row s of S satisfy
// s ⊆ c (proper: s ⊊ c; disjoint: s ∩ c = ∅)?
//
// Replaces the reference's subset tests (SubsetsImplicitTrie::check_contains_subset,
// synchrolib/data_structures/subsets_implicit_trie.hpp:29-266, and its GPU leaf
// kernel cuda/subsets_implicit_trie_kernel.cu:13-92).  The trie's pruning is
// re-expressed as a prefix-partitioned candidate filter:
//   * S is sorted (lexicographically, most frequent states first) and cut into
//     leaf tiles of 32 consecutive rows;
//   * an implicit binary tree over the tiles stores, per node, the AND of all
//     rows below it — the states every set of that range contains.  For sorted
//     rows this is the range's common prefix (the trie node's path) plus
//     incidental shared states;
//   * a query that lacks one of a node's states cannot contain any set below
//     it.
// One warp owns 32 consecutive (hence similar) queries and walks the tree
// depth-first; it descends into a node only if some lane still needs it
// (__any_sync), so the walk is warp-uniform.  A needed leaf tile is loaded
// with one coalesced read (lane r holds row r) and broadcast row by row with
// shuffles; every lane tests its own query with an early exit on word 0.
// Warps stop as soon as all their queries are decided; in meet mode the
// first hit of any warp stops the grid.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "kernels.cuh"

namespace sw {

namespace {
constexpr int kLeafRows = 32;
constexpr int kWarps = 4;
constexpr int kMaxLevels = 32;
constexpr int kStackPerWarp = 2 * kMaxLevels + 2;
constexpr u32 kFullMask = 0xffffffffu;

struct TreeShape {
  int levels;                // level 0 = leaves
  u32 count[kMaxLevels];     // nodes per level
  u32 offset[kMaxLevels];    // first node of the level in the node array
};

TreeShape tree_shape(u32 m) {
  TreeShape t{};
  u32 c = (m + kLeafRows - 1) / kLeafRows;
  u32 off = 0;
  int l = 0;
  while (true) {
    t.count[l] = c;
    t.offset[l] = off;
    off += c;
    ++l;
    if (c <= 1) break;
    c = (c + 1) / 2;
  }
  t.levels = l;
  return t;
}

int sm_count_sc() {
  static int cached = 0;
  if (!cached) {
    int dev = 0;
    SW_CUDA(cudaGetDevice(&dev));
    SW_CUDA(cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev));
  }
  return cached;
}
}  // namespace

// Level 0: AND of each 32-row leaf tile.
template <int W>
__global__ void k_leaf_and(const u64* __restrict__ S, u32 m, u64* __restrict__ nodes) {
  const u32 leaves = (m + kLeafRows - 1) / kLeafRows;
  const u32 id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= leaves * W) return;
  const u32 t = id / W, w = id % W;
  const u32 r0 = t * kLeafRows, r1 = min(m, r0 + kLeafRows);
  u64 a = ~0ULL;
  for (u32 r = r0; r < r1; ++r) a &= S[(size_t)r * W + w];
  nodes[id] = a;
}

// Upper levels, one block, level by level.
template <int W>
__global__ void __launch_bounds__(1024) k_upper_and(u64* nodes, TreeShape t) {
  for (int l = 1; l < t.levels; ++l) {
    const u32 cnt = t.count[l], prev = t.count[l - 1];
    for (u32 id = threadIdx.x; id < cnt * W; id += blockDim.x) {
      const u32 i = id / W, w = id % W;
      const u32 c0 = 2 * i, c1 = 2 * i + 1;
      u64 a = nodes[((size_t)t.offset[l - 1] + c0) * W + w];
      if (c1 < prev) a &= nodes[((size_t)t.offset[l - 1] + c1) * W + w];
      nodes[((size_t)t.offset[l] + i) * W + w] = a;
    }
    __syncthreads();
  }
}

template <int W, int MODE>
__global__ void __launch_bounds__(kWarps * 32) k_subset_tree(const u64* __restrict__ S, u32 m,
                                                             const u64* __restrict__ nodes, TreeShape t,
                                                             int start_level, const u64* __restrict__ Q, u32 q,
                                                             int n, u32* __restrict__ flags, u32* witness, int stop,
                                                             u64* __restrict__ bytes_ctr) {
  __shared__ u32 s_stack[kWarps][kStackPerWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 qi = (blockIdx.x * kWarps + warp) * 32 + lane;
  const bool valid = qi < q;
  u64 c[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    c[w] = valid ? Q[(size_t)qi * W + w] : 0ULL;
    if (MODE == kQueryDisjoint) c[w] = ~c[w] & valid_mask(n, w);
  }
  bool done = !valid || (!stop && flags[qi]);
  bool hit = false;
  u32 hit_idx = 0;
  u64 loaded = 0;
  u32* st = s_stack[warp];
  int sp = 0;
  // this warp's subtree root: node blockIdx.y of level start_level
  if (blockIdx.y < t.count[start_level]) {
    if (lane == 0) st[0] = ((u32)start_level << 26) | blockIdx.y;
    sp = 1;
  }
  __syncwarp();
  int iter = 0;
  while (sp > 0) {
    if (__all_sync(kFullMask, done)) break;
    if (stop && ((++iter & 7) == 0)) {
      u32 f = lane == 0 ? *(volatile u32*)witness : 0u;
      if (__shfl_sync(kFullMask, f, 0)) break;
    }
    --sp;
    const u32 e = st[sp];
    __syncwarp();
    const int l = (int)(e >> 26);
    const u32 i = e & ((1u << 26) - 1);
    const u64* nd = nodes + ((size_t)t.offset[l] + i) * W;
    bool need = !done;
#pragma unroll
    for (int w = 0; w < W; ++w)
      if (nd[w] & ~c[w]) need = false;
    if (!__any_sync(kFullMask, need)) continue;
    if (l == 0) {
      const u32 r0 = i * kLeafRows;
      const u32 rows = min((u32)kLeafRows, m - r0);
      u64 my[W];
#pragma unroll
      for (int w = 0; w < W; ++w) my[w] = (lane < (int)rows) ? S[((size_t)r0 + lane) * W + w] : ~0ULL;
      loaded += rows;
      for (u32 r = 0; r < rows; ++r) {
        u64 s[W];
#pragma unroll
        for (int w = 0; w < W; ++w) s[w] = __shfl_sync(kFullMask, my[w], r);
        if (need && !done) {
          bool sub = !(s[0] & ~c[0]);
          bool eq = (s[0] == c[0]);
#pragma unroll
          for (int w = 1; w < W; ++w) {
            sub = sub && !(s[w] & ~c[w]);
            eq = eq && (s[w] == c[w]);
          }
          if (sub && (MODE != kQueryProperSubset || !eq)) {
            hit = true;
            done = true;
            hit_idx = r0 + r;
          }
        }
      }
      if (stop && hit) {
        if (atomicCAS(witness, 0u, 1u) == 0u) {
          witness[1] = qi;
          witness[2] = hit_idx;
        }
        hit = false;  // recorded
      }
    } else {
      const u32 c0 = 2 * i, c1 = 2 * i + 1;
      if (lane == 0) {
        if (c1 < t.count[l - 1]) st[sp++] = ((u32)(l - 1) << 26) | c1;
        st[sp++] = ((u32)(l - 1) << 26) | c0;
      } else {
        sp += (c1 < t.count[l - 1]) ? 2 : 1;
      }
      __syncwarp();
    }
  }
  if (bytes_ctr && lane == 0 && loaded) atomicAdd(bytes_ctr, loaded * 8ULL * W);
  if (hit && !stop) flags[qi] = 1u;
}

size_t subset_check_temp_bytes(int W, u32 m) {
  TreeShape t = tree_shape(std::max<u32>(m, 1));
  u32 total = t.offset[t.levels - 1] + t.count[t.levels - 1];
  return sizeof(u64) * (size_t)W * (total + 1);
}

void launch_tile_and(int W, const u64* S, u32 m, u64* nodes, cudaStream_t s) {
  if (!m) return;
  TreeShape t = tree_shape(m);
  const u32 threads = t.count[0] * W;
  switch (W) {
    case 1: k_leaf_and<1><<<(threads + 255) / 256, 256, 0, s>>>(S, m, nodes); break;
    case 2: k_leaf_and<2><<<(threads + 255) / 256, 256, 0, s>>>(S, m, nodes); break;
    case 4: k_leaf_and<4><<<(threads + 255) / 256, 256, 0, s>>>(S, m, nodes); break;
    case 8: k_leaf_and<8><<<(threads + 255) / 256, 256, 0, s>>>(S, m, nodes); break;
    default: throw std::runtime_error("tile_and: unsupported width");
  }
  if (t.levels > 1) {
    switch (W) {
      case 1: k_upper_and<1><<<1, 1024, 0, s>>>(nodes, t); break;
      case 2: k_upper_and<2><<<1, 1024, 0, s>>>(nodes, t); break;
      case 4: k_upper_and<4><<<1, 1024, 0, s>>>(nodes, t); break;
      case 8: k_upper_and<8><<<1, 1024, 0, s>>>(nodes, t); break;
    }
  }
  SW_LAUNCH_CHECK();
}

void launch_subset_check(int W, int mode, const u64* S, u32 m, const u64* nodes, const u64* Q, u32 q, int n,
                         u32* flags, u32* witness, bool stop, cudaStream_t s, u64* bytes_ctr) {
  if (!m || !q) return;
  TreeShape t = tree_shape(m);
  const u32 qblocks = (q + kWarps * 32 - 1) / (kWarps * 32);
  // start the walks below the root so that (query blocks x subtrees) covers the GPU ~4x
  const u32 target = (u32)sm_count_sc() * 4;
  int start = t.levels - 1;
  while (start > 0 && qblocks * t.count[start] < target && t.count[start - 1] <= 65535) --start;
  dim3 grid(qblocks, t.count[start]);
#define SW_SC(WW)                                                                                                 \
  case WW:                                                                                                        \
    if (mode == kQuerySubset)                                                                                     \
      k_subset_tree<WW, kQuerySubset><<<grid, kWarps * 32, 0, s>>>(S, m, nodes, t, start, Q, q, n, flags,       \
                                                                   witness, stop, bytes_ctr);                     \
    else if (mode == kQueryProperSubset)                                                                          \
      k_subset_tree<WW, kQueryProperSubset><<<grid, kWarps * 32, 0, s>>>(S, m, nodes, t, start, Q, q, n, flags, \
                                                                         witness, stop, bytes_ctr);               \
    else                                                                                                          \
      k_subset_tree<WW, kQueryDisjoint><<<grid, kWarps * 32, 0, s>>>(S, m, nodes, t, start, Q, q, n, flags,     \
                                                                     witness, stop, bytes_ctr);                   \
    break;
  switch (W) {
    SW_SC(1)
    SW_SC(2)
    SW_SC(4)
    SW_SC(8)
    default:
      throw std::runtime_error("subset check: unsupported width");
  }
#undef SW_SC
  SW_LAUNCH_CHECK();
}

}  // namespace sw
