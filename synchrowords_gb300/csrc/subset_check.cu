// Tiled subset check: for every query row c, does some row s of S satisfy
// s ⊆ c (proper: s ⊊ c; disjoint: s ∩ c = ∅)?
//
// Replaces the reference's subset tests (SubsetsImplicitTrie::check_contains_subset,
// synchrolib/data_structures/subsets_implicit_trie.hpp:29-266, and its GPU leaf
// kernel cuda/subsets_implicit_trie_kernel.cu:13-92).  The trie's pruning is
// re-expressed as a prefix-partitioned candidate filter: S is sorted
// (lexicographically, most frequent states first), cut into tiles of T
// consecutive rows, and every tile keeps the AND of its rows — the states all
// of its sets contain.  A query that lacks one of those states cannot contain
// any set of the tile, so the tile is skipped; a tile is staged into shared
// memory only if some query of the block still needs it.  Each thread owns one
// query in registers and walks the staged rows with an early exit on the
// first word; the block stops as soon as all its queries are decided.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"

namespace sw {

namespace {
constexpr int kTile = 64;      // rows per tile
constexpr int kThreads = 128;  // queries per block

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

template <int W>
__global__ void k_tile_and(const u64* __restrict__ S, u32 m, u64* __restrict__ tile_and) {
  const u32 ntiles = (m + kTile - 1) / kTile;
  const u32 id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= ntiles * W) return;
  const u32 t = id / W, w = id % W;
  const u32 r0 = t * kTile, r1 = min(m, r0 + kTile);
  u64 a = ~0ULL;
  for (u32 r = r0; r < r1; ++r) a &= S[(size_t)r * W + w];
  tile_and[id] = a;
}

template <int W, int MODE>
__global__ void __launch_bounds__(kThreads) k_subset_tiles(const u64* __restrict__ S, u32 m,
                                                           const u64* __restrict__ tile_and, u32 tiles_per_chunk,
                                                           const u64* __restrict__ Q, u32 q, int n,
                                                           u32* __restrict__ flags, u32* witness, int stop,
                                                           u64* __restrict__ bytes_ctr) {
  __shared__ __align__(16) u64 s_tile[kTile * W];
  const u32 qi = blockIdx.x * kThreads + threadIdx.x;
  const bool valid = qi < q;
  u64 c[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    c[w] = valid ? Q[(size_t)qi * W + w] : 0ULL;
    if (MODE == kQueryDisjoint) c[w] = ~c[w] & valid_mask(n, w);
  }
  bool done = !valid;
  if (valid && !stop && flags[qi]) done = true;  // decided by another chunk already
  bool hit = false;
  u32 hit_idx = 0;
  u64 loaded = 0;
  const u32 ntiles = (m + kTile - 1) / kTile;
  const u32 t0 = blockIdx.y * tiles_per_chunk;
  const u32 t1 = min(ntiles, t0 + tiles_per_chunk);
  for (u32 t = t0; t < t1; ++t) {
    // block-uniform exit once any block of the grid found a meeting pair
    if (__syncthreads_or(stop && *(volatile u32*)witness)) break;
    bool need = !done;
    if (need) {
#pragma unroll
      for (int w = 0; w < W; ++w)
        if (tile_and[(size_t)t * W + w] & ~c[w]) need = false;
    }
    if (!__syncthreads_or(need)) {
      if (!__syncthreads_or(!done)) break;
      continue;
    }
    const u32 rows = min((u32)kTile, m - t * kTile);
    const u64* src = S + (size_t)t * kTile * W;
    if (W >= 2) {
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      uint4* d4 = reinterpret_cast<uint4*>(s_tile);
      for (u32 i = threadIdx.x; i < rows * W / 2; i += kThreads) d4[i] = s4[i];
    } else {
      for (u32 i = threadIdx.x; i < rows; i += kThreads) s_tile[i] = src[i];
    }
    loaded += rows;
    __syncthreads();
    if (need) {
      for (u32 r = 0; r < rows; ++r) {
        const u64* s = s_tile + r * W;
        if (s[0] & ~c[0]) continue;
        bool sub = true, eq = (s[0] == c[0]);
#pragma unroll
        for (int w = 1; w < W; ++w) {
          sub = sub && !(s[w] & ~c[w]);
          eq = eq && (s[w] == c[w]);
        }
        if (sub && (MODE != kQueryProperSubset || !eq)) {
          hit = true;
          done = true;
          hit_idx = t * kTile + r;
          break;
        }
      }
    }
    if (hit && stop) {
      if (atomicCAS(witness, 0u, 1u) == 0u) {
        witness[1] = qi;
        witness[2] = hit_idx;
      }
    }
    if (!__syncthreads_or(!done)) break;  // also orders the smem reuse
  }
  if (bytes_ctr && threadIdx.x == 0 && loaded) atomicAdd(bytes_ctr, loaded * 8ULL * W);
  if (hit && !stop) flags[qi] = 1u;
}

size_t subset_check_temp_bytes(int W, u32 m) { return sizeof(u64) * (size_t)W * ((m + kTile - 1) / kTile + 1); }

void launch_tile_and(int W, const u64* S, u32 m, u64* tile_and, cudaStream_t s) {
  if (!m) return;
  const u32 ntiles = (m + kTile - 1) / kTile;
  const u32 threads = ntiles * W;
  switch (W) {
    case 1: k_tile_and<1><<<(threads + 255) / 256, 256, 0, s>>>(S, m, tile_and); break;
    case 2: k_tile_and<2><<<(threads + 255) / 256, 256, 0, s>>>(S, m, tile_and); break;
    case 4: k_tile_and<4><<<(threads + 255) / 256, 256, 0, s>>>(S, m, tile_and); break;
    case 8: k_tile_and<8><<<(threads + 255) / 256, 256, 0, s>>>(S, m, tile_and); break;
    default: throw std::runtime_error("tile_and: unsupported width");
  }
  SW_LAUNCH_CHECK();
}

void launch_subset_check(int W, int mode, const u64* S, u32 m, const u64* tile_and, const u64* Q, u32 q, int n,
                         u32* flags, u32* witness, bool stop, cudaStream_t s, u64* bytes_ctr) {
  if (!m || !q) return;
  const u32 ntiles = (m + kTile - 1) / kTile;
  const u32 qblocks = (q + kThreads - 1) / kThreads;
  // split the tiles into chunks so that the grid covers the GPU ~4x
  const u32 target = (u32)sm_count_sc() * 4;
  u32 chunks = std::max<u32>(1, std::min<u32>(ntiles, (target + qblocks - 1) / qblocks));
  chunks = std::min<u32>(chunks, 65535);
  const u32 per = (ntiles + chunks - 1) / chunks;
  chunks = (ntiles + per - 1) / per;
  dim3 grid(qblocks, chunks);
#define SW_SC(WW)                                                                                               \
  case WW:                                                                                                      \
    if (mode == kQuerySubset)                                                                                   \
      k_subset_tiles<WW, kQuerySubset><<<grid, kThreads, 0, s>>>(S, m, tile_and, per, Q, q, n, flags, witness, \
                                                                 stop, bytes_ctr);                              \
    else if (mode == kQueryProperSubset)                                                                        \
      k_subset_tiles<WW, kQueryProperSubset><<<grid, kThreads, 0, s>>>(S, m, tile_and, per, Q, q, n, flags,    \
                                                                       witness, stop, bytes_ctr);               \
    else                                                                                                        \
      k_subset_tiles<WW, kQueryDisjoint><<<grid, kThreads, 0, s>>>(S, m, tile_and, per, Q, q, n, flags,        \
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
