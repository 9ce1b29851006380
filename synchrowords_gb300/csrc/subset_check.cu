// Tiled subset check: for every query row c, does some row s of S satisfy
// s ⊆ c (proper: s ⊊ c; disjoint: s ∩ c = ∅)?
//
// Replaces the reference's subset tests (SubsetsImplicitTrie::check_contains_subset,
// synchrolib/data_structures/subsets_implicit_trie.hpp:29-266, and its GPU leaf
// kernel cuda/subsets_implicit_trie_kernel.cu:13-92).  The trie's pruning is
// re-expressed as a prefix-partitioned candidate filter:
//   * S is sorted (lexicographically, most frequent states first) and cut into
//     tiles of 64 consecutive rows, grouped 16 to a super-tile;
//   * every tile and super-tile keeps the AND of its rows — the states all of
//     its sets contain.  For sorted rows that is the range's common prefix
//     (the trie node's path) plus incidental shared states;
//   * a query that lacks one of those states cannot contain any set of the
//     range.
// One warp owns 32 consecutive (hence similar) queries and streams the
// super-tiles of its chunk of S: a range is skipped unless some lane still
// needs it (__any_sync), a needed tile is staged into the warp's slice of
// shared memory with one coalesced read, and every lane tests its own query
// against the staged rows with an early exit on word 0.  No block-wide
// barriers: warps of a block proceed independently.  Warps stop as soon as all
// their queries are decided; in meet mode the first hit stops the grid.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"

namespace sw {

namespace {
constexpr int kTileRows = 64;
constexpr int kTilesPerSuper = 16;
constexpr int kSuperRows = kTileRows * kTilesPerSuper;
constexpr int kWarps = 8;
constexpr u32 kMinChunkTiles = 4;
constexpr u32 kFullMask = 0xffffffffu;

int sm_count_sc() { return device_sm_count(); }

__host__ __device__ inline u32 n_tiles(u32 m) { return (m + kTileRows - 1) / kTileRows; }
__host__ __device__ inline u32 n_supers(u32 m) { return (m + kSuperRows - 1) / kSuperRows; }
}  // namespace

// AND masks: tiles first (n_tiles(m) entries), then super-tiles.  One warp
// per tile: each lane ANDs two rows, a butterfly combines the lanes, and the
// tile mask is folded into its super-tile's mask (pre-set to all ones).
template <int W>
__global__ void k_range_and(const u64* __restrict__ S, u32 m, u64* __restrict__ masks) {
  const u32 tiles = n_tiles(m);
  const u32 t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= tiles) return;  // warp-uniform
  const u32 r0 = t * kTileRows + lane, r1 = r0 + 32;
  u64* super_and = masks + (size_t)tiles * W;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    u64 a = r0 < m ? S[(size_t)r0 * W + w] : ~0ULL;
    if (r1 < m) a &= S[(size_t)r1 * W + w];
#pragma unroll
    for (int o = 16; o; o >>= 1) a &= __shfl_xor_sync(kFullMask, a, o);
    if (lane == 0) {
      masks[(size_t)t * W + w] = a;
      atomicAnd(&super_and[(size_t)(t / kTilesPerSuper) * W + w], a);
    }
  }
}

template <int W, int MODE>
__global__ void __launch_bounds__(kWarps * 32) k_subset_scan(const u64* __restrict__ S, u32 m,
                                                             const u64* __restrict__ masks, u32 tiles_per_chunk,
                                                             const u64* __restrict__ Q, u32 q, int n,
                                                             u32* __restrict__ flags, u32* witness, int stop,
                                                             u64* __restrict__ bytes_ctr) {
  __shared__ __align__(16) u64 s_rows[kWarps][kTileRows * W];
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
  const u32 tiles = n_tiles(m);
  const u64* tile_and = masks;
  const u64* super_and = masks + (size_t)tiles * W;
  u64* my_rows = s_rows[warp];
  const u32 t0 = blockIdx.y * tiles_per_chunk;
  const u32 t1 = min(tiles, t0 + tiles_per_chunk);
  bool need_s = false;
  for (u32 t = t0; t < t1; ++t) {
    if (t == t0 || t % kTilesPerSuper == 0) {
      // entering a super-tile: stop checks, then its mask decides for all
      // of its tiles in this chunk
      if (__all_sync(kFullMask, done)) break;
      if (stop) {
        u32 f = lane == 0 ? *(volatile u32*)witness : 0u;
        if (__shfl_sync(kFullMask, f, 0)) break;
      }
      const u32 sp = t / kTilesPerSuper;
      need_s = !done;
#pragma unroll
      for (int w = 0; w < W; ++w)
        if (super_and[(size_t)sp * W + w] & ~c[w]) need_s = false;
      if (!__any_sync(kFullMask, need_s)) {
        t = min(t1, (sp + 1) * kTilesPerSuper) - 1;  // skip the rest of this super-tile
        continue;
      }
    }
    bool need = need_s && !done;
#pragma unroll
    for (int w = 0; w < W; ++w)
      if (tile_and[(size_t)t * W + w] & ~c[w]) need = false;
    if (!__any_sync(kFullMask, need)) continue;
    const u32 r0 = t * kTileRows;
    const u32 rows = min((u32)kTileRows, m - r0);
    const u64* src = S + (size_t)r0 * W;
    if (W >= 2) {
      // 16-byte moves (tile starts are 16-byte aligned: 64 rows of 8W bytes);
      // an odd word count leaves one word for a plain load
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      uint4* d4 = reinterpret_cast<uint4*>(my_rows);
      const u32 words = rows * W;
      for (u32 i = lane; i < words / 2; i += 32) d4[i] = s4[i];
      if ((words & 1u) && lane == 0) my_rows[words - 1] = src[words - 1];
    } else {
      for (u32 i = lane; i < rows; i += 32) my_rows[i] = src[i];
    }
    // rows past the end of S never pass the word-0 test below
    if (rows < (u32)kTileRows)
      for (u32 i = rows * W + lane; i < (u32)kTileRows * W; i += 32) my_rows[i] = ~0ULL;
    loaded += rows;
    __syncwarp();
    if (need) {
      const u64 nc0 = ~c[0];
      // four rows per iteration: independent word-0 tests, full test only
      // for the (rare) rows that pass
      for (u32 r = 0; r < (u32)kTileRows && !done; r += 4) {
        const u64 a0 = my_rows[(r + 0) * W], a1 = my_rows[(r + 1) * W];
        const u64 a2 = my_rows[(r + 2) * W], a3 = my_rows[(r + 3) * W];
        const unsigned pass = (!(a0 & nc0) ? 1u : 0u) | (!(a1 & nc0) ? 2u : 0u) | (!(a2 & nc0) ? 4u : 0u) |
                              (!(a3 & nc0) ? 8u : 0u);
        if (!pass) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (!((pass >> j) & 1u) || r + j >= rows) continue;
          const u64* s = my_rows + (r + j) * W;
          bool sub = true, eq = (s[0] == c[0]);
#pragma unroll
          for (int w = 1; w < W; ++w) {
            sub = sub && !(s[w] & ~c[w]);
            eq = eq && (s[w] == c[w]);
          }
          if (sub && (MODE != kQueryProperSubset || !eq)) {
            hit = true;
            done = true;
            hit_idx = r0 + r + j;
            break;
          }
        }
      }
    }
    __syncwarp();
    if (stop && hit) {
      if (atomicCAS(witness, 0u, 1u) == 0u) {
        witness[1] = qi;
        witness[2] = hit_idx;
      }
      hit = false;  // recorded
    }
  }
  if (bytes_ctr && lane == 0 && loaded) atomicAdd(bytes_ctr, loaded * 8ULL * W);
  if (hit && !stop) flags[qi] = 1u;
}

size_t subset_check_temp_bytes(int W, u32 m) {
  return sizeof(u64) * (size_t)W * (n_tiles(std::max<u32>(m, 1)) + n_supers(std::max<u32>(m, 1)) + 1);
}

void launch_tile_and(int W, const u64* S, u32 m, u64* masks, cudaStream_t s) {
  if (!m) return;
  const u32 tiles = n_tiles(m);
  SW_CUDA(cudaMemsetAsync(masks + (size_t)tiles * W, 0xff, sizeof(u64) * W * n_supers(m), s));
  const u32 blocks = (tiles * 32 + 255) / 256;
  switch (W) {
    case 1: k_range_and<1><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 2: k_range_and<2><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 3: k_range_and<3><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 4: k_range_and<4><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 5: k_range_and<5><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 6: k_range_and<6><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 7: k_range_and<7><<<blocks, 256, 0, s>>>(S, m, masks); break;
    case 8: k_range_and<8><<<blocks, 256, 0, s>>>(S, m, masks); break;
    default: throw std::runtime_error("range_and: unsupported width");
  }
  SW_LAUNCH_CHECK();
}

void launch_subset_check(int W, int mode, const u64* S, u32 m, const u64* masks, const u64* Q, u32 q, int n,
                         u32* flags, u32* witness, bool stop, cudaStream_t s, u64* bytes_ctr) {
  if (!m || !q) return;
  const u32 tiles = n_tiles(m);
  const u32 qblocks = (q + kWarps * 32 - 1) / (kWarps * 32);
  // split S into chunks of tiles so that the grid covers the GPU ~16x: per-warp
  // work varies a lot (early exits, filter hit rates), and many small blocks
  // keep the SMs busy until the slowest ones finish.  A chunk keeps at least
  // kMinChunkTiles tiles so that loading the warp's queries stays amortised.
  const u32 target = (u32)sm_count_sc() * 16;
  u32 chunks = std::max<u32>(1, (target + qblocks - 1) / qblocks);
  chunks = std::min<u32>(chunks, std::max<u32>(1, tiles / kMinChunkTiles));
  chunks = std::min<u32>(chunks, 65535);
  const u32 per = (tiles + chunks - 1) / chunks;
  chunks = (tiles + per - 1) / per;
  dim3 grid(qblocks, chunks);
#define SW_SC(WW)                                                                                              \
  case WW:                                                                                                     \
    if (mode == kQuerySubset)                                                                                  \
      k_subset_scan<WW, kQuerySubset><<<grid, kWarps * 32, 0, s>>>(S, m, masks, per, Q, q, n, flags, witness, \
                                                                   stop, bytes_ctr);                           \
    else if (mode == kQueryProperSubset)                                                                       \
      k_subset_scan<WW, kQueryProperSubset><<<grid, kWarps * 32, 0, s>>>(S, m, masks, per, Q, q, n, flags,    \
                                                                         witness, stop, bytes_ctr);            \
    else                                                                                                       \
      k_subset_scan<WW, kQueryDisjoint><<<grid, kWarps * 32, 0, s>>>(S, m, masks, per, Q, q, n, flags,        \
                                                                     witness, stop, bytes_ctr);                \
    break;
  switch (W) {
    SW_SC(1)
    SW_SC(2)
    SW_SC(3)
    SW_SC(4)
    SW_SC(5)
    SW_SC(6)
    SW_SC(7)
    SW_SC(8)
    default:
      throw std::runtime_error("subset check: unsupported width");
  }
#undef SW_SC
  SW_LAUNCH_CHECK();
}

}  // namespace sw
