// Tiled subset check: for every query row c, does some row s of S satisfy
// s ⊆ c (proper: s ⊊ c; disjoint: s ∩ c = ∅)?
//
// Replaces the reference's subset tests (SubsetsImplicitTrie::check_contains_subset,
// synchrolib/data_structures/subsets_implicit_trie.hpp:29-266, and its GPU leaf
// kernel cuda/subsets_implicit_trie_kernel.cu:13-92).  The trie's pruning is
// re-expressed as a prefix-partitioned candidate filter:
//   * S is sorted (lexicographically, most frequent states first) and cut into
//     tiles of 64 consecutive rows, grouped 16 to a super-tile (the default
//     ScanShape; tile rows, tiles per super-tile, warps per block and the
//     grid's S chunking are runtime parameters that the kernel autotuner
//     picks per row width and list size);
//   * every tile and super-tile keeps the AND of its rows — the states all of
//     its sets contain.  For sorted rows that is the range's common prefix
//     (the trie node's path) plus incidental shared states;
//   * a query that lacks one of those states cannot contain any set of the
//     range.
// One warp owns 32 consecutive (hence similar) queries and streams the
// super-tiles of its chunk of S: a range is skipped unless some lane still
// needs it (__any_sync).  Needed tiles move into the warp's two shared-memory
// buffers by 1-D bulk copies (cp.async.bulk, completion on one mbarrier per
// buffer): while the warp tests one tile — lanes holding the tile's rows,
// the needing queries broadcast one at a time, ballots over the rows' first
// words, the full test only for rows that pass — the next needed tile is
// already on its way.  No block-wide
// barriers: warps of a block proceed independently.  Warps stop as soon as all
// their queries are decided; in meet mode the first hit stops the grid.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"

namespace sw {

namespace {
constexpr int kMaxScanWarps = 16;
constexpr int kMaxTilesPerSuper = 32;
constexpr u32 kMinChunkTiles = 4;
constexpr u32 kFullMask = 0xffffffffu;

int sm_count_sc() { return device_sm_count(); }

int log2_exact(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}
u32 n_tiles(u32 m, const ScanShape& sh) { return (m + sh.tile_rows - 1) / (u32)sh.tile_rows; }
u32 n_supers(u32 m, const ScanShape& sh) {
  const u32 rows = (u32)sh.tile_rows * (u32)sh.tiles_per_super;
  return (m + rows - 1) / rows;
}
}  // namespace

bool scan_shape_valid(int W, const ScanShape& sh) {
  const bool pow2_tr = sh.tile_rows == 32 || sh.tile_rows == 64 || sh.tile_rows == 128;
  const bool warps = sh.warps == 4 || sh.warps == 8 || sh.warps == 16;
  const bool tps = sh.tiles_per_super == 4 || sh.tiles_per_super == 8 || sh.tiles_per_super == 16 ||
                   sh.tiles_per_super == 32;
  const bool grid = sh.grid_factor >= 1 && sh.grid_factor <= 64;
  return W >= 1 && W <= 8 && pow2_tr && warps && tps && grid && scan_smem_bytes(W, sh) <= kMaxScanSmem;
}

size_t scan_smem_bytes(int W, const ScanShape& sh) {
  return sizeof(u64) * (size_t)W * (size_t)sh.tile_rows * 2 * (size_t)sh.warps;  // two tiles per warp
}

// AND masks: tiles first (n_tiles entries), then super-tiles.  One block per
// super-tile, one warp per tile: each lane ANDs the tile's rows lane,
// lane + 32, ..., a butterfly combines the lanes, and warp 0 folds the
// block's tile masks into the super-tile's mask (so no mask needs presetting
// and no atomics are used).
template <int W>
__global__ void __launch_bounds__(kMaxTilesPerSuper * 32) k_range_and(const u64* __restrict__ S, u32 m,
                                                                      u64* __restrict__ masks, int tile_rows) {
  __shared__ u64 s_and[kMaxTilesPerSuper][W];
  const u32 tiles = (m + tile_rows - 1) / (u32)tile_rows;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, tps = blockDim.x >> 5;
  const u32 t = blockIdx.x * tps + warp;
  u64* super_and = masks + (size_t)tiles * W;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    u64 a = ~0ULL;
    for (int i = lane; i < tile_rows; i += 32) {
      const u32 r = t * (u32)tile_rows + (u32)i;
      if (r < m) a &= S[(size_t)r * W + w];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) a &= __shfl_xor_sync(kFullMask, a, o);
    if (lane == 0) {
      if (t < tiles) masks[(size_t)t * W + w] = a;
      s_and[warp][w] = a;  // ~0 for tiles past the end
    }
  }
  __syncthreads();
  if (warp == 0 && lane < W) {
    u64 a = ~0ULL;
    for (int x = 0; x < tps; ++x) a &= s_and[x][lane];
    super_and[(size_t)blockIdx.x * W + lane] = a;
  }
}

// ---- bulk-copy staging: per-warp double buffer, one mbarrier per buffer ----
__device__ __forceinline__ u32 smem_addr(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(u64* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
// One 1-D bulk copy global -> shared (16-byte aligned ends, size a multiple
// of 16) that completes the transaction count of `bar`; issued by one lane.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, u32 bytes, u64* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Waits for phase `parity` of `bar` to complete, at most kWaitLimit polls;
// false when the limit ran out.
constexpr u32 kWaitLimit = 1u << 24;
__device__ __forceinline__ bool mbar_wait(u64* bar, u32 parity) {
  for (u32 it = 0; it < kWaitLimit; ++it) {
    u32 ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Tile rows TR are a template parameter (a runtime row count costs ten
// registers); tiles per super-tile (1 << tps_log2) and the block's warps
// (blockDim.x / 32) are runtime parameters.
template <int W, int MODE, int TR>
__global__ void __launch_bounds__(kMaxScanWarps * 32) k_subset_scan(const u64* __restrict__ S, u32 m,
                                                                    const u64* __restrict__ masks,
                                                                    u32 tiles_per_chunk, const u64* __restrict__ Q,
                                                                    u32 q, int n, u32* __restrict__ flags,
                                                                    u32* witness, int stop,
                                                                    u64* __restrict__ bytes_ctr, u32* err,
                                                                    int tps_log2) {
  // per warp: two tile buffers of tile_rows rows, filled by bulk copies
  extern __shared__ __align__(128) u64 s_tiles[];  // [warps][2][tile_rows * W]
  __shared__ __align__(8) u64 s_bar[kMaxScanWarps][2];
  constexpr u32 kTileRows = TR;
  constexpr int tr_log2 = TR == 32 ? 5 : TR == 64 ? 6 : 7;
  static_assert(TR == 32 || TR == 64 || TR == 128, "tile rows");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const u32 qi = (blockIdx.x * warps + warp) * 32 + lane;
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
  const u32 tiles = (m + kTileRows - 1) >> tr_log2;
  const u64* tile_and = masks;
  const u64* super_and = masks + (size_t)tiles * W;
  // buffer b of this warp; bit b of par = phase parity its next copy completes
  u64* const buf0 = s_tiles + (size_t)(warp * 2) * kTileRows * W;
  auto buf = [&](int b) { return buf0 + (size_t)b * kTileRows * W; };
  u64* const bar0 = &s_bar[warp][0];
  if (lane == 0) {
    mbar_init(&s_bar[warp][0]);
    mbar_init(&s_bar[warp][1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  u32 par = 0;
  const u32 t0 = blockIdx.y * tiles_per_chunk;
  const u32 t1 = min(tiles, t0 + tiles_per_chunk);
  // next tile >= from that some lane still needs (the AND of every range it
  // lies in is inside the lane's query), or t1
  auto advance = [&](u32 from) -> u32 {
    bool need_s = false;
    for (u32 t = from; t < t1; ++t) {
      if (t == from || (t & ((1u << tps_log2) - 1)) == 0) {
        const u32 sp = t >> tps_log2;
        need_s = !done;
#pragma unroll
        for (int w = 0; w < W; ++w)
          if (super_and[(size_t)sp * W + w] & ~c[w]) need_s = false;
        if (!__any_sync(kFullMask, need_s)) {
          t = min(t1, (sp + 1) << tps_log2) - 1;  // skip the rest of this super-tile
          continue;
        }
      }
      bool need = need_s && !done;
#pragma unroll
      for (int w = 0; w < W; ++w)
        if (tile_and[(size_t)t * W + w] & ~c[w]) need = false;
      if (__any_sync(kFullMask, need)) return t;
    }
    return t1;
  };
  // full tiles move as one bulk copy; the last, partial tile of S with plain loads
  auto full_tile = [&](u32 t) { return (t + 1) * kTileRows <= m; };
  auto issue = [&](u32 t, int b) {
    if (!full_tile(t)) return;
    if (lane == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of the buffer come first
      bulk_load(buf(b), S + (size_t)t * kTileRows * W, kTileRows * W * 8, bar0 + b);
    }
  };
  bool failed = false;
  auto land = [&](u32 t, int b) {  // the tile's rows are in buf[b] after this
    if (full_tile(t)) {
      if (!mbar_wait(bar0 + b, (par >> b) & 1u)) failed = true;
      par ^= 1u << b;
      failed = __any_sync(kFullMask, failed);
    } else {
      const u32 r0 = t * kTileRows, rows = m - r0;
      u64* const d = buf(b);
      for (u32 i = lane; i < rows * W; i += 32) d[i] = S[(size_t)r0 * W + i];
      // rows past the end of S never pass the word-0 test below
      for (u32 i = rows * W + lane; i < kTileRows * W; i += 32) d[i] = ~0ULL;
      __syncwarp();
    }
  };
  u32 cur = advance(t0);
  int b = 0;
  if (cur < t1) issue(cur, 0);
  u32 last_super = 0xffffffffu;
  while (cur < t1) {
    const u32 nxt = advance(cur + 1);
    if (nxt < t1) issue(nxt, b ^ 1);  // overlaps with the tests of `cur`
    land(cur, b);
    if (failed) {
      if (lane == 0) atomicExch(err, 1u);
      if (nxt < t1 && full_tile(nxt)) mbar_wait(bar0 + (b ^ 1), (par >> (b ^ 1)) & 1u);  // bounded
      return;
    }
    const u32 rows = min(kTileRows, m - cur * kTileRows);
    loaded += rows;
    bool need = !done;
#pragma unroll
    for (int w = 0; w < W; ++w)
      if (tile_and[(size_t)cur * W + w] & ~c[w]) need = false;
    const u64* my_rows = buf(b);
    // Warp-cooperative test: the lanes hold the tile's rows (lane l rows l,
    // l + 32, ...) and the warp walks only the queries that still need this
    // tile, one at a time: the query's first word is broadcast, every lane
    // tests its rows' first words against it, and ballots collect the rows
    // that pass; only those rows get the full test (their other words
    // against the broadcast query), and the first row that holds gives the
    // hit.  A tile costs a few instructions per needing query instead of a
    // pass over all its rows whenever any lane needs it.
    u32 needy = __ballot_sync(kFullMask, need);
    if (needy) {
      constexpr int kRowsPerLane = TR / 32;
      u64 r0[kRowsPerLane];
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) {
        const u32 r = (u32)t * 32 + lane;
        // rows past the end of S take no part (a query may hold every state of word 0)
        r0[t] = r < rows ? my_rows[(size_t)r * W] : ~0ULL;
      }
      while (needy) {
        const int j = __ffs(needy) - 1;
        needy &= needy - 1;
        const u64 nc0 = ~__shfl_sync(kFullMask, c[0], j);
        u32 pass[kRowsPerLane];
        u32 any_pass = 0;
#pragma unroll
        for (int t = 0; t < kRowsPerLane; ++t) {
          pass[t] = __ballot_sync(kFullMask, !(r0[t] & nc0) && (u32)t * 32 + lane < rows);
          any_pass |= pass[t];
        }
        if (!any_pass) continue;
        int hit_row = -1;
        for (int t = 0; t < kRowsPerLane; ++t) {
          if (!pass[t]) continue;  // warp-uniform
          bool sub = (pass[t] >> lane) & 1u;
          bool eq = sub && r0[t] == ~nc0;
          const u64* srow = my_rows + (size_t)((u32)t * 32 + lane) * W;
#pragma unroll
          for (int w = 1; w < W; ++w) {
            const u64 cw = __shfl_sync(kFullMask, c[w], j);  // every lane takes part in the broadcast
            if (sub) {
              const u64 sw = srow[w];
              sub = !(sw & ~cw);
              eq = eq && (sw == cw);
            }
          }
          if (MODE == kQueryProperSubset && eq) sub = false;
          const u32 hits = __ballot_sync(kFullMask, sub);
          if (hits) {
            hit_row = t * 32 + __ffs(hits) - 1;
            break;
          }
        }
        if (hit_row >= 0 && lane == j) {
          hit = true;
          done = true;
          hit_idx = cur * kTileRows + (u32)hit_row;
        }
      }
    }
    __syncwarp();  // every lane is done with buffer b before it is refilled
    if (stop && hit) {
      if (atomicCAS(witness, 0u, 1u) == 0u) {
        witness[1] = qi;
        witness[2] = hit_idx;
      }
      hit = false;  // recorded
    }
    // leave when every lane is decided or, in meet mode, once any warp met
    bool leave = __all_sync(kFullMask, done);
    const u32 sp = nxt >> tps_log2;
    if (!leave && stop && nxt < t1 && sp != last_super) {
      last_super = sp;
      u32 f = lane == 0 ? *(volatile u32*)witness : 0u;
      leave = __shfl_sync(kFullMask, f, 0) != 0;
    }
    if (leave) {
      if (nxt < t1 && full_tile(nxt)) {  // its copy is in flight: wait (bounded) before the buffer goes away
        if (!mbar_wait(bar0 + (b ^ 1), (par >> (b ^ 1)) & 1u) && lane == 0) atomicExch(err, 1u);
      }
      break;
    }
    cur = nxt;
    b ^= 1;
  }
  if (bytes_ctr && lane == 0 && loaded) atomicAdd(bytes_ctr, loaded * 8ULL * W);
  if (hit && !stop) flags[qi] = 1u;
}

size_t subset_check_temp_bytes(int W, u32 m, const ScanShape& sh) {
  const u32 mm = std::max<u32>(m, 1);
  return sizeof(u64) * (size_t)W * (n_tiles(mm, sh) + n_supers(mm, sh) + 1);
}

void launch_tile_and(int W, const u64* S, u32 m, u64* masks, const ScanShape& sh, cudaStream_t s) {
  if (!m) return;
  if (!scan_shape_valid(W, sh)) throw std::invalid_argument("range_and: invalid scan shape");
  const u32 blocks = n_supers(m, sh);
  const int threads = sh.tiles_per_super * 32;
#define SW_RA(WW) \
  case WW: k_range_and<WW><<<blocks, threads, 0, s>>>(S, m, masks, sh.tile_rows); break;
  switch (W) {
    SW_RA(1)
    SW_RA(2)
    SW_RA(3)
    SW_RA(4)
    SW_RA(5)
    SW_RA(6)
    SW_RA(7)
    SW_RA(8)
    default: throw std::runtime_error("range_and: unsupported width");
  }
#undef SW_RA
  SW_LAUNCH_CHECK();
}

void launch_subset_check(int W, int mode, const u64* S, u32 m, const u64* masks, const u64* Q, u32 q, int n,
                         u32* flags, u32* witness, bool stop, const ScanShape& sh, cudaStream_t s, u64* bytes_ctr,
                         u32* err) {
  if (!m || !q) return;
  if (!err) throw std::invalid_argument("subset check: an error word is required");
  if (!scan_shape_valid(W, sh)) throw std::invalid_argument("subset check: invalid scan shape");
  const u32 tiles = n_tiles(m, sh);
  const u32 qrows = (u32)sh.warps * 32;
  const u32 qblocks = (q + qrows - 1) / qrows;
  // split S into chunks of tiles so that the grid covers the GPU grid_factor
  // times: per-warp work varies a lot (early exits, filter hit rates), and
  // many small blocks keep the SMs busy until the slowest ones finish.  A
  // chunk keeps at least kMinChunkTiles tiles so that loading the warp's
  // queries stays amortised.
  const u32 target = (u32)sm_count_sc() * (u32)sh.grid_factor;
  u32 chunks = std::max<u32>(1, (target + qblocks - 1) / qblocks);
  chunks = std::min<u32>(chunks, std::max<u32>(1, tiles / kMinChunkTiles));
  chunks = std::min<u32>(chunks, 65535);
  const u32 per = (tiles + chunks - 1) / chunks;
  chunks = (tiles + per - 1) / per;
  dim3 grid(qblocks, chunks);
  const size_t smem = scan_smem_bytes(W, sh);
  const int tps_log2 = log2_exact(sh.tiles_per_super);
#define SW_SC_TR(WW, MM, TT)                                                                                      \
  {                                                                                                               \
    if (smem >= 32 * 1024) ensure_smem_limit((const void*)k_subset_scan<WW, MM, TT>, (int)smem);               \
    k_subset_scan<WW, MM, TT><<<grid, qrows, smem, s>>>(S, m, masks, per, Q, q, n, flags, witness, stop, bytes_ctr, \
                                                        err, tps_log2);                                          \
  }
#define SW_SC_ONE(WW, MM)                                 \
  {                                                       \
    if (sh.tile_rows == 32) SW_SC_TR(WW, MM, 32)          \
    else if (sh.tile_rows == 64) SW_SC_TR(WW, MM, 64)     \
    else SW_SC_TR(WW, MM, 128)                            \
  }
#define SW_SC(WW)                                                          \
  case WW:                                                                 \
    if (mode == kQuerySubset) SW_SC_ONE(WW, kQuerySubset)                  \
    else if (mode == kQueryProperSubset) SW_SC_ONE(WW, kQueryProperSubset) \
    else SW_SC_ONE(WW, kQueryDisjoint)                                     \
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
#undef SW_SC_ONE
#undef SW_SC_TR
  SW_LAUNCH_CHECK();
}

}  // namespace sw
