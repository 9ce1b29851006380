// Device-resident exact search: one thread-block cluster per automaton of up
// to 256 states, the whole meet-in-the-middle search in one persistent launch.
//
// The streamed path (exact.cu) drives every BFS level from the host: an
// expansion, a sort, a compaction, a merge and a subset check per level, each
// a launch, with the counts read back in between.  For random automata with a
// few hundred states the lists hold thousands to a few hundred thousand sets,
// so those launches are latency-bound.  Here a cluster of CTAs keeps the
// level loop on the device:
//   * the lists of both sides live in a per-cluster global region (L2
//     resident at these sizes); the CTAs of the cluster split every phase and
//     meet at hardware cluster barriers (barrier.cluster, release/acquire);
//   * expansion is warp-per-parent with ballots (images through the inverse
//     transition lists, preimages of complements through δ), the tables
//     staged in shared memory by every CTA;
//   * duplicate removal uses two open-addressing hash sets in global memory
//     instead of a sort: one over the side's visited rows (every earlier
//     layer) and one over the children of the step.  Slots are tagged with a
//     number unique to the search (visited) or the step (children), so no
//     table is cleared between automata or steps;
//   * the meet check f ⊆ B (f ∩ b' = ∅) stages the backward layer bit-sliced:
//     for every state q a bitmap over the layer's rows (bit j set when q lies
//     in B_j), built in shared memory by a ballot transpose.  A warp then takes
//     one forward set f at a time and ANDs the bitmaps of f's states, rarest
//     first, 32 rows per lane-word, stopping as soon as every word is zero; a
//     word still nonzero when f's states run out names a B_j ⊇ f;
//   * the word is traced back through per-layer origin records.
// The search is the one k_small_batch (batch_small.cu) runs, with the same
// exactness argument: one side grows by one layer per step, every total
// length is checked once, and a set equal to one of an earlier layer of its
// side is dropped (a shorter prefix reaches it).  An automaton whose lists
// outgrow the capacities, or whose search reaches the depth or length limit,
// is reported with the reason and solved again by the streamed path.
//
// Replaces, for these sizes, the reference's MeetInTheMiddle::run loop
// (synchrolib/algorithm/exact/meet_in_the_middle.cpp:58-107) with its BFS /
// IBFS steps (:179-344) and goal check (:90).
#include <algorithm>
#include <mutex>
#include <set>
#include <utility>

#include "algos.cuh"

namespace sw {

namespace {
constexpr int kCtThreads = 1024;
constexpr int kCtWarps = kCtThreads / 32;
constexpr u32 kCtMaxDepth = 1024;   // layers per side
constexpr u32 kCtChunkRows = 4096;  // backward rows per bit-sliced meet-check chunk
constexpr u32 kCtGroups = kCtChunkRows / 32;  // 32-row bitmap words per state and chunk
constexpr u32 kCtFSlice = 32 * kCtWarps;  // forward sets per meet-check unit (32 per warp)
constexpr u32 kCtMaxNK = 4096;      // n * k of the transition table staged per CTA
constexpr u32 kRunning = 255;

__device__ __forceinline__ u32 cluster_rank() {
  u32 r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ u32 cluster_ctas() {
  u32 r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ u32 cluster_index() {
  u32 r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster arrives and waits; the arrive
// releases and the wait acquires at cluster scope, so global-memory writes made
// before the barrier by any CTA of the cluster are visible after it.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ u32 ld_volatile(const u32* p) { return *(const volatile u32*)p; }
__device__ __forceinline__ u64 ld_volatile64(const u64* p) { return *(const volatile u64*)p; }

template <int W>
__device__ __forceinline__ u64 row_hash(const u64* x) {
  u64 h = 0x243F6A8885A308D3ULL;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    h ^= x[w];
    h *= 0x9E3779B97F4A7C15ULL;
    h ^= h >> 29;
  }
  h *= 0xD6E8FEB86659FD93ULL;
  return h ^ (h >> 32);
}

template <int W>
__device__ __forceinline__ bool row_eq(const u64* a, const u64* b) {
  bool e = true;
#pragma unroll
  for (int w = 0; w < W; ++w) e = e && (a[w] == b[w]);
  return e;
}

// Per-cluster control words (one 256-byte block per cluster index).
struct ClusterCtl {
  u32 inst;       // automaton being solved
  u32 vtag;       // tag of this search's visited-table entries
  u32 ltag;       // tag of this step's child-table entries
  u32 fcount[2];  // kept children of the step (by step parity)
  u32 overflow;   // a table probe ran out (never expected: tables hold twice their rows)
  u32 found;      // meet flag
  u32 fi, bj;     // meeting pair: index in the current F layer, in the current B layer
  u32 pad[55];
};
static_assert(sizeof(ClusterCtl) == 256, "control block is one 256-byte line");

}  // namespace

// Byte offsets of one cluster's region (set width W, capacities c).  The hash
// tables come first, at offsets that depend on the capacities only: a launch of
// any width and any cluster count finds every table slot either zero or holding
// a tag an earlier search took, never row data of another layout read as a tag.
struct ClusterRegion {
  size_t vtab[2], ltab, meta, vis[2], org[2], ch, bytes;
};

template <int W>
__host__ __device__ inline ClusterRegion cluster_region(const ClusterCaps& c) {
  ClusterRegion r{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 255) & ~(size_t)255;
    return at;
  };
  r.vtab[0] = take(sizeof(u64) << c.vtab_bits);
  r.vtab[1] = take(sizeof(u64) << c.vtab_bits);
  r.ltab = take(sizeof(u64) << c.ltab_bits);
  r.meta = take(sizeof(u32) * 4 * (kCtMaxDepth + 1));
  r.vis[0] = take(sizeof(u64) * W * (size_t)c.vis);
  r.vis[1] = take(sizeof(u64) * W * (size_t)c.vis);
  r.org[0] = take(sizeof(u32) * (size_t)c.vis);
  r.org[1] = take(sizeof(u32) * (size_t)c.vis);
  r.ch = take(sizeof(u64) * W * (size_t)c.ch);
  r.bytes = o;
  return r;
}

// Scratch = header (tag counter, then one control block per cluster index, for
// kCtMaxClusters clusters) + one region per cluster, every region as large as
// the widest (W = 4) layout needs.
constexpr u32 kCtMaxClusters = 512;
constexpr size_t kCtHeaderBytes = 256 + 256 * (size_t)kCtMaxClusters;

template <int W>
__global__ void __launch_bounds__(kCtThreads, 1)
    k_cluster_batch(const SmallInstance* __restrict__ inst, u32 count, const uint8_t* __restrict__ delta_pool,
                    const uint8_t* __restrict__ seed_pool, SmallResult* results, uint8_t* words, u32 word_stride,
                    uint8_t* scratch, size_t region_stride, ClusterCaps caps, u32* counter, u64* stats) {
  extern __shared__ __align__(16) u32 s_col[];   // bitmaps: s_col[q * kCtGroups + g], q < 64 W
  __shared__ uint8_t s_delta[kCtMaxNK];          // delta[q * k + a]
  __shared__ uint8_t s_isrc[kCtMaxNK];           // preimage lists, letter-major CSR
  __shared__ u32 s_ibeg[kCtMaxNK + 16 + 1];      // list of (a, t): [s_ibeg[a*(n+1)+t], s_ibeg[a*(n+1)+t+1])
  __shared__ u32 s_fill[kCtMaxNK];
  __shared__ u64 s_par[kCtWarps][W];
  __shared__ u32 s_flag;

  const u32 rank = cluster_rank(), CS = cluster_ctas();
  const u32 tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const u32 gtid = rank * kCtThreads + tid, G = CS * kCtThreads;
  const u32 gwarp = gtid >> 5, NW = G >> 5;

  u32* tag_counter = reinterpret_cast<u32*>(scratch);
  ClusterCtl* ctl = reinterpret_cast<ClusterCtl*>(scratch + 256) + cluster_index();
  uint8_t* base = scratch + kCtHeaderBytes + (size_t)cluster_index() * region_stride;
  const ClusterRegion R = cluster_region<W>(caps);
  u32* meta = reinterpret_cast<u32*>(base + R.meta);  // layer offsets and counts per side and depth
  u32* const m_off0 = meta;
  u32* const m_off1 = meta + (kCtMaxDepth + 1);
  u32* const m_cnt0 = meta + 2 * (kCtMaxDepth + 1);
  u32* const m_cnt1 = meta + 3 * (kCtMaxDepth + 1);
  u64* const V0 = reinterpret_cast<u64*>(base + R.vis[0]);
  u64* const V1 = reinterpret_cast<u64*>(base + R.vis[1]);
  u32* const org0 = reinterpret_cast<u32*>(base + R.org[0]);
  u32* const org1 = reinterpret_cast<u32*>(base + R.org[1]);
  u64* const ch = reinterpret_cast<u64*>(base + R.ch);
  u64* const vt0 = reinterpret_cast<u64*>(base + R.vtab[0]);
  u64* const vt1 = reinterpret_cast<u64*>(base + R.vtab[1]);
  u64* const lt = reinterpret_cast<u64*>(base + R.ltab);
  const u32 vmask = (1u << caps.vtab_bits) - 1, lmask = (1u << caps.ltab_bits) - 1;

  for (;;) {
    if (rank == 0 && tid == 0) {
      ctl->inst = atomicAdd(counter, 1u);
      ctl->vtag = atomicAdd(tag_counter, 1u) + 1u;
      ctl->fcount[0] = ctl->fcount[1] = 0;
      ctl->overflow = 0;
      ctl->found = 0;
    }
    cluster_barrier();
    const u32 id = ld_volatile(&ctl->inst);
    if (id >= count) break;  // the same value in every CTA: the cluster leaves together
    const u32 vtag = ld_volatile(&ctl->vtag);
    const SmallInstance I = inst[id];
    const u32 n = I.n, k = I.k, sc = I.seed_count;
    // transition table and its inverse lists, per CTA: the preimages of t
    // under a are s_isrc[s_ibeg[a*(n+1)+t] .. s_ibeg[a*(n+1)+t+1])
    for (u32 e = tid; e < n * k; e += kCtThreads) s_delta[e] = delta_pool[I.delta_off + e];
    for (u32 e = tid; e < k * (n + 1); e += kCtThreads) s_ibeg[e] = 0;
    for (u32 e = tid; e < n * k; e += kCtThreads) s_fill[e] = 0;
    __syncthreads();
    for (u32 e = tid; e < n * k; e += kCtThreads) {
      const u32 q = e / k, a = e - q * k;
      atomicAdd(&s_ibeg[a * (n + 1) + s_delta[e] + 1], 1u);  // in-degree of t, one entry to the right
    }
    __syncthreads();
    if (tid < k) {  // running sum per letter: start of t's list, from a * n
      u32 run = tid * n;
      for (u32 t = 0; t <= n; ++t) {
        run += s_ibeg[tid * (n + 1) + t];
        s_ibeg[tid * (n + 1) + t] = run;
      }
    }
    __syncthreads();
    for (u32 e = tid; e < n * k; e += kCtThreads) {
      const u32 q = e / k, a = e - q * k, t = s_delta[e];
      const u32 slot = atomicAdd(&s_fill[a * n + t], 1u);
      s_isrc[s_ibeg[a * (n + 1) + t] + slot] = (uint8_t)q;
    }
    __syncthreads();
    u32 status = kRunning, why = 0, length = 0;
    if (sc == 0 || sc > caps.vis) {
      status = 1;
      why = 3;
    }
    // seeds: F = {Q}, B = complements of the seed singletons (rows written by rank 0)
    if (rank == 0 && status == kRunning) {
      for (u32 i = tid; i < 1 + sc; i += kCtThreads) {
        const int s = i == 0 ? -1 : (int)seed_pool[I.seed_off + i - 1];
        u64* row = i == 0 ? V0 : V1 + (size_t)(i - 1) * W;
#pragma unroll
        for (int w = 0; w < W; ++w)
          row[w] = valid_mask((int)n, w) & ~(s >= 0 && state_word(s) == w ? state_bit(s) : 0ULL);
      }
      if (tid == 0) {
        m_off0[0] = m_off1[0] = 0;
        m_cnt0[0] = 1;
        m_cnt1[0] = sc;
      }
    }
    cluster_barrier();
    // the seed rows enter the visited tables
    if (status == kRunning) {
      for (u32 j = gtid; j < 1 + sc; j += G) {
        u64* const vtS = j == 0 ? vt0 : vt1;
        const u32 r = j == 0 ? 0 : j - 1;
        const u64* x = (j == 0 ? V0 : V1) + (size_t)r * W;
        u32 slot = (u32)row_hash<W>(x) & vmask;
        const u64 mine = ((u64)vtag << 32) | r;
        for (u32 it = 0; it <= vmask; ++it) {
          const u64 v = ld_volatile64(&vtS[slot]);
          if ((u32)(v >> 32) != vtag && atomicCAS(&vtS[slot], v, mine) == v) break;
          slot = (slot + 1) & vmask;
          if (it == vmask) atomicExch(&ctl->overflow, 1u);
        }
      }
    }
    // per-side counters, identical in every thread of the cluster
    u32 cnt0 = 1, cnt1 = sc, used0 = 1, used1 = sc, cur0 = 0, cur1 = 0, depth0 = 0, depth1 = 0;
    u64 my_pairs = 0, my_children = 0, my_staged = 0;
    u32 steps = 0;
    // cycles between the cluster barriers, per phase (rank 0, thread 0): stats[4..8]
    long long clk = clock64();
    u64 ph[5] = {0, 0, 0, 0, 0};
    auto lap = [&](int i) {
      const long long t = clock64();
      ph[i] += (u64)(t - clk);
      clk = t;
    };
    for (u32 rt = 0; status == kRunning; ++rt) {
      if (rt >= I.max_len) {
        status = 2;
        break;
      }
      const int X = cnt0 <= cnt1 ? 0 : 1;  // expand the smaller frontier
      u64* const VX = X ? V1 : V0;
      u32* const orgX = X ? org1 : org0;
      u64* const vtX = X ? vt1 : vt0;
      const u32 m = X ? cnt1 : cnt0;
      const u32 usedX = X ? used1 : used0;
      const u32 curX = X ? cur1 : cur0;
      const u32 depthX = X ? depth1 : depth0;
      const u64 c64 = (u64)m * k;
      if (c64 > caps.ch || usedX + c64 > caps.vis || depthX + 1 > kCtMaxDepth) {
        status = 1;
        why = c64 > caps.ch ? 1u : (depthX + 1 > kCtMaxDepth ? 4u : 3u);
        break;
      }
      const u32 c = (u32)c64;
      if (rank == 0 && tid == 0) ctl->ltag = atomicAdd(tag_counter, 1u) + 1u;
      // ---- expansion: warp per parent, lane per pair of states of each word ----
      const u64* P = VX + (size_t)curX * W;
      for (u32 p = gwarp; p < m; p += NW) {
        if (lane < (u32)W) s_par[warp][lane] = P[(size_t)p * W + lane];
        __syncwarp();
        for (u32 a = 0; a < k; ++a) {
          u64 out_w = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) {
            u32 b[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const u32 s = 64 * w + 32 * h + lane;
              bool bit = false;
              if (s < n) {
                if (X == 1) {  // preimage of a complement row: s with δ(s, a) in the row
                  const u32 d = s_delta[s * k + a];
                  bit = (s_par[warp][d >> 6] >> (63 - (d & 63))) & 1ULL;
                } else {  // image: some preimage of s under a lies in the row
                  const u32 b0 = s_ibeg[a * (n + 1) + s], b1 = s_ibeg[a * (n + 1) + s + 1];
                  for (u32 j = b0; j < b1 && !bit; ++j) {
                    const u32 q = s_isrc[j];
                    bit = (s_par[warp][q >> 6] >> (63 - (q & 63))) & 1ULL;
                  }
                }
              }
              b[h] = __ballot_sync(0xffffffffu, bit);
            }
            // lane l decided state 64w + l (bit 63 - l) and 64w + 32 + l (bit 31 - l)
            const u64 word = ((u64)__brev(b[0]) << 32) | (u64)__brev(b[1]);
            if (lane == (u32)w) out_w = word;
          }
          if (lane < (u32)W) ch[((size_t)a * m + p) * W + lane] = out_w;
        }
        __syncwarp();
      }
      cluster_barrier();
      lap(0);
      const u32 ltag = ld_volatile(&ctl->ltag);
      // ---- duplicates: drop children equal to a visited row or to a sibling ----
      const u32 par = rt & 1u;
      if (rank == 0 && tid == 0) ctl->fcount[par ^ 1u] = 0;
      for (u32 e0 = gwarp * 32; e0 < c; e0 += G) {
        const u32 e = e0 + lane;
        bool keep = false;
        u64 x[W];
        if (e < c) {
#pragma unroll
          for (int w = 0; w < W; ++w) x[w] = ch[(size_t)e * W + w];
          const u64 h = row_hash<W>(x);
          bool seen = false;
          u32 slot = (u32)h & vmask;
          for (u32 it = 0; it <= vmask; ++it) {
            const u64 v = ld_volatile64(&vtX[slot]);
            if ((u32)(v >> 32) != vtag) break;
            if (row_eq<W>(VX + (size_t)(u32)v * W, x)) {
              seen = true;
              break;
            }
            slot = (slot + 1) & vmask;
          }
          if (!seen) {
            const u64 mine = ((u64)ltag << 32) | e;
            slot = (u32)h & lmask;
            for (u32 it = 0; it <= lmask; ++it) {
              u64 v = ld_volatile64(&lt[slot]);
              if ((u32)(v >> 32) != ltag) {
                const u64 old = atomicCAS(&lt[slot], v, mine);
                if (old == v) {
                  keep = true;
                  break;
                }
                v = old;  // taken meanwhile (by a child of this step)
              }
              if ((u32)(v >> 32) == ltag && row_eq<W>(ch + (size_t)(u32)v * W, x)) break;  // a sibling
              slot = (slot + 1) & lmask;
              if (it == lmask) atomicExch(&ctl->overflow, 1u);
            }
          }
        }
        const u32 kmask = __ballot_sync(0xffffffffu, keep);
        u32 pos0 = 0;
        if (lane == 0 && kmask) pos0 = atomicAdd(&ctl->fcount[par], (u32)__popc(kmask));
        pos0 = __shfl_sync(0xffffffffu, pos0, 0);
        if (keep) {
          const u32 r = usedX + pos0 + __popc(kmask & ((1u << lane) - 1u));
#pragma unroll
          for (int w = 0; w < W; ++w) VX[(size_t)r * W + w] = x[w];
          orgX[r] = e;
        }
      }
      my_children += c;
      cluster_barrier();
      lap(1);
      const u32 f = ld_volatile(&ctl->fcount[par]);
      // ---- the kept rows join the side's visited table ----
      for (u32 j = gtid; j < f; j += G) {
        const u32 r = usedX + j;
        const u64* x = VX + (size_t)r * W;
        u32 slot = (u32)row_hash<W>(x) & vmask;
        const u64 mine = ((u64)vtag << 32) | r;
        for (u32 it = 0; it <= vmask; ++it) {
          const u64 v = ld_volatile64(&vtX[slot]);
          if ((u32)(v >> 32) != vtag && atomicCAS(&vtX[slot], v, mine) == v) break;
          slot = (slot + 1) & vmask;
          if (it == vmask) atomicExch(&ctl->overflow, 1u);
        }
      }
      if (rank == 0 && tid == 0) {
        (X ? m_off1 : m_off0)[depthX + 1] = usedX;
        (X ? m_cnt1 : m_cnt0)[depthX + 1] = f;
      }
      cluster_barrier();
      lap(2);
      if (X) {
        cur1 = usedX;
        used1 = usedX + f;
        cnt1 = f;
        depth1 = depthX + 1;
      } else {
        cur0 = usedX;
        used0 = usedX + f;
        cnt0 = f;
        depth0 = depthX + 1;
      }
      ++steps;
      if (ld_volatile(&ctl->overflow)) {
        status = 1;
        why = 6;
        break;
      }
      if (f == 0) {  // a side died out: no reset word within reach
        status = 2;
        break;
      }
      // ---- meet check of the current layers: some f ⊆ B_j (f ∩ b'_j = ∅) ----
      const u32 nF = cnt0, nB = cnt1;
      const u64* Frows = V0 + (size_t)cur0 * W;
      const u64* Brows = V1 + (size_t)cur1 * W;  // complements b' = Q \ B
      const u32 chunks = (nB + kCtChunkRows - 1) / kCtChunkRows;
      const u32 fslices = (nF + kCtFSlice - 1) / kCtFSlice;
      const u32 units = chunks * fslices;
      my_pairs += (u64)nF * nB;
      u32 staged = 0xffffffffu;
      // Block barriers only around restaging a chunk (every warp of the CTA
      // walks the same unit sequence); a warp that sees the meet flag set
      // skips its remaining work but still takes part in those barriers.
      bool met = false;
      for (u32 u = rank; u < units; u += CS) {
        const u32 chunk = u / fslices, fs = u - chunk * fslices;
        const u32 r0 = chunk * kCtChunkRows;
        const u32 rows = min(kCtChunkRows, nB - r0);
        const u32 groups = (rows + 31) / 32;
        if (chunk != staged) {
          if (tid == 0) s_flag = ld_volatile(&ctl->found);
          __syncthreads();  // every warp is done with the previous chunk
          if (s_flag != 0) break;  // block-uniform: the meet was found
          // transpose: bit j of s_col[q * kCtGroups + g] says state q lies in
          // B_{r0 + 32 g + j}; warp per 32-row group, one ballot per state
          for (u32 g = warp; g < groups; g += kCtWarps) {
            const u32 r = 32 * g + lane;
            u64 b[W];
#pragma unroll
            for (int w = 0; w < W; ++w)
              b[w] = r < rows ? ~Brows[(size_t)(r0 + r) * W + w] & valid_mask((int)n, w) : 0ULL;
#pragma unroll
            for (int w = 0; w < W; ++w) {
              u32 keep0 = 0, keep1 = 0;
#pragma unroll 8
              for (int j = 0; j < 64; ++j) {
                const u32 col = __ballot_sync(0xffffffffu, (b[w] >> (63 - j)) & 1ULL);
                if (lane == (u32)(j & 31)) {
                  if (j < 32) keep0 = col;
                  else keep1 = col;
                }
              }
              s_col[(64 * w + lane) * kCtGroups + g] = keep0;
              s_col[(64 * w + 32 + lane) * kCtGroups + g] = keep1;
            }
          }
          staged = chunk;
          my_staged += (u64)rows * W * 8;
          __syncthreads();
        }
        // warp per 32 forward sets: lane l fetches set f0 + 32 warp + l, then
        // the warp takes them one by one (broadcast by shuffle) and ANDs the
        // bitmaps of each set's states; lane l owns the chunk's 32-row words
        // 4l .. 4l + 3 (one 16-byte shared load per state)
        if (!met) {
          u32 fl = lane == 0 ? ld_volatile(&ctl->found) : 0u;
          met = __shfl_sync(0xffffffffu, fl, 0) != 0;
        }
        if (met) continue;
        const u32 fw0 = fs * kCtFSlice + warp * 32;
        const u32 fw1 = min(nF, fw0 + 32);
        u64 myf[W];
#pragma unroll
        for (int w = 0; w < W; ++w) myf[w] = fw0 + lane < fw1 ? Frows[(size_t)(fw0 + lane) * W + w] : 0ULL;
        u32 acc0[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const u32 g = 4 * lane + i;
          acc0[i] = g < groups ? (32 * g + 32 <= rows ? 0xffffffffu : (1u << (rows - 32 * g)) - 1u) : 0u;
        }
        for (u32 t = 0; fw0 + t < fw1; ++t) {
          u32 acc[4] = {acc0[0], acc0[1], acc0[2], acc0[3]};
          bool alive = true;
          // rarest states first: states are numbered by decreasing frequency,
          // so the last state of f (the lowest set bit of its last word) thins
          // the candidate rows fastest
#pragma unroll
          for (int w = W - 1; w >= 0; --w) {
            u64 v = __shfl_sync(0xffffffffu, myf[w], t);
            while (v && alive) {
              const u32 j = 63 - (__ffsll((long long)v) - 1);  // state 64 w + j (bit 63 - j)
              v &= v - 1;
              const uint4 col = reinterpret_cast<const uint4*>(s_col + (64 * w + j) * kCtGroups)[lane];
              acc[0] &= col.x;
              acc[1] &= col.y;
              acc[2] &= col.z;
              acc[3] &= col.w;
              alive = __any_sync(0xffffffffu, (acc[0] | acc[1] | acc[2] | acc[3]) != 0u);
            }
          }
          if (alive) {  // some B_j contains every state of f
            u32 hit = 0xffffffffu;
#pragma unroll
            for (int i = 3; i >= 0; --i)
              if (acc[i]) hit = 32 * (4 * lane + i) + __ffs(acc[i]) - 1;
            const u32 who = __ballot_sync(0xffffffffu, hit != 0xffffffffu);
            const u32 bj = __shfl_sync(0xffffffffu, hit, __ffs(who) - 1);
            if (lane == 0 && atomicCAS(&ctl->found, 0u, 1u) == 0u) {
              ctl->fi = fw0 + t;
              ctl->bj = r0 + bj;
            }
            break;
          }
        }
      }
      cluster_barrier();
      lap(3);
      if (ld_volatile(&ctl->found)) {
        status = 0;
        length = rt + 1;
      }
    }
    // ---- result and word (forward letters from depth 1 up, then backward letters from the top down) ----
    if (rank == 0 && tid == 0) {
      SmallResult res;
      res.status = status;
      res.length = length;
      res.word_len = 0;
      res.why = why | ((depth0 + depth1) << 8);
      if (status == 0 && length <= word_stride) {
        uint8_t* wout = words + (size_t)id * word_stride;
        u32 idx = ld_volatile(&ctl->fi);
        for (u32 d = depth0; d >= 1; --d) {
          const u32 o = org0[m_off0[d] + idx], pc = m_cnt0[d - 1];
          wout[d - 1] = (uint8_t)(o / pc);
          idx = o % pc;
        }
        idx = ld_volatile(&ctl->bj);
        u32 wpos = depth0;
        for (u32 d = depth1; d >= 1; --d) {
          const u32 o = org1[m_off1[d] + idx], pc = m_cnt1[d - 1];
          wout[wpos++] = (uint8_t)(o / pc);
          idx = o % pc;
        }
        res.word_len = wpos;
      } else if (status == 0) {
        res.status = 1;  // word longer than the buffer: solved again by the streamed path
        res.why = 5 | ((depth0 + depth1) << 8);
      }
      results[id] = res;
      if (stats) {
        atomicAdd(&stats[0], (unsigned long long)my_pairs);
        atomicAdd(&stats[1], (unsigned long long)my_children);
        atomicAdd(&stats[3], (unsigned long long)steps);
        lap(4);
        for (int i = 0; i < 5; ++i) atomicAdd(&stats[4 + i], (unsigned long long)ph[i]);
      }
    }
    if (stats && tid == 0 && my_staged) atomicAdd(&stats[2], (unsigned long long)my_staged);
    cluster_barrier();  // the trace has read this search's records before the next one overwrites them
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {
const void* cluster_fn_w(int W) {
  switch (W) {
    case 1: return (const void*)k_cluster_batch<1>;
    case 2: return (const void*)k_cluster_batch<2>;
    case 3: return (const void*)k_cluster_batch<3>;
    case 4: return (const void*)k_cluster_batch<4>;
  }
  throw std::runtime_error("cluster batch: unsupported width");
}
// bitmaps of 64 W states x kCtGroups words
size_t col_smem(int W) { return sizeof(u32) * 64 * (size_t)W * kCtGroups; }

std::mutex g_cluster_mu;
std::set<std::pair<int, const void*>> g_nonportable;  // (device, kernel) pairs opted in to clusters above 8

// Sets the kernel's attributes once per device, so that a launch issued
// while a stream is being captured makes no attribute call.
void prepare(const void* fn, int W, int cs) {
  std::lock_guard<std::mutex> g(g_cluster_mu);
  ensure_smem_limit(fn, (int)col_smem(W));
  if (cs > 8) {
    int dev = 0;
    SW_CUDA(cudaGetDevice(&dev));
    if (g_nonportable.insert({dev, fn}).second)
      SW_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
}
}  // namespace

ClusterCaps cluster_default_caps() {
  ClusterCaps c;
  c.vis = 1u << 21;
  c.ch = 1u << 20;
  c.vtab_bits = 22;  // two slots per visited row
  c.ltab_bits = 21;  // two slots per child
  return c;
}

size_t cluster_scratch_bytes(u32 clusters, const ClusterCaps& c) {
  return kCtHeaderBytes + (size_t)clusters * cluster_region<4>(c).bytes;
}

u32 cluster_max_clusters_supported() { return kCtMaxClusters; }

u32 cluster_batch_max_clusters(int W, int cs) {
  const void* fn = cluster_fn_w(W);
  prepare(fn, W, cs);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)cs * 64, 1, 1);
  cfg.blockDim = dim3(kCtThreads, 1, 1);
  cfg.dynamicSmemBytes = col_smem(W);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  SW_CUDA(cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg));
  return (u32)std::max(clusters, 0);
}

void launch_cluster_batch(int W, int cs, u32 clusters, const SmallInstance* inst, u32 count,
                          const uint8_t* delta_pool, const uint8_t* seed_pool, SmallResult* results, uint8_t* words,
                          u32 word_stride, void* scratch, const ClusterCaps& caps, u32* counter, u64* stats,
                          cudaStream_t s) {
  if (!count || !clusters) return;
  if (cs < 1 || cs > 16) throw std::invalid_argument("cluster size must be 1..16");
  if (clusters > kCtMaxClusters) throw std::invalid_argument("too many clusters for the scratch header");
  if (caps.vtab_bits > 30 || caps.ltab_bits > 30 || (1ull << caps.vtab_bits) < 2ull * caps.vis ||
      (1ull << caps.ltab_bits) < 2ull * caps.ch)
    throw std::invalid_argument("cluster batch: hash tables must hold twice their rows");
  const void* fn = cluster_fn_w(W);
  prepare(fn, W, cs);
  SW_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(cs * clusters), 1, 1);
  cfg.blockDim = dim3(kCtThreads, 1, 1);
  cfg.dynamicSmemBytes = col_smem(W);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const size_t stride = cluster_region<4>(caps).bytes;  // every width uses the widest region
  uint8_t* sc = static_cast<uint8_t*>(scratch);
  switch (W) {
    case 1:
      SW_CUDA(cudaLaunchKernelEx(&cfg, k_cluster_batch<1>, inst, count, delta_pool, seed_pool, results, words,
                                 word_stride, sc, stride, caps, counter, stats));
      break;
    case 2:
      SW_CUDA(cudaLaunchKernelEx(&cfg, k_cluster_batch<2>, inst, count, delta_pool, seed_pool, results, words,
                                 word_stride, sc, stride, caps, counter, stats));
      break;
    case 3:
      SW_CUDA(cudaLaunchKernelEx(&cfg, k_cluster_batch<3>, inst, count, delta_pool, seed_pool, results, words,
                                 word_stride, sc, stride, caps, counter, stats));
      break;
    case 4:
      SW_CUDA(cudaLaunchKernelEx(&cfg, k_cluster_batch<4>, inst, count, delta_pool, seed_pool, results, words,
                                 word_stride, sc, stride, caps, counter, stats));
      break;
    default:
      throw std::runtime_error("cluster batch: unsupported width");
  }
  SW_LAUNCH_CHECK();
}

}  // namespace sw
