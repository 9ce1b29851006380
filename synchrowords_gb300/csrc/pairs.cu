// Eppstein's greedy upper bound on one block.
//
// Reference: PairsTree::calculate_tree (synchrolib/data_structures/pairs_tree.hpp:25-62)
// and Eppstein::get_automaton_lsw_eppstein (synchrolib/algorithm/eppstein/eppstein.hpp:82-114).
//
// The reference builds its pair tree with one FIFO queue: the first layer
// scans targets t, letters a and preimage pairs (i1 < i2) of t under a; every
// later pair is discovered from the earliest queued pair that reaches it.  The
// letter it records decides which word the greedy phase applies, so the GPU
// version reproduces the queue order exactly, one BFS level per round:
//   * every candidate discovery gets a key (generator, letter, i1, i2) that
//     increases in the reference's enumeration order, the generator being the
//     target state (first layer) or n + the queue position of the parent pair;
//   * discovery:  atomicMin of the key into the candidate pair's slot;
//   * emission:   a candidate wins iff its key survived; threads own
//     contiguous generator slices, so a block-wide prefix sum of their winner
//     counts places winners in key order — the order the reference appends.
// The greedy phase then keeps the current image as a bitset in shared memory,
// finds the closest pair (ties: smallest (p, q), as the reference's strict `<`
// over p < q does) with a block-wide min, and applies that pair's letters.
#include "algos.cuh"

namespace sw {

namespace {
constexpr int kEppThreads = 1024;
constexpr int kEppWarps = kEppThreads / 32;

struct EppLayout {
  size_t best_off, len_off, queue_off, letter_off, total;
};

__host__ __device__ inline EppLayout epp_layout(int n) {
  const size_t nn = (size_t)n * n;
  EppLayout L;
  L.best_off = 0;                                        // u64[n*n]  discovery keys
  L.len_off = L.best_off + 8 * nn;                       // u32[n*n]  merge length (0 = unknown)
  L.queue_off = L.len_off + 4 * nn;                      // u32[n(n-1)/2 + 1]  pairs in queue order
  L.letter_off = L.queue_off + 4 * ((nn - n) / 2 + 1);   // u8[n*n]   first letter of the word
  L.total = L.letter_off + nn + 16;
  return L;
}

__device__ inline u64 cand_key(u32 g, u32 a, u32 i, u32 j) {
  return ((u64)g << 24) | ((u64)a << 20) | ((u64)i << 10) | (u64)j;
}

__device__ inline u32 canon(u32 p, u32 q, u32 n) { return p < q ? p * n + q : q * n + p; }

// Calls f(key, p, q, letter) for every candidate pair of generator g in the
// reference's enumeration order (pairs_tree.hpp:30-41 for g < n, :47-59 else).
template <class F>
__device__ inline void for_candidates(const TransTables& t, const u32* queue, u32 g, F&& f) {
  const u32 n = (u32)t.n;
  for (u32 a = 0; a < (u32)t.k; ++a) {
    const uint16_t* beg = t.inv_beg + a * (n + 1);
    const uint16_t* src = t.inv_src + a * n;
    if (g < n) {
      const u32 b = beg[g], e = beg[g + 1];
      for (u32 i1 = b; i1 < e; ++i1)
        for (u32 i2 = i1 + 1; i2 < e; ++i2) f(cand_key(g, a, i1 - b, i2 - b), (u32)src[i1], (u32)src[i2], a);
    } else {
      const u32 pr = queue[g - n];
      const u32 v1 = pr & 0xffffu, v2 = pr >> 16;
      const u32 b1 = beg[v1], e1 = beg[v1 + 1], b2 = beg[v2], e2 = beg[v2 + 1];
      for (u32 i1 = b1; i1 < e1; ++i1)
        for (u32 i2 = b2; i2 < e2; ++i2) f(cand_key(g, a, i1 - b1, i2 - b2), (u32)src[i1], (u32)src[i2], a);
    }
  }
}

// Exclusive prefix sum of one value per thread; *total = block sum.
__device__ u32 block_exclusive_sum(u32 v, u32* s_warp, u32* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const u32 w = lane < kEppWarps ? s_warp[lane] : 0u;
    u32 inc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane < kEppWarps) s_warp[lane] = inc - w;
    if (lane == 31) *total = inc;
  }
  __syncthreads();
  const u32 r = s_warp[warp] + x - v;
  __syncthreads();  // s_warp is reused by the next call
  return r;
}

__device__ u64 block_min(u64 v, u64* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    u64 w = lane < kEppWarps ? s_red[lane] : ~0ULL;
#pragma unroll
    for (int o = 16; o; o >>= 1) w = min(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (lane == 0) s_red[32] = w;
  }
  __syncthreads();
  const u64 r = s_red[32];
  __syncthreads();
  return r;
}
}  // namespace

__global__ void __launch_bounds__(kEppThreads, 1)
    k_eppstein(TransTables t, u64 upper, unsigned char* scratch, u32* out, uint8_t* word, u64 word_cap) {
  __shared__ u32 s_warp[32];
  __shared__ u32 s_total;
  __shared__ u64 s_red[33];
  __shared__ u64 s_cur[kMaxStates / 64], s_nxt[kMaxStates / 64];
  __shared__ uint16_t s_list[kMaxStates];
  const u32 n = (u32)t.n;
  const u32 tid = threadIdx.x;
  const EppLayout L = epp_layout((int)n);
  u64* best = reinterpret_cast<u64*>(scratch + L.best_off);
  u32* len = reinterpret_cast<u32*>(scratch + L.len_off);
  u32* queue = reinterpret_cast<u32*>(scratch + L.queue_off);
  uint8_t* letter = scratch + L.letter_off;
  const size_t nn = (size_t)n * n;
  for (size_t i = tid; i < nn; i += kEppThreads) {
    best[i] = ~0ULL;
    len[i] = 0;
  }
  __syncthreads();

  // ---- pair tree, one BFS level per round ----
  const u32 pairs_total = n * (n - 1) / 2;
  u32 top = 0, gb = 0, ge = n;  // generators [gb, ge) of this level
  for (u32 level = 1; ge > gb && top < pairs_total && level <= pairs_total; ++level) {
    for (u32 g = gb + tid; g < ge; g += kEppThreads)
      for_candidates(t, queue, g, [&](u64 key, u32 p, u32 q, u32) {
        const u32 c = canon(p, q, n);
        if (len[c] == 0) atomicMin(&best[c], key);
      });
    __syncthreads();
    const u32 G = ge - gb, per = (G + kEppThreads - 1) / kEppThreads;
    const u32 s0 = gb + min(G, tid * per), s1 = gb + min(G, (tid + 1) * per);
    u32 cnt = 0;
    for (u32 g = s0; g < s1; ++g)
      for_candidates(t, queue, g, [&](u64 key, u32 p, u32 q, u32) { cnt += best[canon(p, q, n)] == key; });
    const u32 off = block_exclusive_sum(cnt, s_warp, &s_total);
    const u32 produced = s_total;
    u32 w = top + off;
    for (u32 g = s0; g < s1; ++g)
      for_candidates(t, queue, g, [&](u64 key, u32 p, u32 q, u32 a) {
        const u32 c = canon(p, q, n);
        if (best[c] == key) {
          queue[w++] = p | (q << 16);
          len[c] = level;
          letter[c] = (uint8_t)a;
        }
      });
    __syncthreads();
    gb = n + top;
    ge = n + top + produced;
    top += produced;
  }
  if (top < pairs_total) {
    if (tid == 0) out[0] = kEppNonSynchro;
    return;
  }

  // ---- greedy: merge the closest pair of the current image ----
  if (tid < kMaxStates / 64) {
    const u32 lo = tid * 64;
    s_cur[tid] = lo >= n ? 0ULL : (n - lo >= 64 ? ~0ULL : ((1ULL << (n - lo)) - 1));
  }
  __syncthreads();
  u64 total = 0, wl = 0;
  for (u32 round = 0; round <= n; ++round) {
    u32 bit = 0;
    if (tid < n) bit = (u32)((s_cur[tid >> 6] >> (tid & 63)) & 1ULL);
    const u32 pos = block_exclusive_sum(bit, s_warp, &s_total);
    const u32 m = s_total;
    if (bit) s_list[pos] = (uint16_t)tid;
    __syncthreads();
    u64 bk = ~0ULL;
    for (u32 idx = tid; idx < m * m; idx += kEppThreads) {
      const u32 i = idx / m, j = idx - i * m;
      if (j > i) {
        const u32 c = (u32)s_list[i] * n + s_list[j];
        bk = min(bk, ((u64)len[c] << 32) | c);
      }
    }
    bk = block_min(bk, s_red);
    u32 p = 0, q = 0;
    u64 l = (u64)n * n;  // eppstein.hpp:87: no pair left keeps l = N*N
    if (bk != ~0ULL) {
      l = bk >> 32;
      p = (u32)(bk & 0xffffffffu) / n;
      q = (u32)(bk & 0xffffffffu) % n;
    }
    total += l;
    if (total > upper) {
      if (tid == 0) out[0] = kEppOverBound;
      return;
    }
    for (u32 step = 0; p != q && step <= pairs_total; ++step) {
      const u32 a = letter[canon(p, q, n)];
      if (tid == 0 && wl < word_cap) word[wl] = (uint8_t)a;
      ++wl;
      p = t.delta[a * n + p];
      q = t.delta[a * n + q];
      if (tid < kMaxStates / 64) s_nxt[tid] = 0;
      __syncthreads();
      if (tid < n && ((s_cur[tid >> 6] >> (tid & 63)) & 1ULL)) {
        const u32 d = t.delta[a * n + tid];
        atomicOr(&s_nxt[d >> 6], 1ULL << (d & 63));
      }
      __syncthreads();
      if (tid < kMaxStates / 64) s_cur[tid] = s_nxt[tid];
      __syncthreads();
    }
    u32 size = 0;
#pragma unroll
    for (int i = 0; i < kMaxStates / 64; ++i) size += __popcll(s_cur[i]);
    if (size <= 1) break;
  }
  if (tid == 0) {
    out[0] = wl > word_cap ? kEppWordCapacity : kEppFound;
    out[1] = (u32)(total & 0xffffffffu);
    out[2] = (u32)(total >> 32);
    out[3] = (u32)min(wl, word_cap);
  }
}

size_t eppstein_scratch_bytes(int n) { return epp_layout(n).total; }

void launch_eppstein(const TransTables& t, u64 upper, void* scratch, u32* out, uint8_t* word, u64 word_cap,
                     cudaStream_t s) {
  k_eppstein<<<1, kEppThreads, 0, s>>>(t, upper, static_cast<unsigned char*>(scratch), out, word, word_cap);
  SW_LAUNCH_CHECK();
}

}  // namespace sw
