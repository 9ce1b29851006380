// Batched exact search for small automata: one persistent launch, one block
// per automaton at a time; current layers and children in shared memory,
// visited lists in a per-block global scratch (L2-resident).
//
// Blocks take automata from a shared counter until the batch is done.  Each
// automaton runs the same meet-in-the-middle search as the streamed path
// (Engine::step with duplicate-only reduction): the smaller frontier is
// expanded (forward images of F, preimages of the complements B' of the
// backward sets), the children are sorted (bitonic, in shared memory),
// children equal to a sibling or to a visited set are dropped (binary search
// in the side's sorted visited list), the survivors become the side's layer
// and are merged into its visited list, and the two current layers are
// meet-checked (f ∩ b' = ∅).  The first length with a meeting pair is the
// shortest reset length (both sides grow one layer per step and every pair
// of layer depths is checked once); the word is traced back through
// per-layer origin records.  An automaton whose lists outgrow the
// capacities, or whose search reaches the depth or length limit, is reported
// with the reason and solved again by the streamed path.
#include <mutex>

#include "algos.cuh"

namespace sw {

namespace {
constexpr int kSmThreads = 512;
constexpr int kSmMaxDepth = 256;  // layers per side

// Capacities in rows of W words.  Shared memory holds both current layers,
// the children of one step and their payloads (W = 1: 160 KiB, W = 2: 144 KiB,
// W = 3: 120 KiB, W = 4: 136 KiB); the visited lists live in global memory.
template <int W>
struct SmCaps {
  static constexpr u32 vis = 65536 / W;                  // visited rows per side
  static constexpr u32 layer = 4096 / W;                 // rows of a side's current layer
  static constexpr u32 ch = W <= 2 ? 8192 / W : 2048;    // children of one step (a power of two)
  static constexpr size_t smem = sizeof(u64) * W * (2 * layer + ch) + sizeof(u32) * ch;
};

template <int W>
__device__ __forceinline__ bool rless(const u64* a, const u64* b) {
#pragma unroll
  for (int w = W - 1; w >= 0; --w)
    if (a[w] != b[w]) return a[w] < b[w];
  return false;
}

template <int W>
__device__ __forceinline__ bool requal(const u64* a, const u64* b) {
#pragma unroll
  for (int w = 0; w < W; ++w)
    if (a[w] != b[w]) return false;
  return true;
}

// number of rows of the sorted array A[0..na) strictly less than x
template <int W>
__device__ __forceinline__ u32 lower_rank(const u64* A, u32 na, const u64* x) {
  u32 lo = 0, hi = na;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    if (rless<W>(A + (size_t)mid * W, x)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Exclusive prefix sum of one value per thread (kSmThreads); *total = sum.
__device__ u32 sm_block_scan(u32 v, u32* s_warp, u32* total) {
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
    const u32 w = lane < kSmThreads / 32 ? s_warp[lane] : 0u;
    u32 inc = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane < kSmThreads / 32) s_warp[lane] = inc - w;
    if (lane == 31) *total = inc;
  }
  __syncthreads();
  const u32 r = s_warp[warp] + x - v;
  __syncthreads();
  return r;
}
}  // namespace

template <int W>
__global__ void __launch_bounds__(kSmThreads, 1)
    k_small_batch(const SmallInstance* __restrict__ inst, u32 count, const uint8_t* __restrict__ delta_pool,
                  const uint8_t* __restrict__ seed_pool, SmallResult* results, uint8_t* words, u32 word_stride,
                  u32* origins, u64* visited, u32* counter) {
  using C = SmCaps<W>;
  extern __shared__ __align__(16) u64 sm[];
  u64* cur[2] = {sm, sm + (size_t)C::layer * W};
  u64* ch = sm + 2 * (size_t)C::layer * W;
  u32* chv = reinterpret_cast<u32*>(ch + (size_t)C::ch * W);
  // visited lists in global memory, two buffers per side (merge ping-pong)
  u64* vbase = visited + (size_t)blockIdx.x * 4 * C::vis * W;
  u64* vis[2] = {vbase, vbase + (size_t)C::vis * W};
  u64* vtmp[2] = {vbase + 2 * (size_t)C::vis * W, vbase + 3 * (size_t)C::vis * W};
  __shared__ uint8_t s_delta[1024];
  __shared__ u32 s_off[2][kSmMaxDepth + 1], s_cnt[2][kSmMaxDepth + 1];
  __shared__ u32 s_warp[32], s_total, s_best, s_inst;
  u32* org[2] = {origins + (size_t)blockIdx.x * 2 * C::vis, origins + (size_t)blockIdx.x * 2 * C::vis + C::vis};
  const u32 tid = threadIdx.x;

  for (;;) {
    if (tid == 0) s_inst = atomicAdd(counter, 1u);
    __syncthreads();
    const u32 id = s_inst;
    if (id >= count) break;
    const SmallInstance I = inst[id];
    const u32 n = I.n, k = I.k;
    for (u32 e = tid; e < n * k; e += kSmThreads) s_delta[e] = delta_pool[I.delta_off + e];
    // full set; F starts as {Q}, B as the complements of the seed singletons
    u64 full[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const int lo = 64 * w;
      full[w] = (int)n >= lo + 64 ? ~0ULL : ((int)n <= lo ? 0ULL : ((1ULL << (n - lo)) - 1));
    }
    if (tid == 0) {
#pragma unroll
      for (int w = 0; w < W; ++w) cur[0][w] = vis[0][w] = full[w];
      // seeds ascending by state: their complements descend, so fill backwards
      const u32 sc = I.seed_count;
      for (u32 i = 0; i < sc; ++i) {
        const u32 s = seed_pool[I.seed_off + i];
        u64* r = cur[1] + (size_t)(sc - 1 - i) * W;
#pragma unroll
        for (int w = 0; w < W; ++w) r[w] = full[w];
        r[s >> 6] &= ~(1ULL << (s & 63));
      }
      for (u32 i = 0; i < sc * W; ++i) vis[1][i] = cur[1][i];
      __threadfence_block();
      s_off[0][0] = s_off[1][0] = 0;
      s_cnt[0][0] = 1;
      s_cnt[1][0] = sc;
    }
    __syncthreads();
    u32 cnt[2] = {1, I.seed_count}, vcnt[2] = {1, I.seed_count}, depth[2] = {0, 0}, used[2] = {0, 0};
    u32 status = 2, length = 0, fi = 0, bj = 0, why = 0;
    if (I.seed_count == 0 || I.seed_count > C::layer) status = I.seed_count ? 1 : 2;
    for (u32 rt = 0; status == 2 && I.seed_count && I.seed_count <= C::layer && rt < I.max_len; ++rt) {
      const int X = cnt[0] <= cnt[1] ? 0 : 1;  // expand the smaller frontier
      const u32 m = cnt[X], c = m * k;
      if (c > C::ch || depth[X] + 1 > (u32)kSmMaxDepth) {
        status = 1;
        why = c > C::ch ? 1u : 4u;
        break;
      }
      u32 N = 2;
      while (N < c) N <<= 1;
      // expand: child e = letter * m + parent
      for (u32 e = tid; e < N; e += kSmThreads) {
        u64* out = ch + (size_t)e * W;
        if (e < c) {
          const u32 a = e / m, i = e - a * m;
          const u64* p = cur[X] + (size_t)i * W;
          u64 r[W];
#pragma unroll
          for (int w = 0; w < W; ++w) r[w] = 0;
          if (X == 0) {  // image
#pragma unroll
            for (int w = 0; w < W; ++w) {
              u64 v = p[w];
              while (v) {
                const u32 q = 64 * w + __ffsll((long long)v) - 1;
                v &= v - 1;
                const u32 d = s_delta[q * k + a];
                r[d >> 6] |= 1ULL << (d & 63);
              }
            }
          } else {  // preimage of a complement row is the complement of the preimage
            for (u32 q = 0; q < n; ++q) {
              const u32 d = s_delta[q * k + a];
              if ((p[d >> 6] >> (d & 63)) & 1ULL) r[q >> 6] |= 1ULL << (q & 63);
            }
          }
#pragma unroll
          for (int w = 0; w < W; ++w) out[w] = r[w];
          chv[e] = e;
        } else {
#pragma unroll
          for (int w = 0; w < W; ++w) out[w] = ~0ULL;
          chv[e] = 0xffffffffu;  // padding sorts after every child (payload breaks ties)
        }
      }
      __syncthreads();
      // bitonic sort of (row, payload), ascending
      for (u32 kk = 2; kk <= N; kk <<= 1)
        for (u32 j = kk >> 1; j > 0; j >>= 1) {
          for (u32 t = tid; t < N / 2; t += kSmThreads) {
            const u32 lo = 2 * j * (t / j) + (t % j), hi = lo + j;
            const bool up = (lo & kk) == 0;
            u64* a = ch + (size_t)lo * W;
            u64* b = ch + (size_t)hi * W;
            const bool a_gt = rless<W>(b, a) || (requal<W>(a, b) && chv[lo] > chv[hi]);
            if (a_gt == up) {
#pragma unroll
              for (int w = 0; w < W; ++w) {
                const u64 x = a[w];
                a[w] = b[w];
                b[w] = x;
              }
              const u32 y = chv[lo];
              chv[lo] = chv[hi];
              chv[hi] = y;
            }
          }
          __syncthreads();
        }
      // keep: first of its run of equal rows and not visited; contiguous chunks per thread
      const u32 per = (c + kSmThreads - 1) / kSmThreads;
      const u32 e0 = min(c, tid * per), e1 = min(c, e0 + per);
      u32 mine = 0;
      for (u32 e = e0; e < e1; ++e) {
        const u64* x = ch + (size_t)e * W;
        const bool dup = e > 0 && requal<W>(x, ch + (size_t)(e - 1) * W);
        if (dup) continue;
        const u32 r = lower_rank<W>(vis[X], vcnt[X], x);
        if (r < vcnt[X] && requal<W>(vis[X] + (size_t)r * W, x)) continue;
        ++mine;
      }
      u32 pos = sm_block_scan(mine, s_warp, &s_total);
      const u32 f = s_total;
      if (f > C::layer || vcnt[X] + f > C::vis || used[X] + f > C::vis) {
        status = 1;
        why = f > C::layer ? 2u : 3u;
        break;
      }
      const u32 off = used[X];
      for (u32 e = e0; e < e1; ++e) {
        const u64* x = ch + (size_t)e * W;
        const bool dup = e > 0 && requal<W>(x, ch + (size_t)(e - 1) * W);
        if (dup) continue;
        const u32 r = lower_rank<W>(vis[X], vcnt[X], x);
        if (r < vcnt[X] && requal<W>(vis[X] + (size_t)r * W, x)) continue;
        u64* o = cur[X] + (size_t)pos * W;
#pragma unroll
        for (int w = 0; w < W; ++w) o[w] = x[w];
        org[X][off + pos] = chv[e];
        ++pos;
      }
      __syncthreads();
      // visited := visited ∪ layer (both sorted, disjoint), into the other buffer
      const u32 vc = vcnt[X];
      for (u32 t = tid; t < vc + f; t += kSmThreads) {
        const u64* x;
        u32 p;
        if (t < vc) {
          x = vis[X] + (size_t)t * W;
          p = t + lower_rank<W>(cur[X], f, x);
        } else {
          x = cur[X] + (size_t)(t - vc) * W;
          p = (t - vc) + lower_rank<W>(vis[X], vc, x);
        }
#pragma unroll
        for (int w = 0; w < W; ++w) vtmp[X][(size_t)p * W + w] = x[w];
      }
      {
        u64* t = vis[X];
        vis[X] = vtmp[X];
        vtmp[X] = t;
      }
      __syncthreads();
      ++depth[X];
      if (tid == 0) {
        s_off[X][depth[X]] = off;
        s_cnt[X][depth[X]] = f;
        s_best = 0xffffffffu;
      }
      used[X] += f;
      vcnt[X] = vc + f;
      cnt[X] = f;
      __syncthreads();
      if (f == 0) break;  // a side died out: no reset word within reach
      // meet check of the current layers: some f ∩ b' = ∅
      const u32 nf = cnt[0], nb = cnt[1], pairs = nf * nb;
      for (u32 p = tid; p < pairs; p += kSmThreads) {
        const u32 i = p / nb, j = p - i * nb;
        const u64* a = cur[0] + (size_t)i * W;
        const u64* b = cur[1] + (size_t)j * W;
        bool disjoint = true;
#pragma unroll
        for (int w = 0; w < W; ++w) disjoint = disjoint && !(a[w] & b[w]);
        if (disjoint) atomicMin(&s_best, p);
      }
      __syncthreads();
      const u32 best = s_best;
      __syncthreads();
      if (best != 0xffffffffu) {
        status = 0;
        length = rt + 1;
        fi = best / nb;
        bj = best - fi * nb;
      }
    }
    // word: forward letters from depth 1 up, then backward letters from the top down
    if (tid == 0) {
      SmallResult R;
      R.status = status;
      R.length = length;
      R.word_len = 0;
      R.why = why | ((depth[0] + depth[1]) << 8);
      if (status == 0 && length <= word_stride) {
        uint8_t* wout = words + (size_t)id * word_stride;
        u32 idx = fi;
        for (u32 d = depth[0]; d >= 1; --d) {
          const u32 o = org[0][s_off[0][d] + idx], pc = s_cnt[0][d - 1];
          wout[d - 1] = (uint8_t)(o / pc);
          idx = o % pc;
        }
        idx = bj;
        u32 wpos = depth[0];
        for (u32 d = depth[1]; d >= 1; --d) {
          const u32 o = org[1][s_off[1][d] + idx], pc = s_cnt[1][d - 1];
          wout[wpos++] = (uint8_t)(o / pc);
          idx = o % pc;
        }
        R.word_len = wpos;
      } else if (status == 0) {
        R.status = 1;  // word longer than the buffer: solved again by the streamed path
        R.why = 5;
      }
      results[id] = R;
    }
    __syncthreads();
  }
}

namespace {
u32 vis_cap(int W) {
  switch (W) {
    case 1: return SmCaps<1>::vis;
    case 2: return SmCaps<2>::vis;
    case 3: return SmCaps<3>::vis;
    case 4: return SmCaps<4>::vis;
  }
  throw std::runtime_error("small batch: unsupported width");
}
}  // namespace

size_t small_batch_origin_words(int W, u32 blocks) { return (size_t)blocks * 2 * vis_cap(W); }

size_t small_batch_visited_words(int W, u32 blocks) { return (size_t)blocks * 4 * vis_cap(W) * W; }

int small_batch_blocks() { return device_sm_count(); }

void small_batch_prepare() {
  ensure_smem_limit((const void*)k_small_batch<1>, (int)SmCaps<1>::smem);
  ensure_smem_limit((const void*)k_small_batch<2>, (int)SmCaps<2>::smem);
  ensure_smem_limit((const void*)k_small_batch<3>, (int)SmCaps<3>::smem);
  ensure_smem_limit((const void*)k_small_batch<4>, (int)SmCaps<4>::smem);
}

void launch_small_batch(int W, const SmallInstance* inst, u32 count, const uint8_t* delta_pool,
                        const uint8_t* seed_pool, SmallResult* results, uint8_t* words, u32 word_stride, u32* origins,
                        u64* visited, u32 blocks, u32* counter, cudaStream_t s) {
  if (!count) return;
  SW_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  small_batch_prepare();
#define SW_SMALL(WW)                                                                                              \
  k_small_batch<WW><<<blocks, kSmThreads, SmCaps<WW>::smem, s>>>(inst, count, delta_pool, seed_pool, results, words, \
                                                                 word_stride, origins, visited, counter)
  switch (W) {
    case 1: SW_SMALL(1); break;
    case 2: SW_SMALL(2); break;
    case 3: SW_SMALL(3); break;
    case 4: SW_SMALL(4); break;
    default: throw std::runtime_error("small batch: unsupported width");
  }
#undef SW_SMALL
  SW_LAUNCH_CHECK();
}

}  // namespace sw
