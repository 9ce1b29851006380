// Device kernels of the exact search: warp-per-subset layer expansion, radix
// sort / unique, stream compaction, the binary radix tree over a sorted layer
// and the tree-walking subset queries.  All integer bitset work; see
// common.cuh for the row layout and kernels.cuh for the reference functions
// each kernel replaces.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "kernels.cuh"

namespace sw {

namespace {
std::mutex g_devinfo_mu;
}  // namespace

int device_sm_count() {
  constexpr int kMaxDev = 64;
  static int cached[kMaxDev] = {};
  int dev = 0;
  SW_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDev) {
    int sms = 0;
    SW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
  }
  std::lock_guard<std::mutex> g(g_devinfo_mu);
  if (!cached[dev]) SW_CUDA(cudaDeviceGetAttribute(&cached[dev], cudaDevAttrMultiProcessorCount, dev));
  return cached[dev];
}

cudaStream_t& alloc_stream() {
  thread_local cudaStream_t s = nullptr;
  return s;
}

AllocScope::AllocScope(cudaStream_t s) : prev(alloc_stream()) {
  // keep freed blocks in the device's default pool instead of returning them
  // to the driver at every synchronisation (this process's pool only)
  static std::mutex mu;
  static std::set<int> cached;
  int dev = 0;
  SW_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> g(mu);
    if (cached.insert(dev).second) {
      cudaMemPool_t pool;
      SW_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
      uint64_t keep = ~0ull;
      SW_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
  }
  alloc_stream() = s;
}

void ensure_smem_limit(const void* fn, int bytes) {
  static std::map<std::pair<int, const void*>, int> limits;
  int dev = 0;
  SW_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(g_devinfo_mu);
  int& cur = limits[{dev, fn}];
  if (bytes <= cur) return;
  SW_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  cur = bytes;
}

namespace {

constexpr u32 kFull = 0xffffffffu;

__device__ __forceinline__ u32 lanemask_lt() {
  u32 m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

int sm_count() { return device_sm_count(); }

template <int W>
__device__ __forceinline__ bool row_less(const u64* a, const u64* b) {
#pragma unroll
  for (int w = 0; w < W; ++w) {
    u64 x = a[w], y = b[w];
    if (x != y) return x < y;
  }
  return false;
}

template <int W>
__device__ __forceinline__ bool row_eq(const u64* a, const u64* b) {
#pragma unroll
  for (int w = 0; w < W; ++w)
    if (a[w] != b[w]) return false;
  return true;
}

}  // namespace

template <int W>
__device__ __forceinline__ u64 row_mix(const u64* r, int from) {
  u64 h = 0x9E3779B97F4A7C15ULL;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    if (w < from) continue;
    u64 x = r[w] ^ (h + 0x632BE59BD9B4E019ULL * (u64)(w + 1));
    x ^= x >> 31;
    x *= 0x94D049BB133111EBULL;
    x ^= x >> 29;
    h = (h ^ x) * 0xBF58476D1CE4E5B9ULL;
  }
  return (h ^ (h >> 32)) << 32;
}

template <int W>
__device__ __forceinline__ void layer_key(const u64* r, const KeyMap& map, u64& k0, u64& k1) {
  if (map.identity) {
    k0 = r[0];
    k1 = W > 1 ? row_mix<W>(r, 1) : 0ULL;
    return;
  }
  u64 a = 0;
#pragma unroll 8
  for (int j = 0; j < 64; ++j) {
    const int q = map.q[j];
    a |= ((r[q >> 6] >> (63 - (q & 63))) & 1ULL) << (63 - j);
  }
  k0 = a;
  k1 = row_mix<W>(r, 0);
}

// ===========================================================================
// Layer expansion.  One warp per input set.  The set row is staged in shared
// memory; lane l decides output states l, l+32, ... by a gather:
//   preimage  out[p] = S[delta_a(p)]                  (delta in smem)
//   image     out[t] = OR_{q : delta_a(q) = t} S[q]   (preimage CSR in smem)
// and each 32-state round becomes half an output word through __ballot_sync
// (bit-reversed into the MSB-first layout).  Both directions are
// gathers, so no atomics are needed.
// ===========================================================================
template <int W, bool kImage>
__global__ void __launch_bounds__(256) k_expand(const u64* __restrict__ in, u32 m, TransTables t,
                                                u64* __restrict__ out, u64* __restrict__ keys,
                                                u32* __restrict__ vals, KeyMap map) {
  extern __shared__ uint16_t s_tab[];
  __shared__ u64 s_row[8][W];
  __shared__ u64 s_out[8][W];
  const int n = t.n, k = t.k;
  uint16_t* s_a = s_tab;                  // delta (preimage) or inv_beg (image)
  uint16_t* s_b = s_tab + k * (n + 1);    // inv_src (image)
  if (kImage) {
    for (int i = threadIdx.x; i < k * (n + 1); i += blockDim.x) s_a[i] = t.inv_beg[i];
    for (int i = threadIdx.x; i < k * n; i += blockDim.x) s_b[i] = t.inv_src[i];
  } else {
    for (int i = threadIdx.x; i < k * n; i += blockDim.x) s_a[i] = t.delta[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 stride = gridDim.x * 8u;
  const int rounds = (n + 31) >> 5;
  for (u32 i = blockIdx.x * 8u + warp; i < m; i += stride) {
    if (lane < W) s_row[warp][lane] = in[(size_t)i * W + lane];
    __syncwarp();
    for (int a = 0; a < k; ++a) {
      u64 word = 0;
      for (int r = 0; r < rounds; ++r) {
        const int q = r * 32 + lane;
        bool bit = false;
        if (q < n) {
          if (kImage) {
            const int b = s_a[a * (n + 1) + q], e = s_a[a * (n + 1) + q + 1];
            for (int j = b; j < e; ++j) {
              const int p = s_b[a * n + j];
              if ((s_row[warp][p >> 6] >> (63 - (p & 63))) & 1ULL) {
                bit = true;
                break;
              }
            }
          } else {
            const int p = s_a[a * n + q];
            bit = (s_row[warp][p >> 6] >> (63 - (p & 63))) & 1ULL;
          }
        }
        const u32 bal = __ballot_sync(kFull, bit);
        if (lane == (r >> 1)) {
          const u64 v = (u64)__brev(bal);
          word |= (r & 1) ? v : (v << 32);
        }
      }
      const size_t o = (size_t)a * m + i;
      if (lane < W) out[o * W + lane] = word;
      if (keys) {  // the child's layer key and its index as the sort payload
        if (lane < W) s_out[warp][lane] = word;
        __syncwarp();
        if (lane == 0) {
          u64 k0, k1;
          layer_key<W>(s_out[warp], map, k0, k1);
          keys[2 * o] = k0;
          keys[2 * o + 1] = k1;
          vals[o] = (u32)o;
        }
        __syncwarp();
      }
    }
    __syncwarp();
  }
}

void launch_expand(int W, bool image, const u64* in, u32 m, const TransTables& t, u64* out, cudaStream_t s,
                   u64* keys, u32* vals, const KeyMap& map) {
  if (m == 0) return;
  size_t smem = image ? sizeof(uint16_t) * (size_t)t.k * (2 * t.n + 1) : sizeof(uint16_t) * (size_t)t.k * t.n;
  u32 blocks = std::min<u32>((m + 7) / 8, (u32)sm_count() * 8);
#define SW_EXP(WW)                                                                                  \
  case WW:                                                                                          \
    if (image) {                                                                                    \
      if (smem > 48 * 1024) ensure_smem_limit((const void*)k_expand<WW, true>, (int)smem);         \
      k_expand<WW, true><<<blocks, 256, smem, s>>>(in, m, t, out, keys, vals, map);                 \
    } else {                                                                                        \
      if (smem > 48 * 1024) ensure_smem_limit((const void*)k_expand<WW, false>, (int)smem);        \
      k_expand<WW, false><<<blocks, 256, smem, s>>>(in, m, t, out, keys, vals, map);                \
    }                                                                                               \
    break;
  switch (W) {
    SW_EXP(1)
    SW_EXP(2)
    SW_EXP(3)
    SW_EXP(4)
    SW_EXP(5)
    SW_EXP(6)
    SW_EXP(7)
    SW_EXP(8)
    default:
      throw std::runtime_error("expand: unsupported width");
  }
#undef SW_EXP
  SW_LAUNCH_CHECK();
}

// ===========================================================================
// Device-wide exclusive scan of u32 (three kernels: tile sums, scan of the
// tile sums in one block, tile scans with carry-in).
// ===========================================================================
namespace {
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr u32 kScanTile = kScanThreads * kScanItems;

// Exclusive scan across a 1024-thread block; returns the block total.
__device__ u32 block_exclusive_scan(u32 v, u32& total) {
  __shared__ u32 s_warp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    u32 y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    u32 w = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      u32 y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  total = s_warp[(blockDim.x >> 5) - 1];
  u32 excl = x - v + (warp ? s_warp[warp - 1] : 0);
  __syncthreads();
  return excl;
}
}  // namespace

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const u32* __restrict__ in, u32 n, u32* partial) {
  const size_t base = (size_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  u32 s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
    if (base + j < n) s += in[base + j];
  u32 tot;
  block_exclusive_scan(s, tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partials(u32* partial, u32 nb, u32* total_dev) {
  u32 carry = 0;
  for (u32 base = 0; base < nb; base += kScanTile) {
    u32 v[kScanItems];
    u32 s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      u32 idx = base + threadIdx.x * kScanItems + j;
      v[j] = idx < nb ? partial[idx] : 0;
      s += v[j];
    }
    u32 tot;
    u32 ex = block_exclusive_scan(s, tot);
    u32 run = carry + ex;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      u32 idx = base + threadIdx.x * kScanItems + j;
      if (idx < nb) partial[idx] = run;
      run += v[j];
    }
    carry += tot;
  }
  if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(const u32* __restrict__ in, u32* __restrict__ out, u32 n,
                                                             const u32* partial) {
  const size_t base = (size_t)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  u32 v[kScanItems];
  u32 s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    v[j] = (base + j < n) ? in[base + j] : 0;
    s += v[j];
  }
  u32 tot;
  u32 run = block_exclusive_scan(s, tot) + partial[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
}

size_t scan_temp_bytes(u32 n) { return sizeof(u32) * ((n + kScanTile - 1) / kScanTile + 1); }

// Small arrays: one block walks the array tile by tile with a carry.
__global__ void __launch_bounds__(kScanThreads) k_scan_onepass(const u32* __restrict__ in, u32* __restrict__ out,
                                                               u32 n, u32* total_dev) {
  u32 carry = 0;
  for (u32 base = 0; base < n; base += kScanTile) {
    u32 v[kScanItems];
    u32 s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      u32 idx = base + threadIdx.x * kScanItems + j;
      v[j] = idx < n ? in[idx] : 0;
      s += v[j];
    }
    u32 tot;
    u32 run = carry + block_exclusive_scan(s, tot);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      u32 idx = base + threadIdx.x * kScanItems + j;
      if (idx < n) out[idx] = run;
      run += v[j];
    }
    carry += tot;
  }
  if (threadIdx.x == 0 && total_dev) *total_dev = carry;
}

void launch_scan(const u32* in, u32* out, u32 n, u32* total_dev, void* temp, cudaStream_t s) {
  if (n == 0) {
    if (total_dev) SW_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(u32), s));
    return;
  }
  if (n <= 8 * kScanTile) {
    k_scan_onepass<<<1, kScanThreads, 0, s>>>(in, out, n, total_dev);
    SW_LAUNCH_CHECK();
    return;
  }
  u32 nb = (n + kScanTile - 1) / kScanTile;
  u32* partial = static_cast<u32*>(temp);
  k_scan_reduce<<<nb, kScanThreads, 0, s>>>(in, n, partial);
  k_scan_partials<<<1, kScanThreads, 0, s>>>(partial, nb, total_dev);
  k_scan_final<<<nb, kScanThreads, 0, s>>>(in, out, n, partial);
  SW_LAUNCH_CHECK();
}

// ===========================================================================
// Radix sort of rows (R words, word 0 most significant) with u32 payload.
// Stable LSD over 8-bit digits; digits that are constant over all rows are
// skipped (their OR == AND).  Large inputs: per-pass upsweep (tile digit
// counts) -> scan -> downsweep (stable in-tile rank via __match_any_sync,
// scatter of whole rows).  Inputs of at most one shared-memory tile are sorted
// by a single block in shared memory.
// ===========================================================================
namespace {
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 8;
constexpr u32 kRsTile = kRsThreads * kRsRounds;
constexpr int kSmallThreads = 1024;  // shared-memory sorts: one compare-exchange per thread per stage
constexpr u32 kMergeSortMax = 1u << 20;  // up to here: chunk sorts + merge passes; above: radix passes

// Rows of one shared-memory sort: a power of two, at most 2 * kSmallThreads.
template <int R>
constexpr u32 small_sort_max() {
  return R <= 4 ? 2048u : 1024u;
}
static_assert(2048u <= 2u * (u32)kSmallThreads, "a shared-memory sort stage is one compare-exchange per thread");
template <int R>
constexpr size_t small_sort_smem(u32 rows) {  // keys, payloads, original positions
  return (size_t)rows * (R * sizeof(u64) + 2 * sizeof(u32));
}

// Per-round stable ranking inside a 256-thread block.  `d` is this thread's
// digit (256 = no item).  s_base[256] carries counts of earlier rounds,
// s_wcnt[8][256] is scratch.  Returns the item's rank among equal digits in
// the block so far.
__device__ __forceinline__ u32 block_round_rank(u32 d, u32* s_base, u32 (*s_wcnt)[256]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 peers = __match_any_sync(kFull, d);
  const u32 lrank = __popc(peers & lanemask_lt());
#pragma unroll
  for (int j = 0; j < 8; ++j) s_wcnt[warp][lane * 8 + j] = 0;
  __syncwarp();
  if (d < 256 && lrank == 0) s_wcnt[warp][d] = __popc(peers);
  __syncthreads();
  {
    const int t = threadIdx.x;  // digit owned by this thread
    u32 run = s_base[t];
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      u32 c = s_wcnt[w][t];
      s_wcnt[w][t] = run;
      run += c;
    }
    s_base[t] = run;
  }
  __syncthreads();
  u32 r = (d < 256) ? s_wcnt[warp][d] + lrank : 0;
  __syncthreads();
  return r;
}
}  // namespace

template <int R>
__global__ void k_or_and(const u64* __restrict__ rows, u32 m, u64* orv, u64* andv) {
  u64 o[R], a[R];
#pragma unroll
  for (int w = 0; w < R; ++w) {
    o[w] = 0;
    a[w] = ~0ULL;
  }
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int w = 0; w < R; ++w) {
      u64 v = rows[(size_t)i * R + w];
      o[w] |= v;
      a[w] &= v;
    }
  }
#pragma unroll
  for (int w = 0; w < R; ++w) {
    u64 x = o[w], y = a[w];
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      x |= __shfl_xor_sync(kFull, x, off);
      y &= __shfl_xor_sync(kFull, y, off);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicOr(orv + w, x);
      atomicAnd(andv + w, y);
    }
  }
}

template <int R>
__global__ void __launch_bounds__(kRsThreads) k_rs_upsweep(const u64* __restrict__ keys, u32 m, int word, int shift,
                                                           u32 ntiles, u32* counts) {
  __shared__ u32 hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    size_t idx = base + r * kRsThreads + threadIdx.x;
    u32 d = 256;
    if (idx < m) d = (u32)((keys[idx * R + word] >> shift) & 255ULL);
    u32 peers = __match_any_sync(kFull, d);
    if (d < 256 && __popc(peers & lanemask_lt()) == 0) atomicAdd(&hist[d], __popc(peers));
  }
  __syncthreads();
  counts[threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

template <int R>
__global__ void __launch_bounds__(kRsThreads) k_rs_downsweep(const u64* __restrict__ keys, const u32* __restrict__ vals,
                                                             u32 m, int word, int shift, u32 ntiles,
                                                             const u32* __restrict__ offsets, u64* __restrict__ keys_out,
                                                             u32* __restrict__ vals_out) {
  __shared__ u32 s_off[256];
  __shared__ u32 s_base[256];
  __shared__ u32 s_wcnt[8][256];
  s_off[threadIdx.x] = offsets[threadIdx.x * ntiles + blockIdx.x];
  s_base[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    size_t idx = base + r * kRsThreads + threadIdx.x;
    const bool valid = idx < m;
    u64 row[R];
    u32 val = 0;
    u32 d = 256;
    if (valid) {
#pragma unroll
      for (int w = 0; w < R; ++w) row[w] = keys[idx * R + w];
      val = vals[idx];
      u64 kw = 0;
#pragma unroll
      for (int w = 0; w < R; ++w)
        if (w == word) kw = row[w];
      d = (u32)((kw >> shift) & 255ULL);
    }
    u32 rank = block_round_rank(d, s_base, s_wcnt);
    if (valid) {
      size_t dst = (size_t)s_off[d] + rank;
#pragma unroll
      for (int w = 0; w < R; ++w) keys_out[dst * R + w] = row[w];
      vals_out[dst] = val;
    }
  }
}

// Whole sort (or one chunk of it) in one block, rows in shared memory
// (m <= small_sort_max<R>()): a bitonic network over N, the power of two at
// or above m, padded with rows that order after every real row.  Ties are
// broken by the row's input position, so the result is the stable order the
// radix passes and the merge passes assume (equal keys keep their order).
// N log2(N) (log2(N) + 1) / 4 compare-exchanges, one per thread per stage,
// a block barrier between stages.
template <int R>
__global__ void __launch_bounds__(kSmallThreads) k_bitonic_small(u64* keys, u32* vals, u32 m_total, u32 chunk) {
  // block b sorts rows [b * chunk, min(m_total, (b + 1) * chunk))
  const u32 base = blockIdx.x * chunk;
  const u32 m = min(chunk, m_total - base);
  keys += (size_t)base * R;
  vals += base;
  u32 N = 1;
  while (N < m) N <<= 1;
  extern __shared__ u64 s_mem[];
  u64* sk = s_mem;
  u32* sv = reinterpret_cast<u32*>(sk + (size_t)N * R);
  u32* sp = sv + N;
  for (u32 i = threadIdx.x; i < N; i += kSmallThreads) {
    const bool real = i < m;
#pragma unroll
    for (int w = 0; w < R; ++w) sk[(size_t)i * R + w] = real ? keys[(size_t)i * R + w] : ~0ULL;
    sv[i] = real ? vals[i] : 0xffffffffu;
    sp[i] = real ? i : 0xffffffffu;
  }
  __syncthreads();
  for (u32 kk = 2; kk <= N; kk <<= 1) {
    for (u32 j = kk >> 1; j > 0; j >>= 1) {
      for (u32 t = threadIdx.x; t < N / 2; t += kSmallThreads) {
        const u32 lo = ((t & ~(j - 1)) << 1) | (t & (j - 1)), hi = lo + j;
        u64 a[R], b[R];
#pragma unroll
        for (int w = 0; w < R; ++w) {
          a[w] = sk[(size_t)lo * R + w];
          b[w] = sk[(size_t)hi * R + w];
        }
        int cmp = 0;  // sign of a - b, words first, then input position
#pragma unroll
        for (int w = 0; w < R; ++w)
          if (cmp == 0 && a[w] != b[w]) cmp = a[w] > b[w] ? 1 : -1;
        const u32 pa = sp[lo], pb = sp[hi];
        if (cmp == 0) cmp = pa > pb ? 1 : -1;
        const bool up = (lo & kk) == 0;  // this pair's run ascends
        if ((cmp > 0) == up) {
#pragma unroll
          for (int w = 0; w < R; ++w) {
            sk[(size_t)lo * R + w] = b[w];
            sk[(size_t)hi * R + w] = a[w];
          }
          const u32 va = sv[lo];
          sv[lo] = sv[hi];
          sv[hi] = va;
          sp[lo] = pb;
          sp[hi] = pa;
        }
      }
      // Thread t handles pair t (N / 2 <= kSmallThreads).  At a distance
      // j <= 32 every pair of warp w lies in rows [64w, 64w + 64), so
      // between two such stages only the warp's own lanes exchange rows and
      // a warp barrier suffices; any stage at a larger distance, and the
      // read-out after the last stage, needs the block barrier.
      const u32 next_j = j > 1 ? j >> 1 : kk;
      if (j <= 32 && next_j <= 32 && !(kk == N && j == 1)) __syncwarp();
      else __syncthreads();
    }
  }
  for (u32 i = threadIdx.x; i < m; i += kSmallThreads) {
#pragma unroll
    for (int w = 0; w < R; ++w) keys[(size_t)i * R + w] = sk[(size_t)i * R + w];
    vals[i] = sv[i];
  }
}

size_t sort_temp_bytes(int R, u32 m) {
  u32 ntiles = (m + kRsTile - 1) / kRsTile;
  size_t counts = sizeof(u32) * 256 * (size_t)ntiles;
  // counts + offsets + scan partials + or/and words (+ host-visible copy)
  return 2 * counts + scan_temp_bytes(256 * ntiles) + 2 * sizeof(u64) * 16 + 256;
}

// One merge pass: sorted runs of `run` rows are merged pairwise.  Each row
// finds its rank in the partner run by binary search (left-run rows count
// partner keys strictly smaller, right-run rows count keys not greater, so the
// merge is stable) and is written straight to its final place.
template <int R>
__global__ void k_merge_runs(const u64* __restrict__ ki, const u32* __restrict__ vi, u32 m, u32 run,
                             u64* __restrict__ ko, u32* __restrict__ vo) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const u32 r = i / run;
  const u32 pair = (r & ~1u) * run;
  const bool left = (r & 1u) == 0;
  const u32 own = i - r * run;
  const u32 pstart = left ? pair + run : pair;
  const u32 plen = pstart >= m ? 0u : min(run, m - pstart);
  u64 x[R];
#pragma unroll
  for (int w = 0; w < R; ++w) x[w] = ki[(size_t)i * R + w];
  u32 lo = 0, hi = plen;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    const u64* y = ki + (size_t)(pstart + mid) * R;
    int cmp = 0;  // sign of y - x
#pragma unroll
    for (int w = 0; w < R; ++w)
      if (cmp == 0 && y[w] != x[w]) cmp = y[w] < x[w] ? -1 : 1;
    const bool before = left ? cmp < 0 : cmp <= 0;
    if (before) lo = mid + 1;
    else hi = mid;
  }
  const size_t out = (size_t)pair + own + lo;
#pragma unroll
  for (int w = 0; w < R; ++w) ko[out * R + w] = x[w];
  vo[out] = vi[i];
}

template <int R>
static int radix_sort_rows_t(u64* keys, u32* vals, u64* keys_alt, u32* vals_alt, u32 m, void* temp, cudaStream_t s,
                             int* data_passes) {
  if (data_passes) *data_passes = 0;
  if (m <= 1) return 0;
  // Raise the shared-memory opt-in once per device, to the largest size these
  // sorts use: lowering it per call would race with launches of other host
  // threads.
  ensure_smem_limit((const void*)k_bitonic_small<R>, (int)small_sort_smem<R>(small_sort_max<R>()));
  if (m <= small_sort_max<R>()) {
    u32 N = 1;
    while (N < m) N <<= 1;
    k_bitonic_small<R><<<1, kSmallThreads, small_sort_smem<R>(N), s>>>(keys, vals, m, m);
    SW_LAUNCH_CHECK();
    if (data_passes) *data_passes = 1;
    return 1;
  }
  if (m <= kMergeSortMax) {
    // mid sizes: chunks sorted in shared memory by one block each, then
    // pairwise merges of sorted runs (each a single launch), instead of a
    // 3-launch pass per key digit
    const u32 chunk = small_sort_max<R>();
    const u32 nchunks = (m + chunk - 1) / chunk;
    k_bitonic_small<R><<<nchunks, kSmallThreads, small_sort_smem<R>(chunk), s>>>(keys, vals, m, chunk);
    SW_LAUNCH_CHECK();
    u64 *ki = keys, *ko = keys_alt;
    u32 *vi = vals, *vo = vals_alt;
    int merges = 0;
    for (u32 run = chunk; run < m; run *= 2) {
      k_merge_runs<R><<<(m + 255) / 256, 256, 0, s>>>(ki, vi, m, run, ko, vo);
      SW_LAUNCH_CHECK();
      std::swap(ki, ko);
      std::swap(vi, vo);
      ++merges;
    }
    if (ki != keys) {
      SW_CUDA(cudaMemcpyAsync(keys, ki, sizeof(u64) * R * (size_t)m, cudaMemcpyDeviceToDevice, s));
      SW_CUDA(cudaMemcpyAsync(vals, vi, sizeof(u32) * (size_t)m, cudaMemcpyDeviceToDevice, s));
    }
    if (data_passes) *data_passes = 1 + merges;
    return 1 + merges;
  }
  const u32 ntiles = (m + kRsTile - 1) / kRsTile;
  char* t = static_cast<char*>(temp);
  u32* counts = reinterpret_cast<u32*>(t);
  u32* offsets = counts + 256 * (size_t)ntiles;
  u64* orv = reinterpret_cast<u64*>(offsets + 256 * (size_t)ntiles);
  u64* andv = orv + 16;
  void* scan_tmp = andv + 16;
  SW_CUDA(cudaMemsetAsync(orv, 0, sizeof(u64) * R, s));
  SW_CUDA(cudaMemsetAsync(andv, 0xff, sizeof(u64) * R, s));
  u32 blocks = std::min<u32>((m + 255) / 256, (u32)sm_count() * 4);
  k_or_and<R><<<blocks, 256, 0, s>>>(keys, m, orv, andv);
  SW_LAUNCH_CHECK();
  u64 h_or[R], h_and[R];
  SW_CUDA(cudaMemcpyAsync(h_or, orv, sizeof(u64) * R, cudaMemcpyDeviceToHost, s));
  SW_CUDA(cudaMemcpyAsync(h_and, andv, sizeof(u64) * R, cudaMemcpyDeviceToHost, s));
  SW_CUDA(cudaStreamSynchronize(s));
  u64 *ki = keys, *ko = keys_alt;
  u32 *vi = vals, *vo = vals_alt;
  int passes = 0;
  for (int word = R - 1; word >= 0; --word) {
    const u64 vary = h_or[word] ^ h_and[word];
    for (int shift = 0; shift < 64; shift += 8) {
      if (((vary >> shift) & 255ULL) == 0) continue;
      k_rs_upsweep<R><<<ntiles, kRsThreads, 0, s>>>(ki, m, word, shift, ntiles, counts);
      launch_scan(counts, offsets, 256 * ntiles, nullptr, scan_tmp, s);
      k_rs_downsweep<R><<<ntiles, kRsThreads, 0, s>>>(ki, vi, m, word, shift, ntiles, offsets, ko, vo);
      SW_LAUNCH_CHECK();
      std::swap(ki, ko);
      std::swap(vi, vo);
      ++passes;
    }
  }
  if (ki != keys) {
    SW_CUDA(cudaMemcpyAsync(keys, ki, sizeof(u64) * R * (size_t)m, cudaMemcpyDeviceToDevice, s));
    SW_CUDA(cudaMemcpyAsync(vals, vi, sizeof(u32) * (size_t)m, cudaMemcpyDeviceToDevice, s));
  }
  if (data_passes) *data_passes = passes;
  return 1 + 5 * passes;  // or/and reduction + (upsweep, 3 scan kernels, downsweep) per pass
}

int radix_sort_rows(int R, u64* keys, u32* vals, u64* keys_alt, u32* vals_alt, u32 m, void* temp, cudaStream_t s,
                    int* data_passes) {
  switch (R) {
    case 1: return radix_sort_rows_t<1>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 2: return radix_sort_rows_t<2>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 3: return radix_sort_rows_t<3>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 4: return radix_sort_rows_t<4>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 5: return radix_sort_rows_t<5>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 6: return radix_sort_rows_t<6>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 7: return radix_sort_rows_t<7>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 8: return radix_sort_rows_t<8>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    case 9: return radix_sort_rows_t<9>(keys, vals, keys_alt, vals_alt, m, temp, s, data_passes);
    default: throw std::runtime_error("radix_sort_rows: unsupported row width");
  }
}

// ===========================================================================
// Unique flags, compaction and small helpers.
// ===========================================================================
template <int W>
__global__ void k_unique_flags(const u64* __restrict__ rows, u32 m, u32* flags) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  flags[i] = (i == 0) ? 1u : (row_eq<W>(rows + (size_t)i * W, rows + (size_t)(i - 1) * W) ? 0u : 1u);
}

template <int W>
__global__ void k_compact(const u64* __restrict__ rows, const u32* __restrict__ vals, const u32* __restrict__ flags,
                          const u32* __restrict__ pos, u32 m, u64* __restrict__ out_rows, u32* __restrict__ out_vals) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m || !flags[i]) return;
  const u32 d = pos[i];
#pragma unroll
  for (int w = 0; w < W; ++w) out_rows[(size_t)d * W + w] = rows[(size_t)i * W + w];
  if (out_vals) out_vals[d] = vals[i];
}

template <int W>
__global__ void k_complement(u64* rows, u32 m, int n) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
#pragma unroll
  for (int w = 0; w < W; ++w) rows[(size_t)i * W + w] = ~rows[(size_t)i * W + w] & valid_mask(n, w);
}

template <int W>
__global__ void k_popcount(const u64* rows, u32 m, u32* out) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  u32 c = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) c += __popcll(rows[(size_t)i * W + w]);
  out[i] = c;
}

__global__ void k_keep_flags(const u32* a, const u32* b, u32 m, u32* out) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  out[i] = (a[i] == 0 && b[i] == 0) ? 1u : 0u;
}

__global__ void k_fill_u32(u32* p, u32 v, u32 m) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) p[i] = v;
}

#define SW_DISPATCH_W(W, ...)                               \
  switch (W) {                                              \
    case 1: { constexpr int WW = 1; __VA_ARGS__; } break;   \
    case 2: { constexpr int WW = 2; __VA_ARGS__; } break;   \
    case 3: { constexpr int WW = 3; __VA_ARGS__; } break;   \
    case 4: { constexpr int WW = 4; __VA_ARGS__; } break;   \
    case 5: { constexpr int WW = 5; __VA_ARGS__; } break;   \
    case 6: { constexpr int WW = 6; __VA_ARGS__; } break;   \
    case 7: { constexpr int WW = 7; __VA_ARGS__; } break;   \
    case 8: { constexpr int WW = 8; __VA_ARGS__; } break;   \
    default: throw std::runtime_error("unsupported set width"); \
  }

// Row widths of sort keys: set widths 1..8 and beam keys (1 + set width).
#define SW_DISPATCH_R(R, ...)                                 \
  switch (R) {                                                \
    case 1: { constexpr int RR = 1; __VA_ARGS__; } break;     \
    case 2: { constexpr int RR = 2; __VA_ARGS__; } break;     \
    case 3: { constexpr int RR = 3; __VA_ARGS__; } break;     \
    case 4: { constexpr int RR = 4; __VA_ARGS__; } break;     \
    case 5: { constexpr int RR = 5; __VA_ARGS__; } break;     \
    case 6: { constexpr int RR = 6; __VA_ARGS__; } break;     \
    case 7: { constexpr int RR = 7; __VA_ARGS__; } break;     \
    case 8: { constexpr int RR = 8; __VA_ARGS__; } break;     \
    case 9: { constexpr int RR = 9; __VA_ARGS__; } break;     \
    default: throw std::runtime_error("unsupported row width"); \
  }

void launch_unique_flags(int W, const u64* rows, u32 m, u32* flags, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_R(W, (k_unique_flags<RR><<<(m + 255) / 256, 256, 0, s>>>(rows, m, flags)));
  SW_LAUNCH_CHECK();
}

void launch_compact(int W, const u64* rows, const u32* vals, const u32* flags, const u32* pos, u32 m, u64* out_rows,
                    u32* out_vals, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_R(W, (k_compact<RR><<<(m + 255) / 256, 256, 0, s>>>(rows, vals, flags, pos, m, out_rows, out_vals)));
  SW_LAUNCH_CHECK();
}

void launch_complement(int W, u64* rows, u32 m, int n, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_W(W, (k_complement<WW><<<(m + 255) / 256, 256, 0, s>>>(rows, m, n)));
  SW_LAUNCH_CHECK();
}

void launch_popcount(int W, const u64* rows, u32 m, u32* out, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_W(W, (k_popcount<WW><<<(m + 255) / 256, 256, 0, s>>>(rows, m, out)));
  SW_LAUNCH_CHECK();
}

void launch_keep_flags(const u32* a, const u32* b, u32 m, u32* out, cudaStream_t s) {
  if (!m) return;
  k_keep_flags<<<(m + 255) / 256, 256, 0, s>>>(a, b, m, out);
  SW_LAUNCH_CHECK();
}

void launch_fill_u32(u32* p, u32 value, u32 m, cudaStream_t s) {
  if (!m) return;
  k_fill_u32<<<(m + 255) / 256, 256, 0, s>>>(p, value, m);
  SW_LAUNCH_CHECK();
}

// ===========================================================================
// Merge of two sorted disjoint row arrays: each element finds its output
// position by a binary search in the other array (merge path per element).
// ===========================================================================
template <int W>
__global__ void k_merge(const u64* __restrict__ A, u32 na, const u64* __restrict__ B, u32 nb, u64* __restrict__ out) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na + nb) return;
  const bool fromA = i < na;
  const u64* x = fromA ? A + (size_t)i * W : B + (size_t)(i - na) * W;
  const u64* other = fromA ? B : A;
  u32 lo = 0, hi = fromA ? nb : na;
  while (lo < hi) {
    u32 mid = (lo + hi) >> 1;
    if (row_less<W>(other + (size_t)mid * W, x)) lo = mid + 1;
    else hi = mid;
  }
  const size_t pos = (size_t)(fromA ? i : i - na) + lo;
#pragma unroll
  for (int w = 0; w < W; ++w) out[pos * W + w] = x[w];
}

void launch_merge(int W, const u64* A, u32 na, const u64* B, u32 nb, u64* out, cudaStream_t s) {
  if (na + nb == 0) return;
  SW_DISPATCH_W(W, (k_merge<WW><<<(na + nb + 255) / 256, 256, 0, s>>>(A, na, B, nb, out)));
  SW_LAUNCH_CHECK();
}

// ===========================================================================
// Layer keys: (64 chosen states packed into one word, 32-bit mix of the row).
// Sorting by this key groups sets by the pattern of their side's most
// frequent states and makes equal sets adjacent; distinct sets with equal
// keys are possible only through a hash collision, which can at worst leave a
// duplicate in a layer (harmless).  With the identity map the first word is
// the row's word 0 (states 0..63).
// ===========================================================================
template <int W>
__global__ void k_layer_keys(const u64* __restrict__ rows, u32 m, KeyMap map, u64* __restrict__ keys) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  u64 k0, k1;
  layer_key<W>(rows + (size_t)i * W, map, k0, k1);
  keys[2 * (size_t)i] = k0;
  keys[2 * (size_t)i + 1] = k1;
}

void launch_layer_keys(int W, const u64* rows, u32 m, u64* keys, cudaStream_t s, const KeyMap& map) {
  if (!m) return;
  SW_DISPATCH_W(W, (k_layer_keys<WW><<<(m + 255) / 256, 256, 0, s>>>(rows, m, map, keys)));
  SW_LAUNCH_CHECK();
}

// Merge of two arrays sorted by layer key (A first on equal keys).
template <int W>
__global__ void k_merge_key(const u64* __restrict__ A, u32 na, const u64* __restrict__ B, u32 nb, KeyMap map,
                            u64* __restrict__ out) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na + nb) return;
  const bool fromA = i < na;
  const u64* x = fromA ? A + (size_t)i * W : B + (size_t)(i - na) * W;
  u64 x0, x1;
  layer_key<W>(x, map, x0, x1);
  const u64* other = fromA ? B : A;
  u32 lo = 0, hi = fromA ? nb : na;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    u64 y0, y1;
    layer_key<W>(other + (size_t)mid * W, map, y0, y1);
    // A element: count B keys strictly less; B element: count A keys <= its key
    const bool before = fromA ? (y0 < x0 || (y0 == x0 && y1 < x1)) : (y0 < x0 || (y0 == x0 && y1 <= x1));
    if (before) lo = mid + 1;
    else hi = mid;
  }
  const size_t pos = (size_t)(fromA ? i : i - na) + lo;
#pragma unroll
  for (int w = 0; w < W; ++w) out[pos * W + w] = x[w];
}

void launch_merge_key(int W, const u64* A, u32 na, const u64* B, u32 nb, u64* out, cudaStream_t s,
                      const KeyMap& map) {
  if (na + nb == 0) return;
  SW_DISPATCH_W(W, (k_merge_key<WW><<<(na + nb + 255) / 256, 256, 0, s>>>(A, na, B, nb, map, out)));
  SW_LAUNCH_CHECK();
}

// flags[i] = 1 when row i of C equals some row of V (both sorted by the same
// layer key): a binary search for C's key in V, then a scan of V's rows with
// that key.
template <int W>
__global__ void k_member_key(const u64* __restrict__ V, u32 nv, const u64* __restrict__ C, u32 nc, KeyMap map,
                             u32* __restrict__ flags) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const u64* x = C + (size_t)i * W;
  u64 x0, x1;
  layer_key<W>(x, map, x0, x1);
  u32 lo = 0, hi = nv;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    u64 y0, y1;
    layer_key<W>(V + (size_t)mid * W, map, y0, y1);
    if (y0 < x0 || (y0 == x0 && y1 < x1)) lo = mid + 1;
    else hi = mid;
  }
  for (u32 j = lo; j < nv; ++j) {
    const u64* y = V + (size_t)j * W;
    u64 y0, y1;
    layer_key<W>(y, map, y0, y1);
    if (y0 != x0 || y1 != x1) break;
    if (row_eq<W>(x, y)) {
      flags[i] = 1u;
      return;
    }
  }
}

// flags[i] = 0 for rows of C (with flags[i] = 1) equal to some row of V.
template <int W>
__global__ void k_clear_members(const u64* __restrict__ V, u32 nv, const u64* __restrict__ C, u32 nc, KeyMap map,
                                u32* __restrict__ flags) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc || !flags[i]) return;
  const u64* x = C + (size_t)i * W;
  u64 x0, x1;
  layer_key<W>(x, map, x0, x1);
  u32 lo = 0, hi = nv;
  while (lo < hi) {
    const u32 mid = (lo + hi) >> 1;
    u64 y0, y1;
    layer_key<W>(V + (size_t)mid * W, map, y0, y1);
    if (y0 < x0 || (y0 == x0 && y1 < x1)) lo = mid + 1;
    else hi = mid;
  }
  for (u32 j = lo; j < nv; ++j) {
    const u64* y = V + (size_t)j * W;
    u64 y0, y1;
    layer_key<W>(y, map, y0, y1);
    if (y0 != x0 || y1 != x1) break;
    if (row_eq<W>(x, y)) {
      flags[i] = 0u;
      return;
    }
  }
}

void launch_clear_members(int W, const u64* V, u32 nv, const u64* C, u32 nc, u32* flags, cudaStream_t s,
                          const KeyMap& map) {
  if (!nc || !nv) return;
  SW_DISPATCH_W(W, (k_clear_members<WW><<<(nc + 255) / 256, 256, 0, s>>>(V, nv, C, nc, map, flags)));
  SW_LAUNCH_CHECK();
}

// Duplicate test over a key-sorted layer, without materialising the sorted
// rows: position i of the sort holds child vals[i] of C (its layer key
// keys[2i..2i+1]); it is kept when that child differs from child vals[i-1]
// and equals no row of the key-sorted visited list V.
template <int W>
__device__ __forceinline__ bool dedup_keep(const u64* __restrict__ C, const u32* __restrict__ vals,
                                           const u64* __restrict__ keys, u32 i, const u64* __restrict__ V, u32 nv,
                                           const KeyMap& map) {
  const u64* x = C + (size_t)vals[i] * W;
  bool keep = i == 0 || !row_eq<W>(x, C + (size_t)vals[i - 1] * W);
  if (keep && nv) {
    const u64 x0 = keys[2 * (size_t)i], x1 = keys[2 * (size_t)i + 1];
    u32 lo = 0, hi = nv;
    while (lo < hi) {
      const u32 mid = (lo + hi) >> 1;
      u64 y0, y1;
      layer_key<W>(V + (size_t)mid * W, map, y0, y1);
      if (y0 < x0 || (y0 == x0 && y1 < x1)) lo = mid + 1;
      else hi = mid;
    }
    for (u32 j = lo; j < nv && keep; ++j) {
      const u64* y = V + (size_t)j * W;
      u64 y0, y1;
      layer_key<W>(y, map, y0, y1);
      if (y0 != x0 || y1 != x1) break;
      if (row_eq<W>(x, y)) keep = false;
    }
  }
  return keep;
}

// ---- single-pass duplicate removal and compaction ----
// One launch flags the children, counts the kept ones and gathers them: each
// block takes the next tile of kDcTile children (a dynamic tile index from
// `ctr`, so every tile a block waits on belongs to a block that is already
// running), flags its children, scans the flags in shared memory, and finds
// the count kept before its tile by decoupled look-back over the earlier
// tiles' published words: (flag << 62) | (epoch << 32) | count, flag 1 = the
// tile's own count, 2 = the inclusive count of every tile up to it.  `epoch`
// (1..2^30-1, new per launch) tags the words, so the array is never cleared.
// Every wait polls at most kDcWaitLimit times; one that runs out sets *err
// to 2 and the launch's output is incomplete.  The block that drew the last
// tile index resets `ctr` for the next launch on the stream and stores the
// total.
constexpr u32 kDcTile = 512;
constexpr u32 kDcWaitLimit = 1u << 22;

__device__ __forceinline__ u64 ld_acquire_u64(const u64* p) {
  u64 v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(u64* p, u64 v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <int W>
__global__ void __launch_bounds__(kDcTile) k_dedup_compact(const u64* __restrict__ C, const u32* __restrict__ vals,
                                                          const u64* __restrict__ keys, u32 m,
                                                          const u64* __restrict__ V, u32 nv, KeyMap map,
                                                          u64* __restrict__ out_rows, u32* __restrict__ out_vals,
                                                          u32* total, u64* status, u32* ctr, u32 epoch, u32* err) {
  __shared__ u32 s_tile, s_warp[kDcTile / 32], s_excl;
  const u32 ntiles = (m + kDcTile - 1) / kDcTile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ctr, 1u);
  __syncthreads();
  const u32 tile = s_tile;
  if (threadIdx.x == 0 && tile == ntiles - 1) *ctr = 0u;  // every block has drawn its index
  const u32 i = tile * kDcTile + threadIdx.x;
  const bool keep = i < m && dedup_keep<W>(C, vals, keys, i, V, nv, map);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u32 ballot = __ballot_sync(0xffffffffu, keep);
  const u32 before_in_warp = __popc(ballot & ((1u << lane) - 1u));
  if (lane == 0) s_warp[warp] = __popc(ballot);
  __syncthreads();
  if (warp == 0) {
    const u32 c = lane < kDcTile / 32 ? s_warp[lane] : 0u;
    u32 incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const u32 agg = __shfl_sync(0xffffffffu, incl, 31);
    if (lane < kDcTile / 32) s_warp[lane] = incl - c;  // exclusive count of the earlier warps
    if (lane == 0) {
      const u64 tag = (u64)(epoch & 0x3fffffffu) << 32;
      u32 excl = 0;
      if (tile == 0) {
        st_release_u64(status, (2ull << 62) | tag | agg);
      } else {
        st_release_u64(status + tile, (1ull << 62) | tag | agg);
        u32 j = tile - 1, polls = 0;
        for (;;) {
          const u64 w = ld_acquire_u64(status + j);
          const u32 f = (u32)(w >> 62);
          if (f == 0 || (w & (0x3fffffffull << 32)) != tag) {  // not published yet
            if (++polls > kDcWaitLimit) {
              atomicExch(err, 2u);
              break;
            }
            continue;
          }
          excl += (u32)w;
          if (f == 2 || j == 0) break;
          --j;
        }
        st_release_u64(status + tile, (2ull << 62) | tag | (excl + agg));
      }
      s_excl = excl;
      if (tile == ntiles - 1) *total = excl + agg;
    }
  }
  __syncthreads();
  if (keep) {
    const u32 d = s_excl + s_warp[warp] + before_in_warp, src = vals[i];
#pragma unroll
    for (int w = 0; w < W; ++w) out_rows[(size_t)d * W + w] = C[(size_t)src * W + w];
    out_vals[d] = src;
  }
}

size_t dedup_compact_status_words(u32 m) { return (m + kDcTile - 1) / kDcTile; }

void launch_dedup_compact(int W, const u64* C, const u32* vals, const u64* keys, u32 m, const u64* V, u32 nv,
                          const KeyMap& map, u64* out_rows, u32* out_vals, u32* total, u64* status, u32* ctr,
                          u32 epoch, u32* err, cudaStream_t s) {
  if (!m) {
    SW_CUDA(cudaMemsetAsync(total, 0, sizeof(u32), s));
    return;
  }
  if (epoch == 0 || epoch >= (1u << 30)) throw std::invalid_argument("dedup_compact: epoch must be 1..2^30-1");
  const u32 blocks = (m + kDcTile - 1) / kDcTile;
  SW_DISPATCH_W(W, (k_dedup_compact<WW><<<blocks, kDcTile, 0, s>>>(C, vals, keys, m, V, nv, map, out_rows, out_vals,
                                                                  total, status, ctr, epoch, err)));
  SW_LAUNCH_CHECK();
}

void launch_member_key(int W, const u64* V, u32 nv, const u64* C, u32 nc, u32* flags, cudaStream_t s,
                       const KeyMap& map) {
  if (!nc || !nv) return;
  SW_DISPATCH_W(W, (k_member_key<WW><<<(nc + 255) / 256, 256, 0, s>>>(V, nv, C, nc, map, flags)));
  SW_LAUNCH_CHECK();
}

// counts[q] += number of rows containing state q (block histograms in shared memory).
template <int W>
__global__ void k_state_counts(const u64* __restrict__ rows, u32 m, u32* __restrict__ counts) {
  __shared__ u32 h[W * 64];
  for (int i = threadIdx.x; i < W * 64; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int w = 0; w < W; ++w) {
      u64 v = rows[(size_t)i * W + w];
      while (v) {
        const int b = __clzll(v);
        atomicAdd(&h[w * 64 + b], 1u);
        v &= ~(1ULL << (63 - b));
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < W * 64; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[i], h[i]);
}

void launch_state_counts(int W, const u64* rows, u32 m, u32* counts, cudaStream_t s) {
  if (!m) return;
  const u32 blocks = std::min<u32>((m + 255) / 256, (u32)sm_count() * 2);
  SW_DISPATCH_W(W, (k_state_counts<WW><<<blocks, 256, 0, s>>>(rows, m, counts)));
  SW_LAUNCH_CHECK();
}

// ===========================================================================
// Gathers and beam keys.
// ===========================================================================
__global__ void k_iota(u32* p, u32 m) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) p[i] = i;
}

template <int W>
__global__ void k_gather_rows(const u64* __restrict__ src, const u32* __restrict__ idx, u32 m, u64* __restrict__ dst) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const u64* s = src + (size_t)idx[i] * W;
#pragma unroll
  for (int w = 0; w < W; ++w) dst[(size_t)i * W + w] = s[w];
}

// key = [n - |S|, reference-layout words...]: sorting keys ascending orders
// sets by cardinality descending, ties by the reference's raw word order
// (Subset::comp_fast, subset.hpp:78-84; the reference's words are the
// bit-reversed device words).
template <int W>
__global__ void k_beam_keys(const u64* __restrict__ rows, u32 m, int n, int R, u64* __restrict__ keys) {
  u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  u32 c = 0;
  u64 r[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    r[w] = rows[(size_t)i * W + w];
    c += __popcll(r[w]);
  }
  keys[(size_t)i * R] = (u64)(n - (int)c);
#pragma unroll
  for (int w = 0; w < W; ++w)
    if (w + 1 < R) keys[(size_t)i * R + 1 + w] = __brevll(r[w]);
}

void launch_iota(u32* p, u32 m, cudaStream_t s) {
  if (!m) return;
  k_iota<<<(m + 255) / 256, 256, 0, s>>>(p, m);
  SW_LAUNCH_CHECK();
}

void launch_gather_rows(int W, const u64* src, const u32* idx, u32 m, u64* dst, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_W(W, (k_gather_rows<WW><<<(m + 255) / 256, 256, 0, s>>>(src, idx, m, dst)));
  SW_LAUNCH_CHECK();
}

void launch_beam_keys(int W, const u64* rows, u32 m, int n, int R, u64* keys, cudaStream_t s) {
  if (!m) return;
  SW_DISPATCH_W(W, (k_beam_keys<WW><<<(m + 255) / 256, 256, 0, s>>>(rows, m, n, R, keys)));
  SW_LAUNCH_CHECK();
}

__global__ void k_gather_u32(const u32* __restrict__ src, const u32* __restrict__ idx, u32 m, u32* __restrict__ dst) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[i] = src[idx[i]];
}

void launch_gather_u32(const u32* src, const u32* idx, u32 m, u32* dst, cudaStream_t s) {
  if (!m) return;
  k_gather_u32<<<(m + 255) / 256, 256, 0, s>>>(src, idx, m, dst);
  SW_LAUNCH_CHECK();
}

__global__ void k_score_keys(const float* __restrict__ score, const u32* __restrict__ counts, u32 m,
                             u64* __restrict__ keys) {
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  u32 s = 0;
  if (score) {
    s = __float_as_uint(score[i]);
    s = (s & 0x80000000u) ? ~s : (s | 0x80000000u);  // IEEE order -> unsigned order
  }
  u32 u;
  if (score && counts)
    u = (counts[i] << 16) | (s >> 16);  // size first, then the score's leading 16 bits
  else
    u = score ? s : counts[i];
  keys[i] = ((u64)u << 32) | i;
}

void launch_score_keys(const float* score, const u32* counts, u32 m, u64* keys, cudaStream_t s) {
  if (!m) return;
  k_score_keys<<<(m + 255) / 256, 256, 0, s>>>(score, counts, m, keys);
  SW_LAUNCH_CHECK();
}

}  // namespace sw
