// Power-set breadth-first search for automata with at most 32 states.
//
// Reference: Brute::bfs (synchrolib/algorithm/brute/brute.hpp:88-122): BFS
// over bit masks from the full set, one distance byte per mask, stopping at
// the first singleton.  Here the distance array becomes a 2^n-bit visited
// bitmap in HBM and the queue becomes one frontier array per level; the
// images of a mask come from four 256-entry byte tables per letter staged in
// shared memory (image = OR of the four byte images).
#include <mutex>

#include "algos.cuh"

namespace sw {

namespace {
constexpr int kBruteThreads = 256;

__device__ inline u32 image_of(const u32* lut, u32 a, u32 m) {
  const u32* t = lut + a * 1024;
  return t[m & 255u] | t[256 + ((m >> 8) & 255u)] | t[512 + ((m >> 16) & 255u)] | t[768 + (m >> 24)];
}

// lut[a*1024 + b*256 + v] = image under letter a of the states 8b+j, j in v.
__device__ inline void build_lut(u32* lut, const uint16_t* delta, int n, int k) {
  for (int e = threadIdx.x; e < k * 1024; e += blockDim.x) {
    const int a = e >> 10, b = (e >> 8) & 3, v = e & 255;
    u32 r = 0;
    for (int j = 0; j < 8; ++j) {
      const int q = 8 * b + j;
      if (((v >> j) & 1) && q < n) r |= 1u << delta[a * n + q];
    }
    lut[e] = r;
  }
  __syncthreads();
}
}  // namespace

__global__ void __launch_bounds__(kBruteThreads) k_brute_level(const uint16_t* __restrict__ delta, int n, int k,
                                                               const u32* __restrict__ frontier, u32 count,
                                                               u32* visited, u32* next, u32 next_cap,
                                                               u32* next_count, u32* found) {
  extern __shared__ u32 s_lut[];
  build_lut(s_lut, delta, n, k);
  const int lane = threadIdx.x & 31;
  const u64 total = (u64)count * (u64)k;
  const u64 stride = (u64)gridDim.x * blockDim.x;
  // warp-uniform trip count so that the append below can aggregate per warp
  for (u64 base = (u64)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
    const u64 idx = base + lane;
    bool emit = false;
    u32 img = 0;
    if (idx < total) {
      const u32 i = (u32)(idx / (u64)k), a = (u32)(idx % (u64)k);
      img = image_of(s_lut, a, frontier[i]);
      const u32 w = img >> 5, bit = 1u << (img & 31u);
      if (!(visited[w] & bit)) emit = !(atomicOr(&visited[w], bit) & bit);
    }
    const u32 mask = __ballot_sync(0xffffffffu, emit);
    if (!mask) continue;
    u32 pos0 = 0;
    const int leader = __ffs(mask) - 1;
    if (lane == leader) pos0 = atomicAdd(next_count, (u32)__popc(mask));
    pos0 = __shfl_sync(0xffffffffu, pos0, leader);
    if (emit) {
      const u32 pos = pos0 + (u32)__popc(mask & ((1u << lane) - 1u));
      if (pos < next_cap) next[pos] = img;
      if (__popc(img) == 1) {
        found[1] = img;
        found[0] = 1;
      }
    }
  }
}

__global__ void __launch_bounds__(kBruteThreads) k_brute_parent(const uint16_t* __restrict__ delta, int n, int k,
                                                                const u32* __restrict__ level, u32 count, u32 target,
                                                                u64* best) {
  extern __shared__ u32 s_lut[];
  build_lut(s_lut, delta, n, k);
  const u64 total = (u64)count * (u64)k;
  for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (u64)gridDim.x * blockDim.x) {
    const u32 i = (u32)(idx / (u64)k), a = (u32)(idx % (u64)k);
    if (image_of(s_lut, a, level[i]) == target) atomicMin(best, idx);
  }
}

size_t brute_visited_bytes(int n) { return n >= 5 ? ((size_t)1 << n) / 8 : 4; }

namespace {
int brute_grid(u64 work) {
  const int sms = device_sm_count();
  const u64 blocks = (work + kBruteThreads - 1) / kBruteThreads;
  return (int)std::max<u64>(1, std::min<u64>(blocks, (u64)sms * 8));
}
void brute_smem_attr() {
  ensure_smem_limit((const void*)k_brute_level, kMaxLetters * 4096);
  ensure_smem_limit((const void*)k_brute_parent, kMaxLetters * 4096);
}
}  // namespace

void launch_brute_level(const uint16_t* delta, int n, int k, const u32* frontier, u32 count, u32* visited,
                        u32* next, u32 next_cap, u32* next_count, u32* found, cudaStream_t s) {
  if (!count) return;
  brute_smem_attr();
  k_brute_level<<<brute_grid((u64)count * k), kBruteThreads, (size_t)k * 4096, s>>>(
      delta, n, k, frontier, count, visited, next, next_cap, next_count, found);
  SW_LAUNCH_CHECK();
}

void launch_brute_parent(const uint16_t* delta, int n, int k, const u32* level, u32 count, u32 target, u64* best,
                         cudaStream_t s) {
  if (!count) return;
  brute_smem_attr();
  k_brute_parent<<<brute_grid((u64)count * k), kBruteThreads, (size_t)k * 4096, s>>>(delta, n, k, level, count,
                                                                                      target, best);
  SW_LAUNCH_CHECK();
}

}  // namespace sw
