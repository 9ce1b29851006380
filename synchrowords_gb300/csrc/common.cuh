// Shared definitions for the synchrowords GB300 library (host + device).
//
// Set layout on the device ("MSB-first rows"): a set of n states is a row of
// W = ceil(n/64) 64-bit words, 1..8 (n = 160 / 320 / 384 use 24 / 40 /
// 48-byte rows); state q is
// bit (63 - q % 64) of word q / 64.  With this layout the numeric order of
// rows (word 0 most significant) is the reference's lexicographic order of
// sets (state 0 most significant, synchrolib/data_structures/subset.hpp:71-77),
// so one radix sort of raw words yields the order the prefix trie needs.
// Unused tail bits are zero.  Rows are 8*W bytes; row arrays start 16-byte
// aligned, so 64-row tiles can be moved as uint4.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

namespace sw {

using u64 = unsigned long long;
using u32 = uint32_t;

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

#define SW_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t _e = (call);                                                               \
    if (_e != cudaSuccess)                                                                 \
      throw ::sw::CudaError(std::string(#call) + " failed: " + cudaGetErrorString(_e) +  \
                            " at " + __FILE__ + ":" + std::to_string(__LINE__));           \
  } while (0)

#define SW_LAUNCH_CHECK() SW_CUDA(cudaGetLastError())

constexpr int kMaxStates = 512;
constexpr int kMaxLetters = 16;

inline int words_for(int n) { return n <= 64 ? 1 : (n + 63) / 64; }

// Device-side bit helpers for the MSB-first layout.
__host__ __device__ inline u64 state_bit(int q) { return 1ULL << (63 - (q & 63)); }
__host__ __device__ inline int state_word(int q) { return q >> 6; }

// Mask of valid bits of word `w` for an n-state set.
__host__ __device__ inline u64 valid_mask(int n, int w) {
  int lo = w * 64;
  if (n >= lo + 64) return ~0ULL;
  if (n <= lo) return 0ULL;
  int bits = n - lo;
  return ~0ULL << (64 - bits);
}

// Per-device launch facts, looked up once per device and safe to call from
// several host threads (kernels.cu).  Both act on the current device.
int device_sm_count();
// Raises `fn`'s dynamic shared-memory limit to at least `bytes` on the
// current device.  Limits only grow, so a concurrent launch of `fn` on
// another host thread never sees its limit lowered below what it asked for.
void ensure_smem_limit(const void* fn, int bytes);

// Stream on which the calling thread's DevBuf growth is ordered (set by an
// AllocScope around a search on one stream).  With one, growing a buffer
// frees the old block and takes the new one stream-ordered
// (cudaFreeAsync / cudaMallocAsync from the device's default pool, which the
// scope keeps cached), so the grow waits for nothing but that stream;
// without one it uses cudaFree, which waits for every stream of the device.
// Buffers grown inside a scope must only be used on that stream, or after it
// has been synchronised.
cudaStream_t& alloc_stream();
struct AllocScope {
  cudaStream_t prev;
  explicit AllocScope(cudaStream_t s);
  ~AllocScope() { alloc_stream() = prev; }
  AllocScope(const AllocScope&) = delete;
  AllocScope& operator=(const AllocScope&) = delete;
};

// Grow-only device buffer (the context keeps them across steps and solves,
// so a solve performs no per-step cudaMalloc).
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  void reserve(size_t bytes) {
    if (bytes <= cap) return;
    const size_t want = bytes + bytes / 4 + 256;
    if (cudaStream_t s = alloc_stream()) {
      if (p) SW_CUDA(cudaFreeAsync(p, s));
      p = nullptr;
      cap = 0;
      SW_CUDA(cudaMallocAsync(&p, want, s));
    } else {
      if (p) SW_CUDA(cudaFree(p));
      p = nullptr;
      cap = 0;
      SW_CUDA(cudaMalloc(&p, want));
    }
    cap = want;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// Pinned host staging for small readbacks.
struct HostPinned {
  void* p = nullptr;
  size_t cap = 0;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
  void reserve(size_t bytes) {
    if (bytes <= cap) return;
    if (p) SW_CUDA(cudaFreeHost(p));
    SW_CUDA(cudaMallocHost(&p, bytes));
    cap = bytes;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

}  // namespace sw
