// Allocation-free subset check on caller-owned device buffers.
//
// Some callers cannot let a library allocate device memory: a host
// application that hands its whole device budget to its own pool allocator, or
// a service that forbids allocations once it is serving requests (a
// cudaMalloc there can stall every stream on the device or fail outright when
// the pool already holds the memory).  For them this entry point runs the
// tiled subset check (subset_check.cu) without calling cudaMalloc, cudaFree or
// any allocating routine: inputs and outputs are the caller's device buffers,
// and the only scratch — the per-tile and per-super-tile AND masks of the set
// list — lives in the file-scope device array below, sized for at most
// SW_NOALLOC_MAX_SETS sets of up to 512 states.  Every GPU that loads the
// library holds that array until the process exits.
//
// The array is shared by every call: a call overwrites what the previous call
// left there, and calls whose work overlaps on the GPU (different streams or
// host threads without ordering between them) race on it.  Callers must
// order such calls themselves.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/synchrowords.h"
#include "kernels.cuh"

namespace sw {
namespace {

// masks for SW_NOALLOC_MAX_SETS rows of 8 words: one per 64-row tile plus one
// per 1024-row super-tile (the default ScanShape, which this entry point
// always uses, whatever shapes a context was tuned to), plus 4 words: three
// for the unused meet-mode witness, one for the kernel's copy-timeout word
constexpr size_t kMaxTiles = (SW_NOALLOC_MAX_SETS + 63) / 64;
constexpr size_t kMaxSupers = (SW_NOALLOC_MAX_SETS + 1023) / 1024;
constexpr size_t kScratchWords = (kMaxTiles + kMaxSupers) * 8 + 4;  // + witness, error word

__device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
int scratch_address(void** out, std::string& err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice failed: ") + cudaGetErrorString(e);
    return SW_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device index out of range for the scratch table";
    return SW_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
      return SW_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SW_OK;
}

}  // namespace

void set_last_error(const std::string& msg);  // abi.cpp: the message sw_last_error() returns

}  // namespace sw

extern "C" int sw_subsets_check_device_noalloc(uint32_t n, const uint64_t* d_sets, uint64_t set_count,
                                               const uint64_t* d_checks, uint64_t check_count, int32_t proper,
                                               uint32_t* d_results, void* stream) {
  using namespace sw;
  std::string g_err;
  struct Report {  // hand the message (or "") to sw_last_error() on every return
    std::string& m;
    ~Report() { set_last_error(m); }
  } report{g_err};
  if (n == 0 || n > (uint32_t)kMaxStates) {
    g_err = "n must be in [1, 512]";
    return SW_ERR_INVALID_ARGUMENT;
  }
  if (set_count > SW_NOALLOC_MAX_SETS) {
    g_err = "set_count " + std::to_string(set_count) + " exceeds SW_NOALLOC_MAX_SETS (" +
            std::to_string((unsigned long long)SW_NOALLOC_MAX_SETS) + "), the size of the static scratch";
    return SW_ERR_CAPACITY;
  }
  if (check_count > 0xffffffffULL) {
    g_err = "check_count exceeds 2^32 - 1";
    return SW_ERR_INVALID_ARGUMENT;
  }
  if ((set_count && !d_sets) || (check_count && (!d_checks || !d_results))) {
    g_err = "NULL device buffer";
    return SW_ERR_INVALID_ARGUMENT;
  }
  // the set tiles are copied with 16-byte loads, check rows with 8-byte
  // loads, results written as 4-byte words: a misaligned pointer would fault
  // on the GPU, so it is refused here
  if (((uintptr_t)d_sets & 15u) || ((uintptr_t)d_checks & 7u) || ((uintptr_t)d_results & 3u)) {
    g_err = "misaligned device buffer: d_sets needs 16-byte, d_checks 8-byte and d_results 4-byte alignment";
    return SW_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (check_count == 0) return SW_OK;
  // look the scratch up before queuing anything, so that a failed lookup
  // returns with the caller's buffers untouched
  void* scratch = nullptr;
  if (set_count) {
    int rc = scratch_address(&scratch, g_err);
    if (rc != SW_OK) return rc;
  }
  // results start at zero: the kernel only ever sets flags
  cudaError_t e = cudaMemsetAsync(d_results, 0, sizeof(uint32_t) * check_count, s);
  if (e != cudaSuccess) {
    g_err = std::string("cudaMemsetAsync failed: ") + cudaGetErrorString(e);
    return SW_ERR_CUDA;
  }
  if (set_count == 0) return SW_OK;
  const int W = words_for((int)n);
  auto* masks = static_cast<u64*>(scratch);
  u32* witness = reinterpret_cast<u32*>(masks + kScratchWords - 4);
  try {
    const ScanShape sh{};
    static_assert(ScanShape{}.tile_rows == 64 && ScanShape{}.tiles_per_super == 16, "scratch sized for 64 x 16");
    launch_tile_and(W, reinterpret_cast<const u64*>(d_sets), (u32)set_count, masks, sh, s);
    launch_subset_check(W, proper ? kQueryProperSubset : kQuerySubset, reinterpret_cast<const u64*>(d_sets),
                        (u32)set_count, masks, reinterpret_cast<const u64*>(d_checks), (u32)check_count, (int)n,
                        d_results, witness, false, sh, s, nullptr, witness + 3);
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return SW_ERR_CUDA;
  }
  return SW_OK;
}
