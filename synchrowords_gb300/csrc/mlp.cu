// Kernels of the learned distance model (mlp.cuh).
//
// The generic product C = A · B runs on the fifth-generation tensor cores:
// one CTA of eight warps owns a 128-row tile of C with all of its N (64 or
// 128) columns.  Per 64-deep slice of K the warps stage A (128 x 64) and B
// (N x 64) in shared memory as bf16 in the canonical K-major layout without
// swizzle (8 x 8 "core matrices" of 128 contiguous bytes, K-adjacent cores
// 128 bytes apart, 8-row groups 1024 bytes apart); one thread then issues four
// tcgen05.mma (kind::f16: bf16 x bf16 -> fp32, M = 128, K = 16 each) into a
// TMEM accumulator of N columns and commits them to an mbarrier.  At the end
// each warp reads 32 accumulator rows (its TMEM lanes) and half of the
// columns back with tcgen05.ld.  Contiguous operands move as 16-byte loads.  Operands are
// read through strided views, so the same kernel serves the forward products
// and the transposed products of the backward pass.  Every wait is bounded: a
// wait that runs out sets an error word (tc_error()), the CTA frees its TMEM
// and stops.
#include "mlp.cuh"

namespace sw {
namespace mlp {

namespace {
constexpr int kTM = 128;     // rows of C per CTA (the MMA's M)
constexpr int kTK = 64;      // K per staged slice (four MMAs of K = 16)
constexpr int kMaxN = 128;   // columns of C per CTA (the MMA's N; the TMEM columns)
constexpr int kTcThreads = 256;  // eight warps stage; warps w and w + 4 share TMEM lanes 32 (w % 4) ..
constexpr u32 kTcWaitLimit = 1u << 24;
// shared memory: A slice, B slice (bf16, core-matrix layout), then the mbarrier and the TMEM address.
// A CTA asks for 60 KB so that at most three share an SM: three accumulators
// of 128 columns fit the SM's 512 TMEM columns, so an allocation never waits.
constexpr int kSmemA = kTM * kTK * 2;
constexpr int kSmemB = kMaxN * kTK * 2;
constexpr int kTcSmem = 60 * 1024;
static_assert(kSmemA + kSmemB + 64 <= kTcSmem, "slices and barrier fit the CTA's shared memory");

__device__ u32 g_tc_error = 0;

__device__ __forceinline__ u32 sm_addr(const void* p) { return (u32)__cvta_generic_to_shared(p); }

// byte offset of element (row r, k) of a slice in the canonical no-swizzle
// K-major layout: core matrix (r / 8, k / 8), 16-byte rows inside it
__device__ __forceinline__ u32 core_offset(int r, int k) {
  return (u32)((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// tcgen05 shared-memory descriptor: start address, leading-dimension byte
// offset (K-adjacent core matrices), stride byte offset (8-row groups),
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(u32 addr) {
  const uint64_t start = (addr & 0x3FFFFu) >> 4;
  const uint64_t lbo = 128u >> 4, sbo = 1024u >> 4;
  return start | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 and M >> 4
__device__ __forceinline__ u32 instr_desc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((u32)(n >> 3) << 17) | ((u32)(kTM >> 4) << 24);
}

__device__ __forceinline__ bool bar_wait(u32 bar, u32 parity) {
  for (u32 it = 0; it < kTcWaitLimit; ++it) {
    u32 ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
}  // namespace

__global__ void __launch_bounds__(kTcThreads) k_gemm_tc(View A, View B, float* __restrict__ C, int ldc, int M, int N,
                                                        int K, int k_slice, int atomic) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + kSmemA;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kSmemA + kSmemB);
  u32* tmem_slot = reinterpret_cast<u32*>(smem + kSmemA + kSmemB + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = blockIdx.x * kTM;
  const int kb = blockIdx.z * k_slice, ke = min(K, kb + k_slice);
  const u32 ncols = N <= 64 ? 64u : 128u;  // TMEM columns: a power of two >= 32
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sm_addr(tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const u32 tmem = *tmem_slot;
  const __nv_bfloat16 zero = __float2bfloat16(0.0f);
  // rows of A (columns of B) contiguous along the staged dimension and 16-byte aligned: vector loads
  const bool vecA = A.sk == 1 && A.si % 8 == 0 && ((uintptr_t)A.p & 15) == 0;
  const bool vecB = B.sk == 1 && B.si % 8 == 0 && ((uintptr_t)B.p & 15) == 0;
  u32 parity = 0;
  bool ok = true, first = true;
  for (int k0 = kb; k0 < ke && ok; k0 += kTK) {
    // stage the slices (rows / columns past M, N and k past the slice are zero)
    if (vecA) {
      // eight consecutive k of a row: one 16-byte load, one 16-byte core-matrix row
      for (int e = tid; e < kTM * (kTK / 8); e += kTcThreads) {
        const int r = e / (kTK / 8), kk = (e % (kTK / 8)) * 8, i = i0 + r, k = k0 + kk;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (i < M && k + 8 <= ke) {
          v = *reinterpret_cast<const uint4*>(A.p + (long long)i * A.si + k);
        } else if (i < M && k < ke) {
          __nv_bfloat16 t[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) t[j] = k + j < ke ? A.p[(long long)i * A.si + k + j] : zero;
          v = *reinterpret_cast<const uint4*>(t);
        }
        *reinterpret_cast<uint4*>(sA + core_offset(r, kk)) = v;
      }
    } else {
      for (int e = tid; e < kTM * kTK; e += kTcThreads) {
        const int r = e / kTK, kk = e % kTK, i = i0 + r, k = k0 + kk;
        const __nv_bfloat16 v = (i < M && k < ke) ? A.p[(long long)i * A.si + (long long)k * A.sk] : zero;
        *reinterpret_cast<__nv_bfloat16*>(sA + core_offset(r, kk)) = v;
      }
    }
    if (vecB) {
      // eight consecutive columns of one k: one 16-byte load, eight core-matrix rows
      for (int e = tid; e < (int)(ncols / 8) * kTK; e += kTcThreads) {
        const int kk = e / (int)(ncols / 8), c = (e % (int)(ncols / 8)) * 8, k = k0 + kk;
        __nv_bfloat16 t[8];
        if (k < ke && c + 8 <= N) {
          *reinterpret_cast<uint4*>(t) = *reinterpret_cast<const uint4*>(B.p + (long long)k * B.si + c);
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) t[j] = (k < ke && c + j < N) ? B.p[(long long)k * B.si + c + j] : zero;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) *reinterpret_cast<__nv_bfloat16*>(sB + core_offset(c + j, kk)) = t[j];
      }
    } else {
      for (int e = tid; e < (int)ncols * kTK; e += kTcThreads) {
        const int c = e / kTK, kk = e % kTK, k = k0 + kk;
        const __nv_bfloat16 v = (c < N && k < ke) ? B.p[(long long)k * B.si + (long long)c * B.sk] : zero;
        *reinterpret_cast<__nv_bfloat16*>(sB + core_offset(c, kk)) = v;
      }
    }
    // the tensor cores read shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const u32 idesc = instr_desc((int)ncols);
#pragma unroll
      for (int s = 0; s < kTK / 16; ++s) {
        const uint64_t da = smem_desc(sm_addr(sA) + s * 256);  // K = 16 s: two cores of 128 bytes further
        const uint64_t db = smem_desc(sm_addr(sB) + s * 256);
        const u32 acc = (first && s == 0) ? 0u : 1u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sm_addr(bar))
                   : "memory");
    }
    first = false;
    // the MMAs must have read the slices before they are overwritten
    ok = bar_wait(sm_addr(bar), parity);
    parity ^= 1u;
    ok = __syncthreads_and(ok);
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) {
    if (tid == 0) atomicExch(&g_tc_error, 1u);
  } else if (!first) {
    // warp w reads accumulator rows 32 (w % 4) .. + 31 (its TMEM lanes), half
    // of the columns each for w < 4 and w >= 4, 16 columns at a time
    const int q = warp & 3, half = warp >> 2;
    const int i = i0 + q * 32 + lane;
    const int cbeg = half * (int)(ncols / 2), cend = cbeg + (int)(ncols / 2);
    for (int c0 = cbeg; c0 < cend; c0 += 16) {
      u32 v[16];
      const u32 taddr = tmem + ((u32)(q * 32) << 16) + (u32)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (i < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = c0 + j;
          if (col < N) {
            float* dst = C + (long long)i * ldc + col;
            if (atomic)
              atomicAdd(dst, __uint_as_float(v[j]));
            else
              *dst = __uint_as_float(v[j]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

void gemm(View A, View B, float* C, int ldc, int M, int N, int K, bool atomic, int split, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  if (N > kMaxN) throw std::invalid_argument("mlp gemm: N above 128");
  split = std::max(1, split);
  int slice = (K + split - 1) / split;
  slice = (slice + kTK - 1) / kTK * kTK;
  split = (K + slice - 1) / slice;
  if (split > 1) atomic = true;
  ensure_smem_limit((const void*)k_gemm_tc, kTcSmem);
  dim3 grid((M + kTM - 1) / kTM, 1, split);
  k_gemm_tc<<<grid, kTcThreads, kTcSmem, s>>>(A, B, C, ldc, M, N, K, slice, atomic ? 1 : 0);
  SW_LAUNCH_CHECK();
}

bool tc_error() {
  u32 v = 0;
  SW_CUDA(cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(u32)));
  return v != 0;
}

__global__ void k_bits_to_dense(const u64* __restrict__ rows, int W, int n, u32 count, __nv_bfloat16* out, int ld) {
  const long long total = (long long)count * ld;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ld;
    const int q = (int)(e % ld);
    float v = 0.0f;
    if (q < n) v = (rows[b * W + (q >> 6)] & state_bit(q)) ? 1.0f : 0.0f;
    out[e] = __float2bfloat16(v);
  }
}

void bits_to_dense(const u64* rows, int W, int n, u32 count, __nv_bfloat16* out, int ld, cudaStream_t s) {
  if (!count) return;
  const long long total = (long long)count * ld;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  k_bits_to_dense<<<blocks, 256, 0, s>>>(rows, W, n, count, out, ld);
  SW_LAUNCH_CHECK();
}

__global__ void k_bias_act(const float* __restrict__ in, const float* __restrict__ bias, int rows, int cols, int relu,
                           float* pre, __nv_bfloat16* act) {
  const long long total = (long long)rows * cols;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    float v = in[e] + (bias ? bias[e % cols] : 0.0f);
    if (pre) pre[e] = v;
    if (relu) v = fmaxf(v, 0.0f);
    act[e] = __float2bfloat16(v);
  }
}

void bias_act(const float* in, const float* bias, int rows, int cols, bool relu, float* pre, __nv_bfloat16* act,
              cudaStream_t s) {
  const long long total = (long long)rows * cols;
  if (!total) return;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  k_bias_act<<<blocks, 256, 0, s>>>(in, bias, rows, cols, relu ? 1 : 0, pre, act);
  SW_LAUNCH_CHECK();
}

// one warp per row
__global__ void k_head(const __nv_bfloat16* __restrict__ H, const float* __restrict__ params, int rows,
                       float* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= rows) return;
  float acc = 0.0f;
  for (int j = lane; j < kHidden; j += 32)
    acc += __bfloat162float(H[(long long)row * kHidden + j]) * params[kOffW3 + j];
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc + params[kOffB3];
}

void head(const __nv_bfloat16* H, const float* params, int rows, float* y, cudaStream_t s) {
  if (!rows) return;
  k_head<<<(rows * 32 + 255) / 256, 256, 0, s>>>(H, params, rows, y);
  SW_LAUNCH_CHECK();
}

__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ tgt, int rows, float* dy, float* loss) {
  __shared__ float s_sum[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (i < rows) {
    const float d = y[i] - tgt[i];
    dy[i] = 2.0f * d / (float)rows;
    l = d * d / (float)rows;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += s_sum[w];
    atomicAdd(loss, b);
  }
}

void mse(const float* y, const float* t, int rows, float* dy, float* loss, cudaStream_t s) {
  if (!rows) return;
  k_mse<<<(rows + 255) / 256, 256, 0, s>>>(y, t, rows, dy, loss);
  SW_LAUNCH_CHECK();
}

// Pairwise ranking term over the rows of one group (one BFS layer): for every
// pair with t_a < t_b, w / rows * softplus(y_a - y_b), so that a set nearer to
// a singleton scores lower than its sibling; its gradient is added to dy.
__global__ void k_rank_add(const float* __restrict__ y, const float* __restrict__ tgt, const uint32_t* __restrict__ grp,
                           int rows, float w, float* dy, float* loss) {
  __shared__ float s_sum[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (i < rows) {
    const float yi = y[i], ti = tgt[i];
    const uint32_t gi = grp[i];
    float g = 0.0f;
    for (int j = 0; j < rows; ++j) {
      if (grp[j] != gi) continue;
      const float tj = tgt[j];
      if (ti < tj) {  // i should score below j
        const float z = yi - y[j];
        g += 1.0f / (1.0f + __expf(-z));
        l += z > 20.0f ? z : log1pf(__expf(z));
      } else if (tj < ti) {  // j should score below i
        g -= 1.0f / (1.0f + __expf(-(y[j] - yi)));
      }
    }
    dy[i] += w * g / (float)rows;
    l *= w / (float)rows;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.0f;
    for (int x = 0; x < (int)(blockDim.x >> 5); ++x) b += s_sum[x];
    atomicAdd(loss, b);
  }
}

void rank_add(const float* y, const float* t, const uint32_t* grp, int rows, float w, float* dy, float* loss,
              cudaStream_t s) {
  if (!rows || w == 0.0f) return;
  k_rank_add<<<(rows + 255) / 256, 256, 0, s>>>(y, t, grp, rows, w, dy, loss);
  SW_LAUNCH_CHECK();
}

// block of 128 threads = one hidden column each; rows in chunks
__global__ void k_head_back(const float* __restrict__ dy, const __nv_bfloat16* __restrict__ H,
                            const float* __restrict__ pre, const float* __restrict__ params, int rows, int rows_per_block,
                            float* grad, float* dH, __nv_bfloat16* dHb) {
  const int j = threadIdx.x;  // hidden unit
  const int r0 = blockIdx.x * rows_per_block, r1 = min(rows, r0 + rows_per_block);
  const float w = params[kOffW3 + j];
  float gw = 0.0f, gb = 0.0f;
  for (int r = r0; r < r1; ++r) {
    const long long e = (long long)r * kHidden + j;
    const float d = dy[r];
    gw += d * __bfloat162float(H[e]);
    gb += d;
    const float v = pre[e] > 0.0f ? d * w : 0.0f;
    dH[e] = v;
    dHb[e] = __float2bfloat16(v);
  }
  atomicAdd(&grad[kOffW3 + j], gw);
  if (j == 0) atomicAdd(&grad[kOffB3], gb);
}

void head_back(const float* dy, const __nv_bfloat16* H, const float* pre, const float* params, int rows, float* grad,
               float* dH, __nv_bfloat16* dHb, cudaStream_t s) {
  if (!rows) return;
  const int per = 64;
  k_head_back<<<(rows + per - 1) / per, kHidden, 0, s>>>(dy, H, pre, params, rows, per, grad, dH, dHb);
  SW_LAUNCH_CHECK();
}

__global__ void k_relu_back(float* d, const float* __restrict__ pre, int count, __nv_bfloat16* db) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const float v = pre[e] > 0.0f ? d[e] : 0.0f;
    d[e] = v;
    if (db) db[e] = __float2bfloat16(v);
  }
}

void relu_back(float* d, const float* pre, int count, __nv_bfloat16* db, cudaStream_t s) {
  if (!count) return;
  const int blocks = std::min((count + 255) / 256, 152 * 16);
  k_relu_back<<<blocks, 256, 0, s>>>(d, pre, count, db);
  SW_LAUNCH_CHECK();
}

// grid.x = column blocks of 32 columns, grid.y = row chunks; block 32 x 8
__global__ void k_col_sum(const float* __restrict__ M, int rows, int cols, int rows_per_block, float* out) {
  __shared__ float s_part[8][32];
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int r0 = blockIdx.y * rows_per_block, r1 = min(rows, r0 + rows_per_block);
  float acc = 0.0f;
  if (j < cols)
    for (int r = r0 + threadIdx.y; r < r1; r += 8) acc += M[(long long)r * cols + j];
  s_part[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && j < cols) {
    float sum = 0.0f;
    for (int y = 0; y < 8; ++y) sum += s_part[y][threadIdx.x];
    atomicAdd(&out[j], sum);
  }
}

void col_sum(const float* M, int rows, int cols, float* out, cudaStream_t s) {
  if (!rows || !cols) return;
  const int per = 256;
  dim3 grid((cols + 31) / 32, (rows + per - 1) / per);
  k_col_sum<<<grid, dim3(32, 8), 0, s>>>(M, rows, cols, per, out);
  SW_LAUNCH_CHECK();
}

__global__ void k_to_bf16(const float* __restrict__ in, __nv_bfloat16* out, int count) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x)
    out[e] = __float2bfloat16(in[e]);
}

void to_bf16(const float* in, __nv_bfloat16* out, int count, cudaStream_t s) {
  if (!count) return;
  const int blocks = std::min((count + 255) / 256, 152 * 16);
  k_to_bf16<<<blocks, 256, 0, s>>>(in, out, count);
  SW_LAUNCH_CHECK();
}

// Adam (Kingma & Ba 2015) with beta1 = 0.9, beta2 = 0.999, eps = 1e-8.
__global__ void k_adam(float* p, const float* __restrict__ g, float* m, float* v, int count, float lr, float c1,
                       float c2) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const float gr = g[e];
    const float mm = 0.9f * m[e] + 0.1f * gr;
    const float vv = 0.999f * v[e] + 0.001f * gr * gr;
    m[e] = mm;
    v[e] = vv;
    p[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
  }
}

void adam(float* p, const float* g, float* m, float* v, int count, float lr, int t, cudaStream_t s) {
  const float c1 = 1.0f - std::pow(0.9f, (float)t), c2 = 1.0f - std::pow(0.999f, (float)t);
  const int blocks = std::min((count + 255) / 256, 152 * 4);
  k_adam<<<blocks, 256, 0, s>>>(p, g, m, v, count, lr, c1, c2);
  SW_LAUNCH_CHECK();
}

}  // namespace mlp
}  // namespace sw
