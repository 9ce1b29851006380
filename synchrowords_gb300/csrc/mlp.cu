// Kernels of the learned distance model (mlp.cuh).
//
// The generic product C = A · B is tiled 64 x 64 x 32 per block of four warps;
// each warp owns 16 rows of the tile and issues mma.sync m16n8k16 (bf16 in,
// fp32 accumulate) over the tile's eight 8-column slices.  Operands are
// staged in shared memory through strided loads so that the same kernel
// serves the forward products and the transposed products of the backward
// pass.  Fragment layouts are the ones PTX defines for m16n8k16 with
// .row.col: with g = lane / 4 and t = lane % 4, A registers hold (g, 2t..2t+1),
// (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..); B registers hold (k = 2t..2t+1,
// n = g) and (k = 2t+8.., n = g); C holds (g, 2t..2t+1) and (g+8, 2t..2t+1).
#include "mlp.cuh"

namespace sw {
namespace mlp {

namespace {
constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;

__device__ inline uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
}  // namespace

__global__ void __launch_bounds__(128) k_gemm(View A, View B, float* __restrict__ C, int ldc, int M, int N, int K,
                                              int k_slice, int atomic) {
  __shared__ __nv_bfloat16 sA[kBM][kBK + kPad];  // [row][k]
  __shared__ __nv_bfloat16 sB[kBN][kBK + kPad];  // [col][k]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int i0 = blockIdx.y * kBM, j0 = blockIdx.x * kBN;
  const int kb = blockIdx.z * k_slice, ke = min(K, kb + k_slice);
  const __nv_bfloat16 zero = __float2bfloat16(0.0f);
  float acc[8][4];
#pragma unroll
  for (int s = 0; s < 8; ++s)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[s][r] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += kBK) {
    for (int e = tid; e < kBM * kBK; e += 128) {
      const int r = e / kBK, kk = e % kBK;
      const int i = i0 + r, k = k0 + kk;
      sA[r][kk] = (i < M && k < ke) ? A.p[(long long)i * A.si + (long long)k * A.sk] : zero;
    }
    for (int e = tid; e < kBN * kBK; e += 128) {
      const int c = e / kBK, kk = e % kBK;
      const int j = j0 + c, k = k0 + kk;
      sB[c][kk] = (j < N && k < ke) ? B.p[(long long)k * B.si + (long long)j * B.sk] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kBK; ks += 16) {
      const int r = warp * 16 + g;
      uint32_t a[4];
      a[0] = pack2(sA[r][ks + 2 * t], sA[r][ks + 2 * t + 1]);
      a[1] = pack2(sA[r + 8][ks + 2 * t], sA[r + 8][ks + 2 * t + 1]);
      a[2] = pack2(sA[r][ks + 2 * t + 8], sA[r][ks + 2 * t + 9]);
      a[3] = pack2(sA[r + 8][ks + 2 * t + 8], sA[r + 8][ks + 2 * t + 9]);
#pragma unroll
      for (int s = 0; s < 8; ++s) {
        const int c = s * 8 + g;
        uint32_t b0 = pack2(sB[c][ks + 2 * t], sB[c][ks + 2 * t + 1]);
        uint32_t b1 = pack2(sB[c][ks + 2 * t + 8], sB[c][ks + 2 * t + 9]);
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(acc[s][0]), "+f"(acc[s][1]), "+f"(acc[s][2]), "+f"(acc[s][3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < 8; ++s)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = i0 + warp * 16 + g + (r >= 2 ? 8 : 0);
      const int j = j0 + s * 8 + 2 * t + (r & 1);
      if (i < M && j < N) {
        float* dst = C + (long long)i * ldc + j;
        if (atomic)
          atomicAdd(dst, acc[s][r]);
        else
          *dst = acc[s][r];
      }
    }
}

void gemm(View A, View B, float* C, int ldc, int M, int N, int K, bool atomic, int split, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return;
  split = std::max(1, split);
  int slice = (K + split - 1) / split;
  slice = (slice + kBK - 1) / kBK * kBK;
  split = (K + slice - 1) / slice;
  if (split > 1) atomic = true;
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM, split);
  k_gemm<<<grid, 128, 0, s>>>(A, B, C, ldc, M, N, K, slice, atomic ? 1 : 0);
  SW_LAUNCH_CHECK();
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
