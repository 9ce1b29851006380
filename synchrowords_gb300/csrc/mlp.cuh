// Learned distance model: a set S of states is scored by
//   E   = relu(feat · Phi + c)                  per-state embeddings, n x 64 (bf16)
//   x   = sum over q in S of E[q]                (= bits(S) · E, a tensor-core GEMM)
//   h1  = relu(x · W1 + b1),  h2 = relu(h1 · W2 + b2)   (64 -> 128 -> 128)
//   y   = h2 · w3 + b3                            predicted shortest merge length
// feat is a fixed per-state feature vector of the automaton (automaton.cpp),
// so one trained model applies to automata of any size.  Dense products run
// on the tensor cores (tcgen05.mma, bf16 inputs, fp32 accumulation in TMEM);
// master weights, gradients and Adam moments are fp32.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace sw {
namespace mlp {

constexpr int kFeat = 16;    // per-state features
constexpr int kEmb = 64;     // embedding width
constexpr int kHidden = 128; // hidden width

// Offsets (floats) into the flat parameter vector.
constexpr int kOffPhi = 0;                            // [kFeat][kEmb]
constexpr int kOffC = kOffPhi + kFeat * kEmb;         // [kEmb]
constexpr int kOffW1 = kOffC + kEmb;                  // [kEmb][kHidden]
constexpr int kOffB1 = kOffW1 + kEmb * kHidden;       // [kHidden]
constexpr int kOffW2 = kOffB1 + kHidden;              // [kHidden][kHidden]
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;    // [kHidden]
constexpr int kOffW3 = kOffB2 + kHidden;              // [kHidden]
constexpr int kOffB3 = kOffW3 + kHidden;              // [1]
constexpr int kParams = kOffB3 + 1;

// A bf16 matrix view: element (i, k) at p[i * si + k * sk].
struct View {
  const __nv_bfloat16* p;
  long long si, sk;
};

// C[i*ldc + j] (= or +=) sum_k A(i,k) B(k,j) for i < M, j < N <= 128; `atomic`
// accumulates with atomicAdd (required when split > 1: K is cut in `split`
// slices, one per grid z).
void gemm(View A, View B, float* C, int ldc, int M, int N, int K, bool atomic, int split, cudaStream_t s);
// True once a product's bounded wait for its tensor-core work ran out (its
// results are then incomplete); synchronises with the device.
bool tc_error();

// Set rows (device layout, W words) -> dense 0/1 bf16 rows of width ld (>= n).
void bits_to_dense(const u64* rows, int W, int n, u32 count, __nv_bfloat16* out, int ld, cudaStream_t s);

// act = bf16(relu(in + bias)); keeps `in + bias` in `pre` when pre != nullptr.
// With relu == false only the bias is added.
void bias_act(const float* in, const float* bias, int rows, int cols, bool relu, float* pre, __nv_bfloat16* act,
              cudaStream_t s);

// y[b] = sum_j H[b][j] * w3[j] + b3 (w3, b3 from the fp32 parameters).
void head(const __nv_bfloat16* H, const float* params, int rows, float* y, cudaStream_t s);

// Loss 1/B sum (y - t)^2 (loss[0] += ...) and dy = 2 (y - t) / B.
void mse(const float* y, const float* t, int rows, float* dy, float* loss, cudaStream_t s);
// Adds w/B sum over pairs of one group with t_a < t_b of softplus(y_a - y_b)
// to the loss and its gradient to dy (a within-layer ranking term).
void rank_add(const float* y, const float* t, const uint32_t* grp, int rows, float w, float* dy, float* loss,
              cudaStream_t s);

// From dy: grad of w3 and b3 (grad vector, accumulated), and the masked
// hidden gradient dH = dy w3^T * [pre > 0] (fp32 and bf16).
void head_back(const float* dy, const __nv_bfloat16* H, const float* pre, const float* params, int rows, float* grad,
               float* dH, __nv_bfloat16* dHb, cudaStream_t s);

// d = d * [pre > 0] in place, bf16 copy in db (nullptr: none).
void relu_back(float* d, const float* pre, int count, __nv_bfloat16* db, cudaStream_t s);

// out[j] += sum_i M[i*cols + j].
void col_sum(const float* M, int rows, int cols, float* out, cudaStream_t s);

// fp32 -> bf16.
void to_bf16(const float* in, __nv_bfloat16* out, int count, cudaStream_t s);

// Adam step (t = 1-based step count) on the parameter vector.
void adam(float* p, const float* g, float* m, float* v, int count, float lr, int t, cudaStream_t s);

}  // namespace mlp
}  // namespace sw
