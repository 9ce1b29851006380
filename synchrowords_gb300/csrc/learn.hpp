// Host side of the learned distance model (mlp.cuh): parameters, the
// per-automaton embedding table, forward scoring, the backward pass and Adam.
#pragma once
#include <cuda_bf16.h>

#include <vector>

#include "automaton.hpp"
#include "common.cuh"
#include "mlp.cuh"

namespace sw {

class MlpRunner {
 public:
  explicit MlpRunner(cudaStream_t s) : stream_(s) {}

  // Parameters: host vector of mlp::kParams floats (layout in mlp.cuh).
  void set_params(const float* host);
  void get_params(float* host);
  bool has_params() const { return loaded_; }

  // Embedding table of automaton A (its state features through Phi, c, relu).
  void prepare(const Automaton& A);

  // y[i] = predicted distance of rows[i] (device layout, W words per row),
  // for the automaton last prepared.  Activations stay for backward().
  void forward(const u64* rows, int W, u32 count, float* y);

  // After forward() on the same rows: gradient of the mean squared error
  // against targets t (device) added into grad(); loss added into loss().
  // With `grp` (a group id per row, e.g. its BFS layer) and rank_w > 0 the
  // loss adds rank_w times a pairwise ranking term within each group.
  void backward(const float* t, u32 count, const uint32_t* grp = nullptr, float rank_w = 0.0f);

  void zero_grad();
  void adam_step(float lr);  // then refreshes the bf16 weight copies
  float* grad() { return grad_.as<float>(); }
  float* loss() { return loss_.as<float>(); }

 private:
  cudaStream_t stream_;
  bool loaded_ = false;
  int n_ = 0, step_ = 0;
  std::vector<uint32_t> feat_key_;  // automaton whose features are in feat_ (n, k, table)
  u32 count_ = 0;
  DevBuf params_, grad_, m_, v_, loss_;
  DevBuf phi_b_, w1_b_, w2_b_, feat_, feat_b_, epre_, e_b_;
  DevBuf bits_, x_, xb_, h1_, h1b_, h2_, h2b_, dy_, dh2_, dh2b_, dh1_, dh1b_, dx_, dxb_, de_, deb_;
  void refresh_bf16();
  void reserve_batch(u32 count);
};

}  // namespace sw
