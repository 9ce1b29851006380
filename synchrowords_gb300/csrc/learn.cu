// MlpRunner (learn.hpp): the forward and backward products of the learned
// distance model as sequences of tensor-core GEMMs (mlp.cu).
#include "learn.hpp"

namespace sw {

using mlp::View;
using bf16 = __nv_bfloat16;

namespace {
View view(const DevBuf& b, long long si, long long sk) { return View{b.as<bf16>(), si, sk}; }
View view(const bf16* p, long long si, long long sk) { return View{p, si, sk}; }
int splits_for(u32 k_rows) { return (int)std::max<u32>(1, std::min<u32>(64, k_rows / 512)); }
}  // namespace

void MlpRunner::set_params(const float* host) {
  params_.reserve(sizeof(float) * mlp::kParams);
  grad_.reserve(sizeof(float) * mlp::kParams);
  m_.reserve(sizeof(float) * mlp::kParams);
  v_.reserve(sizeof(float) * mlp::kParams);
  loss_.reserve(sizeof(float) * 4);
  SW_CUDA(cudaMemcpyAsync(params_.p, host, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaMemsetAsync(m_.p, 0, sizeof(float) * mlp::kParams, stream_));
  SW_CUDA(cudaMemsetAsync(v_.p, 0, sizeof(float) * mlp::kParams, stream_));
  step_ = 0;
  refresh_bf16();
  SW_CUDA(cudaStreamSynchronize(stream_));
  loaded_ = true;
}

void MlpRunner::get_params(float* host) {
  SW_CUDA(cudaMemcpyAsync(host, params_.p, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
}

void MlpRunner::refresh_bf16() {
  phi_b_.reserve(sizeof(bf16) * mlp::kFeat * mlp::kEmb);
  w1_b_.reserve(sizeof(bf16) * mlp::kEmb * mlp::kHidden);
  w2_b_.reserve(sizeof(bf16) * mlp::kHidden * mlp::kHidden);
  const float* p = params_.as<float>();
  mlp::to_bf16(p + mlp::kOffPhi, phi_b_.as<bf16>(), mlp::kFeat * mlp::kEmb, stream_);
  mlp::to_bf16(p + mlp::kOffW1, w1_b_.as<bf16>(), mlp::kEmb * mlp::kHidden, stream_);
  mlp::to_bf16(p + mlp::kOffW2, w2_b_.as<bf16>(), mlp::kHidden * mlp::kHidden, stream_);
}

void MlpRunner::prepare(const Automaton& A) {
  if (!loaded_) throw std::runtime_error("no distance model loaded");
  n_ = (int)A.n;
  std::vector<uint32_t> key{A.n, A.k};
  key.insert(key.end(), A.t.begin(), A.t.end());
  if (key != feat_key_) {  // features depend on the automaton only: computed once per automaton
    const std::vector<float> f = state_features(A);
    feat_.reserve(sizeof(float) * f.size());
    feat_b_.reserve(sizeof(bf16) * f.size());
    SW_CUDA(cudaMemcpyAsync(feat_.p, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice, stream_));
    mlp::to_bf16(feat_.as<float>(), feat_b_.as<bf16>(), (int)f.size(), stream_);
    SW_CUDA(cudaStreamSynchronize(stream_));  // f is released at the end of this block
    feat_key_ = std::move(key);
  }
  epre_.reserve(sizeof(float) * n_ * mlp::kEmb);
  e_b_.reserve(sizeof(bf16) * n_ * mlp::kEmb);
  // Epre = feat · Phi (+ c), E = relu(Epre)
  mlp::gemm(view(feat_b_, mlp::kFeat, 1), view(phi_b_, mlp::kEmb, 1), epre_.as<float>(), mlp::kEmb, n_, mlp::kEmb,
            mlp::kFeat, false, 1, stream_);
  mlp::bias_act(epre_.as<float>(), params_.as<float>() + mlp::kOffC, n_, mlp::kEmb, true, epre_.as<float>(),
                e_b_.as<bf16>(), stream_);
}

void MlpRunner::reserve_batch(u32 count) {
  const size_t c = std::max<u32>(count, 1);
  bits_.reserve(sizeof(bf16) * c * n_);
  x_.reserve(sizeof(float) * c * mlp::kEmb);
  xb_.reserve(sizeof(bf16) * c * mlp::kEmb);
  h1_.reserve(sizeof(float) * c * mlp::kHidden);
  h1b_.reserve(sizeof(bf16) * c * mlp::kHidden);
  h2_.reserve(sizeof(float) * c * mlp::kHidden);
  h2b_.reserve(sizeof(bf16) * c * mlp::kHidden);
}

void MlpRunner::forward(const u64* rows, int W, u32 count, float* y) {
  if (!count) return;
  count_ = count;
  reserve_batch(count);
  const float* p = params_.as<float>();
  mlp::bits_to_dense(rows, W, n_, count, bits_.as<bf16>(), n_, stream_);
  // x = bits · E
  mlp::gemm(view(bits_, n_, 1), view(e_b_, mlp::kEmb, 1), x_.as<float>(), mlp::kEmb, (int)count, mlp::kEmb, n_,
            false, 1, stream_);
  mlp::bias_act(x_.as<float>(), nullptr, (int)count, mlp::kEmb, false, nullptr, xb_.as<bf16>(), stream_);
  // h1 = relu(x · W1 + b1)
  mlp::gemm(view(xb_, mlp::kEmb, 1), view(w1_b_, mlp::kHidden, 1), h1_.as<float>(), mlp::kHidden, (int)count,
            mlp::kHidden, mlp::kEmb, false, 1, stream_);
  mlp::bias_act(h1_.as<float>(), p + mlp::kOffB1, (int)count, mlp::kHidden, true, h1_.as<float>(), h1b_.as<bf16>(),
                stream_);
  // h2 = relu(h1 · W2 + b2)
  mlp::gemm(view(h1b_, mlp::kHidden, 1), view(w2_b_, mlp::kHidden, 1), h2_.as<float>(), mlp::kHidden, (int)count,
            mlp::kHidden, mlp::kHidden, false, 1, stream_);
  mlp::bias_act(h2_.as<float>(), p + mlp::kOffB2, (int)count, mlp::kHidden, true, h2_.as<float>(), h2b_.as<bf16>(),
                stream_);
  mlp::head(h2b_.as<bf16>(), p, (int)count, y, stream_);
}

void MlpRunner::zero_grad() {
  SW_CUDA(cudaMemsetAsync(grad_.p, 0, sizeof(float) * mlp::kParams, stream_));
  SW_CUDA(cudaMemsetAsync(loss_.p, 0, sizeof(float), stream_));
}

void MlpRunner::backward(const float* t, u32 count, const uint32_t* grp, float rank_w) {
  if (!count || count != count_) throw std::runtime_error("backward: batch differs from the forward batch");
  const size_t c = count;
  dy_.reserve(sizeof(float) * c * 2);
  dh2_.reserve(sizeof(float) * c * mlp::kHidden);
  dh2b_.reserve(sizeof(bf16) * c * mlp::kHidden);
  dh1_.reserve(sizeof(float) * c * mlp::kHidden);
  dh1b_.reserve(sizeof(bf16) * c * mlp::kHidden);
  dx_.reserve(sizeof(float) * c * mlp::kEmb);
  dxb_.reserve(sizeof(bf16) * c * mlp::kEmb);
  de_.reserve(sizeof(float) * n_ * mlp::kEmb);
  deb_.reserve(sizeof(bf16) * n_ * mlp::kEmb);
  float* g = grad_.as<float>();
  const int B = (int)count, split = splits_for(count);
  // the output is recomputed from h2 (one small launch) so that backward()
  // needs only the targets
  float* yy = dy_.as<float>() + c;
  mlp::head(h2b_.as<bf16>(), params_.as<float>(), B, yy, stream_);
  mlp::mse(yy, t, B, dy_.as<float>(), loss_.as<float>(), stream_);
  if (grp && rank_w > 0.0f) mlp::rank_add(yy, t, grp, B, rank_w, dy_.as<float>(), loss_.as<float>(), stream_);
  // head: dw3, db3, dH2 = dy w3^T * [h2 > 0]
  mlp::head_back(dy_.as<float>(), h2b_.as<bf16>(), h2_.as<float>(), params_.as<float>(), B, g, dh2_.as<float>(),
                 dh2b_.as<bf16>(), stream_);
  mlp::col_sum(dh2_.as<float>(), B, mlp::kHidden, g + mlp::kOffB2, stream_);
  // dW2 = h1^T · dH2
  mlp::gemm(view(h1b_, 1, mlp::kHidden), view(dh2b_, mlp::kHidden, 1), g + mlp::kOffW2, mlp::kHidden, mlp::kHidden,
            mlp::kHidden, B, true, split, stream_);
  // dH1 = dH2 · W2^T * [h1 > 0]
  mlp::gemm(view(dh2b_, mlp::kHidden, 1), view(w2_b_, 1, mlp::kHidden), dh1_.as<float>(), mlp::kHidden, B,
            mlp::kHidden, mlp::kHidden, false, 1, stream_);
  mlp::relu_back(dh1_.as<float>(), h1_.as<float>(), B * mlp::kHidden, dh1b_.as<bf16>(), stream_);
  mlp::col_sum(dh1_.as<float>(), B, mlp::kHidden, g + mlp::kOffB1, stream_);
  // dW1 = x^T · dH1
  mlp::gemm(view(xb_, 1, mlp::kEmb), view(dh1b_, mlp::kHidden, 1), g + mlp::kOffW1, mlp::kHidden, mlp::kEmb,
            mlp::kHidden, B, true, split, stream_);
  // dX = dH1 · W1^T
  mlp::gemm(view(dh1b_, mlp::kHidden, 1), view(w1_b_, 1, mlp::kHidden), dx_.as<float>(), mlp::kEmb, B, mlp::kEmb,
            mlp::kHidden, false, 1, stream_);
  mlp::to_bf16(dx_.as<float>(), dxb_.as<bf16>(), B * mlp::kEmb, stream_);
  // dE = bits^T · dX, then through the embedding relu
  SW_CUDA(cudaMemsetAsync(de_.p, 0, sizeof(float) * n_ * mlp::kEmb, stream_));
  mlp::gemm(view(bits_, 1, n_), view(dxb_, mlp::kEmb, 1), de_.as<float>(), mlp::kEmb, n_, mlp::kEmb, B, true, split,
            stream_);
  mlp::relu_back(de_.as<float>(), epre_.as<float>(), n_ * mlp::kEmb, deb_.as<bf16>(), stream_);
  mlp::col_sum(de_.as<float>(), n_, mlp::kEmb, g + mlp::kOffC, stream_);
  // dPhi = feat^T · dEpre
  mlp::gemm(view(feat_b_, 1, mlp::kFeat), view(deb_, mlp::kEmb, 1), g + mlp::kOffPhi, mlp::kEmb, mlp::kFeat,
            mlp::kEmb, n_, true, 1, stream_);
}

void MlpRunner::adam_step(float lr) {
  ++step_;
  mlp::adam(params_.as<float>(), grad_.as<float>(), m_.as<float>(), v_.as<float>(), mlp::kParams, lr, step_, stream_);
  refresh_bf16();
}

}  // namespace sw
