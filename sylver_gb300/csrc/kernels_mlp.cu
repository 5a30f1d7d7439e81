// Small MLP (D0 -> H -> H -> 1, ReLU) that predicts the log factorization time
// of a schedule; trained and evaluated on the GPU by the kernels below
// (forward, backward, Adam).  It only chooses kernel paths: it never touches
// the arithmetic of a factorization.
//
// Parameters live in one FP32 device vector:
//   W1 (H x D0), b1 (H), W2 (H x H), b2 (H), W3 (1 x H), b3 (1)
// Inputs are row-major B x D0.  Loss: mean squared error over the batch.
#include <cmath>
#include <random>
#include <vector>

#include "../../include/sylver_gb300.h"
#include "numeric.hpp"

namespace sylver_gb300 {

namespace {

// out[b][j] = act(sum_i W[j][i] in[b][i] + bias[j])
__global__ void k_dense(const float* __restrict__ W, const float* __restrict__ bias,
                        const float* __restrict__ in, float* __restrict__ out, int B, int nin,
                        int nout, bool relu) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= B * nout) return;
  int b = e / nout, j = e % nout;
  float s = bias[j];
  for (int i = 0; i < nin; ++i) s = fmaf(W[(int64_t)j * nin + i], in[(int64_t)b * nin + i], s);
  out[e] = relu ? fmaxf(s, 0.f) : s;
}

// d[b] = 2 (yhat[b] - y[b]) / B ; loss partials
__global__ void k_out_delta(const float* __restrict__ yhat, const float* __restrict__ y, int B,
                            float* __restrict__ d, float* __restrict__ loss) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (b < B) {
    float r = yhat[b] - y[b];
    d[b] = 2.f * r / (float)B;
    l = r * r / (float)B;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// gW[j][i] = sum_b delta[b][j] in[b][i] ; gb[j] = sum_b delta[b][j]
__global__ void k_wgrad(const float* __restrict__ delta, const float* __restrict__ in,
                        float* __restrict__ gW, float* __restrict__ gb, int B, int nin,
                        int nout) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nout * (nin + 1)) return;
  int j = e / (nin + 1), i = e % (nin + 1);
  float s = 0.f;
  if (i < nin)
    for (int b = 0; b < B; ++b) s = fmaf(delta[(int64_t)b * nout + j], in[(int64_t)b * nin + i], s);
  else
    for (int b = 0; b < B; ++b) s += delta[(int64_t)b * nout + j];
  if (i < nin) gW[(int64_t)j * nin + i] = s;
  else gb[j] = s;
}

// din[b][i] = (sum_j delta[b][j] W[j][i]) * (act[b][i] > 0)
__global__ void k_back(const float* __restrict__ delta, const float* __restrict__ W,
                       const float* __restrict__ act, float* __restrict__ din, int B, int nin,
                       int nout) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= B * nin) return;
  int b = e / nin, i = e % nin;
  float s = 0.f;
  for (int j = 0; j < nout; ++j) s = fmaf(delta[(int64_t)b * nout + j], W[(int64_t)j * nin + i], s);
  din[e] = act[e] > 0.f ? s : 0.f;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

inline int nb(int64_t n, int bs = 256) { return (int)((n + bs - 1) / bs); }

}  // namespace

struct Mlp {
  int d0, h;
  int64_t np;
  DevMem p, g, m, v, x, y, h1, h2, yo, d3, dh2, dh1, loss;
  int cap = 0;
  int64_t steps = 0;

  Mlp(int nin, int nh) : d0(nin), h(nh) {
    np = (int64_t)h * d0 + h + (int64_t)h * h + h + h + 1;
    p.ensure(np * 4);
    g.ensure(np * 4);
    m.ensure(np * 4);
    v.ensure(np * 4);
    loss.ensure(4);
    SG_CUDA(cudaMemset(m.p, 0, np * 4));
    SG_CUDA(cudaMemset(v.p, 0, np * 4));
  }
  float* W1() { return p.as<float>(); }
  float* b1() { return W1() + (int64_t)h * d0; }
  float* W2() { return b1() + h; }
  float* b2() { return W2() + (int64_t)h * h; }
  float* W3() { return b2() + h; }
  float* b3() { return W3() + h; }
  float* G(int64_t off) { return g.as<float>() + off; }

  void reserve(int B) {
    if (B <= cap) return;
    x.ensure((size_t)B * d0 * 4);
    y.ensure((size_t)B * 4);
    h1.ensure((size_t)B * h * 4);
    h2.ensure((size_t)B * h * 4);
    yo.ensure((size_t)B * 4);
    d3.ensure((size_t)B * 4);
    dh2.ensure((size_t)B * h * 4);
    dh1.ensure((size_t)B * h * 4);
    cap = B;
  }
  void forward(int B, cudaStream_t s) {
    k_dense<<<nb((int64_t)B * h), 256, 0, s>>>(W1(), b1(), x.as<float>(), h1.as<float>(), B, d0, h,
                                               true);
    k_dense<<<nb((int64_t)B * h), 256, 0, s>>>(W2(), b2(), h1.as<float>(), h2.as<float>(), B, h, h,
                                               true);
    k_dense<<<nb(B), 256, 0, s>>>(W3(), b3(), h2.as<float>(), yo.as<float>(), B, h, 1, false);
  }
  // loss into `loss` (device), gradient into g
  void backward(int B, cudaStream_t s) {
    SG_CUDA(cudaMemsetAsync(loss.p, 0, 4, s));
    k_out_delta<<<nb(B), 256, 0, s>>>(yo.as<float>(), y.as<float>(), B, d3.as<float>(),
                                      loss.as<float>());
    const int64_t oW1 = 0, ob1 = (int64_t)h * d0, oW2 = ob1 + h, ob2 = oW2 + (int64_t)h * h,
                  oW3 = ob2 + h, ob3 = oW3 + h;
    k_wgrad<<<nb(h + 1), 256, 0, s>>>(d3.as<float>(), h2.as<float>(), G(oW3), G(ob3), B, h, 1);
    k_back<<<nb((int64_t)B * h), 256, 0, s>>>(d3.as<float>(), W3(), h2.as<float>(),
                                              dh2.as<float>(), B, h, 1);
    k_wgrad<<<nb((int64_t)h * (h + 1)), 256, 0, s>>>(dh2.as<float>(), h1.as<float>(), G(oW2),
                                                     G(ob2), B, h, h);
    k_back<<<nb((int64_t)B * h), 256, 0, s>>>(dh2.as<float>(), W2(), h1.as<float>(),
                                              dh1.as<float>(), B, h, h);
    k_wgrad<<<nb((int64_t)h * (d0 + 1)), 256, 0, s>>>(dh1.as<float>(), x.as<float>(), G(oW1),
                                                      G(ob1), B, d0, h);
  }
  void adam(float lr, cudaStream_t s) {
    steps++;
    const float b1c = 0.9f, b2c = 0.999f;
    float c1 = 1.f - std::pow(b1c, (float)steps), c2 = 1.f - std::pow(b2c, (float)steps);
    k_adam<<<nb(np), 256, 0, s>>>(p.as<float>(), g.as<float>(), m.as<float>(), v.as<float>(),
                                  (int)np, lr, b1c, b2c, 1e-8f, c1, c2);
  }
  void upload(const float* xh, const float* yh, int B, cudaStream_t s) {
    reserve(B);
    SG_CUDA(cudaMemcpyAsync(x.p, xh, (size_t)B * d0 * 4, cudaMemcpyHostToDevice, s));
    if (yh) SG_CUDA(cudaMemcpyAsync(y.p, yh, (size_t)B * 4, cudaMemcpyHostToDevice, s));
  }
};

}  // namespace sylver_gb300

using namespace sylver_gb300;

extern "C" {

void* sylver_gb300_mlp_create(int nin, int nhidden, unsigned seed) {
  if (nin < 1 || nhidden < 1) return nullptr;
  Runtime& rt = Runtime::get();
  if (!rt.init()) return nullptr;
  try {
    Mlp* m = new Mlp(nin, nhidden);
    // He-style initialisation on the host (deterministic for a seed)
    std::vector<float> p(m->np, 0.f);
    std::mt19937 gen(seed);
    auto fill = [&](int64_t off, int rows, int cols) {
      std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)cols));
      for (int64_t k = 0; k < (int64_t)rows * cols; ++k) p[off + k] = nd(gen);
    };
    int64_t o = 0;
    fill(o, nhidden, nin);
    o += (int64_t)nhidden * nin + nhidden;
    fill(o, nhidden, nhidden);
    o += (int64_t)nhidden * nhidden + nhidden;
    fill(o, 1, nhidden);
    SG_CUDA(cudaMemcpy(m->p.p, p.data(), m->np * 4, cudaMemcpyHostToDevice));
    return m;
  } catch (const std::exception&) {
    return nullptr;
  }
}

void sylver_gb300_mlp_free(void* mlp) { delete static_cast<Mlp*>(mlp); }

long sylver_gb300_mlp_num_params(void const* mlp) {
  return mlp ? (long)static_cast<const Mlp*>(mlp)->np : -1;
}

int sylver_gb300_mlp_set_params(void* mlp, float const* params) {
  Mlp* m = static_cast<Mlp*>(mlp);
  if (!m || !params) return SYLVER_ERROR_UNKNOWN;
  try {
    SG_CUDA(cudaMemcpy(m->p.p, params, m->np * 4, cudaMemcpyHostToDevice));
    SG_CUDA(cudaMemset(m->m.p, 0, m->np * 4));
    SG_CUDA(cudaMemset(m->v.p, 0, m->np * 4));
    m->steps = 0;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
  return 0;
}

int sylver_gb300_mlp_get_params(void const* mlp, float* params) {
  const Mlp* m = static_cast<const Mlp*>(mlp);
  if (!m || !params) return SYLVER_ERROR_UNKNOWN;
  if (cudaMemcpy(params, m->p.p, m->np * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SYLVER_ERROR_CUDA_UNKNOWN;
  return 0;
}

int sylver_gb300_mlp_forward(void* mlp, float const* x, int batch, float* y) {
  Mlp* m = static_cast<Mlp*>(mlp);
  if (!m || !x || !y || batch < 1) return SYLVER_ERROR_UNKNOWN;
  cudaStream_t s = Runtime::get().stream;
  try {
    m->upload(x, nullptr, batch, s);
    m->forward(batch, s);
    SG_CUDA(cudaMemcpyAsync(y, m->yo.p, (size_t)batch * 4, cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
  return 0;
}

int sylver_gb300_mlp_loss_grad(void* mlp, float const* x, float const* y, int batch, float* loss,
                               float* grad) {
  Mlp* m = static_cast<Mlp*>(mlp);
  if (!m || !x || !y || batch < 1) return SYLVER_ERROR_UNKNOWN;
  cudaStream_t s = Runtime::get().stream;
  try {
    m->upload(x, y, batch, s);
    m->forward(batch, s);
    m->backward(batch, s);
    if (loss) SG_CUDA(cudaMemcpyAsync(loss, m->loss.p, 4, cudaMemcpyDeviceToHost, s));
    if (grad) SG_CUDA(cudaMemcpyAsync(grad, m->g.p, m->np * 4, cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
  return 0;
}

int sylver_gb300_mlp_train(void* mlp, float const* x, float const* y, int batch, int epochs,
                           float lr, float* final_loss) {
  Mlp* m = static_cast<Mlp*>(mlp);
  if (!m || !x || !y || batch < 1 || epochs < 0) return SYLVER_ERROR_UNKNOWN;
  cudaStream_t s = Runtime::get().stream;
  try {
    m->upload(x, y, batch, s);
    for (int e = 0; e < epochs; ++e) {
      m->forward(batch, s);
      m->backward(batch, s);
      m->adam(lr, s);
    }
    m->forward(batch, s);
    m->backward(batch, s);
    if (final_loss) SG_CUDA(cudaMemcpyAsync(final_loss, m->loss.p, 4, cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
  return 0;
}

}  // extern "C"
