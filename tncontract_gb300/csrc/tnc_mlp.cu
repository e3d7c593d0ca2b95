// Kernels of the learned rank predictor: a small fully connected network
// (dense layers with ReLU / sigmoid) trained on the GPU with hand-written
// forward, backward and Adam kernels, plus the Gaussian fill used for the
// randomized-SVD sketches it sizes.  No counterpart in the reference: the
// predictor sizes a randomized SVD that replaces left_canonise's full SVD
// (tncontract/onedim/onedim_core.py:317) when the predicted rank is small.
//
// Shapes are tiny (batch x 128): one thread per output element, FP32.
#include "tnc_common.cuh"

namespace tnc {

// out[b][o] = act(sum_i W[o][i] in[b][i] + bias[o]); act 0 = identity, 1 = relu, 2 = sigmoid
__global__ void dense_fwd_kernel(const float* __restrict__ W, const float* __restrict__ bias,
                                 const float* __restrict__ in, float* __restrict__ out, int batch, int nin, int nout,
                                 int act) {
  const int64_t total = (int64_t)batch * nout;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / nout), o = (int)(e - (int64_t)b * nout);
    float acc = bias[o];
    const float* w = W + (int64_t)o * nin;
    const float* x = in + (int64_t)b * nin;
    for (int i = 0; i < nin; ++i) acc = fmaf(w[i], x[i], acc);
    if (act == 1) acc = acc > 0.f ? acc : 0.f;
    else if (act == 2) acc = 1.f / (1.f + expf(-acc));
    out[e] = acc;
  }
}

// dW[o][i] = sum_b g[b][o] in[b][i];  dbias[o] = sum_b g[b][o]
__global__ void dense_bwd_w_kernel(const float* __restrict__ g, const float* __restrict__ in, float* __restrict__ dW,
                                   float* __restrict__ db, int batch, int nin, int nout) {
  const int64_t total = (int64_t)nout * (nin + 1);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int o = (int)(e / (nin + 1)), i = (int)(e - (int64_t)o * (nin + 1));
    float acc = 0.f;
    if (i < nin) {
      for (int b = 0; b < batch; ++b) acc = fmaf(g[(int64_t)b * nout + o], in[(int64_t)b * nin + i], acc);
      dW[(int64_t)o * nin + i] = acc;
    } else {
      for (int b = 0; b < batch; ++b) acc += g[(int64_t)b * nout + o];
      db[o] = acc;
    }
  }
}

// gin[b][i] = (sum_o W[o][i] g[b][o]) * (mask_act ? (act_in[b][i] > 0) : 1)
__global__ void dense_bwd_in_kernel(const float* __restrict__ W, const float* __restrict__ g,
                                    const float* __restrict__ act_in, float* __restrict__ gin, int batch, int nin,
                                    int nout, int relu_mask) {
  const int64_t total = (int64_t)batch * nin;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / nin), i = (int)(e - (int64_t)b * nin);
    float acc = 0.f;
    for (int o = 0; o < nout; ++o) acc = fmaf(W[(int64_t)o * nin + i], g[(int64_t)b * nout + o], acc);
    if (relu_mask && !(act_in[e] > 0.f)) acc = 0.f;
    gin[e] = acc;
  }
}

// g[b] = 2 (y[b] - t[b]) y[b] (1 - y[b]) / batch: mean-squared error through the sigmoid
__global__ void mse_sigmoid_grad_kernel(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ g,
                                        int batch) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x) {
    const float d = y[b] - t[b];
    g[b] = 2.f * d * y[b] * (1.f - y[b]) / (float)batch;
  }
}

// Adam (Kingma & Ba 2015) with bias correction for step t >= 1
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Counter-based uniform pair -> standard normal (Box-Muller).  The hash is
// a 64-bit mix (splitmix64 finaliser) of (seed, index).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
template <typename R>
__device__ __forceinline__ void gauss2(uint64_t seed, uint64_t idx, R& a, R& b) {
  const uint64_t h = mix64(seed * 0xD1B54A32D192ED03ull + idx);
  const double u1 = ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = ((double)(mix64(h) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double r = sqrt(-2.0 * log(u1));
  a = (R)(r * cos(6.283185307179586 * u2));
  b = (R)(r * sin(6.283185307179586 * u2));
}

template <typename T>
__global__ void gaussian_kernel(int64_t n, uint64_t seed, T* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    typename traits<T>::real a, b;
    gauss2(seed, (uint64_t)i, a, b);
    if constexpr (traits<T>::is_complex) out[i] = T(a, b);
    else out[i] = a;
  }
}

}  // namespace tnc

using namespace tnc;

extern "C" {

int tnc_dense_forward(const float* W, const float* bias, const float* in, float* out, int batch, int nin, int nout,
                      int act, void* stream) {
  if (!W || !bias || !in || !out || batch <= 0 || nin <= 0 || nout <= 0 || act < 0 || act > 2) return TNC_ERR_ARG;
  dense_fwd_kernel<<<grid1d((int64_t)batch * nout, 128), 128, 0, (cudaStream_t)stream>>>(W, bias, in, out, batch, nin,
                                                                                      nout, act);
  return launch_status();
}

int tnc_dense_backward(const float* W, const float* in, const float* act_in, const float* g, float* dW, float* db,
                       float* gin, int batch, int nin, int nout, int relu_mask, void* stream) {
  if (!W || !in || !g || !dW || !db || batch <= 0 || nin <= 0 || nout <= 0) return TNC_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  dense_bwd_w_kernel<<<grid1d((int64_t)nout * (nin + 1), 128), 128, 0, st>>>(g, in, dW, db, batch, nin, nout);
  int n = 1;
  if (gin) {
    if (relu_mask && !act_in) return TNC_ERR_ARG;
    dense_bwd_in_kernel<<<grid1d((int64_t)batch * nin, 128), 128, 0, st>>>(W, g, act_in, gin, batch, nin, nout,
                                                                           relu_mask);
    n = 2;
  }
  return launch_status(n);
}

int tnc_mse_sigmoid_grad(const float* y, const float* target, float* g, int batch, void* stream) {
  if (!y || !target || !g || batch <= 0) return TNC_ERR_ARG;
  mse_sigmoid_grad_kernel<<<grid1d(batch, 128), 128, 0, (cudaStream_t)stream>>>(y, target, g, batch);
  return launch_status();
}

int tnc_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, double lr, double beta1,
                  double beta2, double eps, int step, void* stream) {
  if (!params || !grads || !m || !v || n <= 0 || step < 1) return TNC_ERR_ARG;
  const float c1 = (float)(1.0 - pow(beta1, step)), c2 = (float)(1.0 - pow(beta2, step));
  adam_kernel<<<grid1d(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, (float)lr, (float)beta1,
                                                                (float)beta2, (float)eps, c1, c2);
  return launch_status();
}

int tnc_fill_gaussian(int dtype, int64_t n, uint64_t seed, void* out, void* stream) {
  if (n < 0 || !out) return TNC_ERR_ARG;
  if (n == 0) return TNC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  TNC_DISPATCH(dtype, T, gaussian_kernel<T><<<grid1d(n, 256), 256, 0, st>>>(n, seed, (T*)out));
  return launch_status();
}

}  // extern "C"
