// The learned cost model: a small fp32 MLP (structure features -> predicted
// log time of every tuner configuration), with its training kernels.
//
// Network: x -> (x - mu) / sigma -> [Linear -> GELU] x layers -> Linear; the
// outputs are ln(time in microseconds), one per tuner configuration.
// Parameters live in one flat fp32 array:
//   mu[in], sigma[in]                      (input normalisation, not trained)
//   W0[hidden x in], b0[hidden]            (row-major: W[o * fan_in + i])
//   W1..W{layers-1}[hidden x hidden], b
//   W_out[out x hidden], b_out[out]
// GELU is the exact form 0.5 x (1 + erf(x / sqrt 2)).
//
// Training minimises the masked mean squared error over (sample, config)
// pairs with mask 1: loss = sum(mask (y - t)^2) / sum(mask). The backward pass
// keeps every layer's pre-activation Z and activation A in a workspace;
// weight gradients reduce over the batch inside one CTA per output unit, so
// the gradient is deterministic. Adam updates only the trained range.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include "internal.h"

namespace spmm {
namespace {

struct Layout {
  int in, hidden, layers, out;
  long long norm_floats() const { return 2LL * in; }
  int fan_in(int l) const { return l == 0 ? in : hidden; }
  int fan_out(int l) const { return l == layers ? out : hidden; }
  long long w_off(int l) const {
    long long o = norm_floats();
    for (int k = 0; k < l; ++k) o += (long long)fan_out(k) * fan_in(k) + fan_out(k);
    return o;
  }
  long long b_off(int l) const { return w_off(l) + (long long)fan_out(l) * fan_in(l); }
  long long params() const { return w_off(layers + 1); }
  // workspace: Xn[B x in], per hidden layer Z[B x hidden] and A[B x hidden], Y[B x out],
  // two gradient buffers [B x max(hidden, out)]
  long long ws(int batch) const {
    const int wmax = hidden > out ? hidden : out;
    return (long long)batch * (in + 2LL * hidden * layers + out + 2LL * wmax);
  }
};

bool valid(const spmm_mlp_shape* s) {
  // fan-ins up to 128 keep a 64-row slice of a layer's input within 32 KB of shared memory
  return s && s->in > 0 && s->hidden > 0 && s->layers > 0 && s->out > 0 && s->in <= 128 && s->hidden <= 128 &&
         s->out <= 1024 && s->layers <= 16;
}
Layout layout(const spmm_mlp_shape* s) { return Layout{s->in, s->hidden, s->layers, s->out}; }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void k_normalize(const float* __restrict__ X, const float* __restrict__ mu,
                            const float* __restrict__ sigma, int batch, int in, float* __restrict__ Xn) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)batch * in) return;
  const int f = (int)(i % in);
  Xn[i] = (X[i] - mu[f]) / sigma[f];
}

// Z[b][o] = sum_i X[b][i] W[o][i] + bias[o]; A = GELU(Z) when A != NULL.
// One thread per (b, o); the CTA's 64-row slice of X is staged in shared memory.
__global__ void k_dense(const float* __restrict__ X, const float* __restrict__ W, const float* __restrict__ bias,
                        int batch, int I, int O, float* __restrict__ Z, float* __restrict__ A) {
  extern __shared__ float sx[];   // [rows x I]
  constexpr int rows = 64;
  const int b0 = blockIdx.x * rows;
  for (int t = threadIdx.x; t < rows * I; t += blockDim.x) {
    const int r = t / I, i = t % I;
    sx[t] = (b0 + r < batch) ? X[(long long)(b0 + r) * I + i] : 0.f;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < rows * O; t += blockDim.x) {
    const int r = t / O, o = t % O;
    if (b0 + r >= batch) continue;
    const float* w = W + (long long)o * I;
    const float* x = sx + r * I;
    float acc = bias[o];
    for (int i = 0; i < I; ++i) acc = fmaf(x[i], __ldg(w + i), acc);
    Z[(long long)(b0 + r) * O + o] = acc;
    if (A) A[(long long)(b0 + r) * O + o] = gelu(acc);
  }
}

// Masked MSE: loss = sum(m (y - t)^2) / sum(m); dY = 2 m (y - t) / sum(m).
// One CTA (the batch is small); sums in double for a stable loss value.
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ M,
                      long long n, float* __restrict__ dY, float* __restrict__ loss) {
  __shared__ double s_sum[1024], s_cnt[1024];
  double sum = 0, cnt = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float m = M[i];
    if (m != 0.f) {
      const double d = (double)Y[i] - (double)T[i];
      sum += m * d * d;
      cnt += m;
    }
  }
  s_sum[threadIdx.x] = sum;
  s_cnt[threadIdx.x] = cnt;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_sum[threadIdx.x] += s_sum[threadIdx.x + w];
      s_cnt[threadIdx.x] += s_cnt[threadIdx.x + w];
    }
    __syncthreads();
  }
  const double total = s_cnt[0] > 0 ? s_cnt[0] : 1.0;
  if (threadIdx.x == 0 && loss) *loss = (float)(s_sum[0] / total);
  const float scale = (float)(2.0 / total);
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float m = M[i];
    dY[i] = m != 0.f ? scale * m * (Y[i] - T[i]) : 0.f;
  }
}

// dW[o][i] = sum_b dZ[b][o] X[b][i]; db[o] = sum_b dZ[b][o]. One CTA per o;
// thread t takes input i = t % I and the batch rows b = t / I (mod slices).
__global__ void k_dweight(const float* __restrict__ dZ, const float* __restrict__ X, int batch, int I, int O,
                          float* __restrict__ dW, float* __restrict__ db) {
  extern __shared__ float red[];   // [blockDim.x] + [slices]
  const int o = blockIdx.x;
  const int slices = blockDim.x / I;
  const int t = threadIdx.x;
  const int i = t % I, sl = t / I;
  float acc = 0.f, accb = 0.f;
  if (sl < slices) {
    for (int b = sl; b < batch; b += slices) {
      const float g = dZ[(long long)b * O + o];
      acc = fmaf(g, X[(long long)b * I + i], acc);
      if (i == 0) accb += g;
    }
  }
  red[t] = acc;
  float* redb = red + blockDim.x;
  if (i == 0 && sl < slices) redb[sl] = accb;
  __syncthreads();
  if (t < I) {
    float s = 0.f;
    for (int k = 0; k < slices; ++k) s += red[k * I + t];
    dW[(long long)o * I + t] = s;
  }
  if (t == 0) {
    float s = 0.f;
    for (int k = 0; k < slices; ++k) s += redb[k];
    db[o] = s;
  }
}

// dX[b][i] = sum_o dZ[b][o] W[o][i], then times GELU'(Zprev[b][i]) when Zprev != NULL.
__global__ void k_dinput(const float* __restrict__ dZ, const float* __restrict__ W, int batch, int I, int O,
                         const float* __restrict__ Zprev, float* __restrict__ dX) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)batch * I) return;
  const int b = (int)(k / I), i = (int)(k % I);
  const float* g = dZ + (long long)b * O;
  float acc = 0.f;
  for (int o = 0; o < O; ++o) acc = fmaf(g[o], __ldg(W + (long long)o * I + i), acc);
  if (Zprev) acc *= gelu_grad(Zprev[k]);
  dX[k] = acc;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float wd,
                       float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mhat = mi / c1, vhat = vi / c2;
  p[i] -= lr * (mhat / (sqrtf(vhat) + eps) + wd * p[i]);
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// Forward pass into the workspace; returns the pointer to Y inside it.
spmm_status forward_ws(const Layout& L, const float* params, const float* X, int batch, float* ws,
                       cudaStream_t s, float** Y_out) {
  float* Xn = ws;
  float* cur = Xn;
  k_normalize<<<blocks_for((long long)batch * L.in, 256), 256, 0, s>>>(X, params, params + L.in, batch, L.in, Xn);
  float* p = Xn + (long long)batch * L.in;
  for (int l = 0; l <= L.layers; ++l) {
    const int I = L.fan_in(l), O = L.fan_out(l);
    float* Z = p;
    float* A = l < L.layers ? p + (long long)batch * O : nullptr;
    const size_t sm = (size_t)64 * I * sizeof(float);
    k_dense<<<blocks_for(batch, 64), 256, sm, s>>>(cur, params + L.w_off(l), params + L.b_off(l), batch, I, O, Z,
                                                   A);
    if (l < L.layers) {
      cur = A;
      p += 2LL * batch * O;
    } else {
      *Y_out = Z;
    }
  }
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

}  // namespace
}  // namespace spmm

using namespace spmm;

struct spmm_cost_model {
  spmm_mlp_shape shape;
  float* d_params = nullptr;
  float* d_ws = nullptr;    // workspace for a batch of one
  float* d_x = nullptr;
  int device = -1;
};

extern "C" {

long long spmm_mlp_param_count(const spmm_mlp_shape* shape) {
  return valid(shape) ? layout(shape).params() : -1;
}

long long spmm_mlp_workspace_floats(const spmm_mlp_shape* shape, int batch) {
  return valid(shape) && batch > 0 ? layout(shape).ws(batch) : -1;
}

spmm_status spmm_mlp_forward(const spmm_mlp_shape* shape, const float* params, const float* X, int batch,
                             float* Y, float* work, void* stream) {
  if (!valid(shape) || !params || !X || !Y || !work || batch <= 0)
    return fail(SPMM_ERR_INVALID_ARG, "bad MLP forward arguments");
  const Layout L = layout(shape);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float* Yw = nullptr;
  spmm_status st = forward_ws(L, params, X, batch, work, s, &Yw);
  if (st != SPMM_OK) return st;
  SPMM_CUDA_TRY(cudaMemcpyAsync(Y, Yw, sizeof(float) * batch * L.out, cudaMemcpyDeviceToDevice, s));
  return SPMM_OK;
}

spmm_status spmm_mlp_backward(const spmm_mlp_shape* shape, const float* params, const float* X, const float* T,
                              const float* mask, int batch, float* grad, float* loss, float* work, void* stream) {
  if (!valid(shape) || !params || !X || !T || !mask || !grad || !work || batch <= 0)
    return fail(SPMM_ERR_INVALID_ARG, "bad MLP backward arguments");
  const Layout L = layout(shape);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float* Y = nullptr;
  spmm_status st = forward_ws(L, params, X, batch, work, s, &Y);
  if (st != SPMM_OK) return st;
  const int wmax = L.hidden > L.out ? L.hidden : L.out;
  float* g0 = Y + (long long)batch * L.out;
  float* g1 = g0 + (long long)batch * wmax;
  SPMM_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(float) * L.norm_floats(), s));
  k_mse<<<1, 1024, 0, s>>>(Y, T, mask, (long long)batch * L.out, g0, loss);
  // layer l's input activation: Xn for l = 0, else A_{l-1}; its pre-activation Z_{l-1}
  auto act_in = [&](int l) -> const float* {
    if (l == 0) return work;
    return work + (long long)batch * L.in + (2LL * (l - 1) + 1) * batch * L.hidden;
  };
  auto z_of = [&](int l) -> const float* {   // Z of hidden layer l
    return work + (long long)batch * L.in + 2LL * l * batch * L.hidden;
  };
  float* dZ = g0;
  float* dX = g1;
  for (int l = L.layers; l >= 0; --l) {
    const int I = L.fan_in(l), O = L.fan_out(l);
    const int slices = 256 / I > 0 ? 256 / I : 1;
    const int threads = slices * I <= 1024 ? slices * I : I;
    k_dweight<<<O, threads, sizeof(float) * (threads + slices), s>>>(dZ, act_in(l), batch, I, O,
                                                                     grad + L.w_off(l), grad + L.b_off(l));
    if (l > 0) {
      k_dinput<<<blocks_for((long long)batch * I, 256), 256, 0, s>>>(dZ, params + L.w_off(l), batch, I, O,
                                                                     z_of(l - 1), dX);
      float* t = dZ;
      dZ = dX;
      dX = t;
    }
  }
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_mlp_adam(float* params, const float* grad, float* m, float* v, long long n, long long offset,
                          float lr, float beta1, float beta2, float eps, float weight_decay, int step,
                          void* stream) {
  if (!params || !grad || !m || !v || n <= 0 || offset < 0 || offset >= n || step < 1)
    return fail(SPMM_ERR_INVALID_ARG, "bad Adam arguments");
  const long long cnt = n - offset;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<blocks_for(cnt, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      params + offset, grad + offset, m + offset, v + offset, cnt, lr, beta1, beta2, eps, weight_decay, c1, c2);
  SPMM_CUDA_TRY(cudaGetLastError());
  return SPMM_OK;
}

spmm_status spmm_cost_model_create(const spmm_mlp_shape* shape, const float* host_params,
                                   spmm_cost_model** out) {
  if (!out) return fail(SPMM_ERR_INVALID_ARG, "null output");
  *out = nullptr;
  if (!valid(shape) || !host_params) return fail(SPMM_ERR_INVALID_ARG, "bad cost model arguments");
  if (shape->out != spmm_tune_config_count())
    return fail(SPMM_ERR_INVALID_ARG, "the model must predict one time per tuner configuration");
  const Layout L = layout(shape);
  spmm_cost_model* m = new spmm_cost_model();
  m->shape = *shape;
  cudaGetDevice(&m->device);
  cudaError_t ce = cudaMalloc(&m->d_params, sizeof(float) * L.params());
  if (ce == cudaSuccess)
    ce = cudaMemcpy(m->d_params, host_params, sizeof(float) * L.params(), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMalloc(&m->d_ws, sizeof(float) * L.ws(1));
  if (ce == cudaSuccess) ce = cudaMalloc(&m->d_x, sizeof(float) * (L.in + L.out));
  if (ce != cudaSuccess) {
    spmm_cost_model_destroy(m);
    return cuda_fail(ce, "creating the cost model");
  }
  *out = m;
  return SPMM_OK;
}

spmm_status spmm_cost_model_load(const char* path, spmm_cost_model** out) {
  if (!path || !out) return fail(SPMM_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(SPMM_ERR_INVALID_ARG, std::string("cannot open ") + path);
  char magic[8];
  int32_t dims[4];
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "SPMMCM01", 8) == 0 &&
            std::fread(dims, sizeof(int32_t), 4, f) == 4;
  spmm_mlp_shape s{dims[0], dims[1], dims[2], dims[3]};
  std::vector<float> params;
  if (ok && valid(&s)) {
    params.resize((size_t)layout(&s).params());
    ok = std::fread(params.data(), sizeof(float), params.size(), f) == params.size();
  } else {
    ok = false;
  }
  std::fclose(f);
  if (!ok) return fail(SPMM_ERR_INVALID_ARG, std::string("not a cost model file: ") + path);
  return spmm_cost_model_create(&s, params.data(), out);
}

spmm_status spmm_cost_model_destroy(spmm_cost_model* m) {
  if (!m) return SPMM_OK;
  if (m->d_params) cudaFree(m->d_params);
  if (m->d_ws) cudaFree(m->d_ws);
  if (m->d_x) cudaFree(m->d_x);
  delete m;
  return SPMM_OK;
}

spmm_status spmm_cost_model_select(const spmm_cost_model* m, const spmm_bcsr_desc* A, int N, spmm_config* out,
                                   float* predicted, void* stream) {
  if (!m || !A || !out) return fail(SPMM_ERR_INVALID_ARG, "null argument");
  const Layout L = layout(&m->shape);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (L.in != SPMM_FEATURES) return fail(SPMM_ERR_INVALID_ARG, "the model's input must be the structure features");
  std::vector<float> f(SPMM_FEATURES, 0.f), y(L.out);
  spmm_status st = spmm_structure_features(A, N, f.data(), stream);
  if (st != SPMM_OK) return st;
  SPMM_CUDA_TRY(cudaMemcpyAsync(m->d_x, f.data(), sizeof(float) * L.in, cudaMemcpyHostToDevice, s));
  float* Y = nullptr;
  st = forward_ws(L, m->d_params, m->d_x, 1, m->d_ws, s, &Y);
  if (st != SPMM_OK) return st;
  SPMM_CUDA_TRY(cudaMemcpyAsync(y.data(), Y, sizeof(float) * L.out, cudaMemcpyDeviceToHost, s));
  SPMM_CUDA_TRY(cudaStreamSynchronize(s));
  int best = -1;
  for (int i = 0; i < L.out; ++i) {
    spmm_config c;
    spmm_tune_config(i, &c);
    const bool ok = spmm_config_supported(A->bR, A->dtype, N, &c) == SPMM_OK;
    if (predicted) predicted[i] = ok ? std::exp(y[i]) * 1e-3f : INFINITY;   // outputs are ln(microseconds)
    if (ok && (best < 0 || y[i] < y[best])) best = i;
  }
  if (best < 0) return fail(SPMM_ERR_UNSUPPORTED, "no configuration runs this product");
  return spmm_tune_config(best, out);
}

}  // extern "C"
