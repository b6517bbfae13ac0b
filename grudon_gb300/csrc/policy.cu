// Learned round policy: GPU training (forward + backward kernels, Adam) and
// batched inference of the MLP whose per-round inference runs in k_policy.
// No reference counterpart (the reference has no learned component).
//
// Parameters are kept as one flat fp32 master vector in the order
// w1 [64x8], b1 [64], w2 [64x64], b2 [64], w3 [4x64], b3 [4]; every forward
// pass uses the weights rounded to fp16 (the precision inference uses), and
// the gradient is taken with respect to those rounded values.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "kernels.cuh"
#include "policy.cuh"

using namespace grd;

namespace {

thread_local std::string g_policy_error;

constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + P_HID * P_IN;
constexpr int OFF_W2 = OFF_B1 + P_HID;
constexpr int OFF_B2 = OFF_W2 + P_HID * P_HID;
constexpr int OFF_W3 = OFF_B2 + P_HID;
constexpr int OFF_B3 = OFF_W3 + P_OUT * P_HID;
constexpr int NPARAM = OFF_B3 + P_OUT;
static_assert(NPARAM == GRD_POLICY_NPARAM, "parameter layout");

__device__ __forceinline__ bool is_bias(int i) {
  return (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) || i >= OFF_B3;
}

// Flat fp32 parameters -> model (weights rounded to fp16).
__global__ void k_params_to_model(const float* p, grd_policy_model* m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
    const float v = p[i];
    const uint16_t h = __half_as_ushort(__float2half_rn(v));
    if (i < OFF_B1) m->w1[i - OFF_W1] = h;
    else if (i < OFF_W2) m->b1[i - OFF_B1] = v;
    else if (i < OFF_B2) m->w2[i - OFF_W2] = h;
    else if (i < OFF_W3) m->b2[i - OFF_B2] = v;
    else if (i < OFF_B3) m->w3[i - OFF_W3] = h;
    else m->b3[i - OFF_B3] = v;
  }
}

// Forward + backward over samples blockIdx.x, blockIdx.x + gridDim.x, ...;
// one block of P_HID threads, thread j owns hidden unit j of both layers.
// Gradients are accumulated per thread and added to `grad` once per block;
// loss_sum receives the block's sum of masked squared errors.
__global__ void __launch_bounds__(P_HID) k_mlp_grad(const grd_policy_model* m, const float* x, const float* y,
                                                    const uint8_t* mask, uint32_t n, float inv_count, float* grad,
                                                    float* loss_sum) {
  __shared__ float s_x[P_IN], s_h1[P_HID], s_h2[P_HID], s_a1[P_HID], s_a2[P_HID], s_do[P_OUT], s_dh2[P_HID];
  const int j = threadIdx.x;
  float gw1[P_IN], gw2[P_HID], gw3[P_OUT];
#pragma unroll
  for (int i = 0; i < P_IN; ++i) gw1[i] = 0.0f;
#pragma unroll
  for (int k = 0; k < P_HID; ++k) gw2[k] = 0.0f;
#pragma unroll
  for (int o = 0; o < P_OUT; ++o) gw3[o] = 0.0f;
  float gb1 = 0.0f, gb2 = 0.0f, gb3 = 0.0f, loss = 0.0f;
  for (uint32_t s = blockIdx.x; s < n; s += gridDim.x) {
    if (j < P_IN) s_x[j] = policy_input(m, j, x[(size_t)s * P_IN + j]);
    __syncthreads();
    // forward (same arithmetic as mlp_eval)
    float a = m->b1[j];
#pragma unroll
    for (int i = 0; i < P_IN; ++i) a = fmaf(h2f(m->w1[j * P_IN + i]), s_x[i], a);
    s_a1[j] = a;
    s_h1[j] = fmaxf(a, 0.0f);
    __syncthreads();
    a = m->b2[j];
#pragma unroll 8
    for (int k = 0; k < P_HID; ++k) a = fmaf(h2f(m->w2[j * P_HID + k]), s_h1[k], a);
    s_a2[j] = a;
    s_h2[j] = fmaxf(a, 0.0f);
    __syncthreads();
    if (j < P_OUT) {
      float o = m->b3[j];
#pragma unroll 8
      for (int k = 0; k < P_HID; ++k) o = fmaf(h2f(m->w3[j * P_HID + k]), s_h2[k], o);
      const bool on = mask[(size_t)s * P_OUT + j] != 0;
      const float e = on ? o - y[(size_t)s * P_OUT + j] : 0.0f;
      loss = fmaf(e, e, loss);
      s_do[j] = 2.0f * e * inv_count;
    }
    __syncthreads();
    // backward
    float d2 = 0.0f;
#pragma unroll
    for (int o = 0; o < P_OUT; ++o) {
      d2 = fmaf(h2f(m->w3[o * P_HID + j]), s_do[o], d2);
      gw3[o] = fmaf(s_do[o], s_h2[j], gw3[o]);
    }
    if (j < P_OUT) gb3 += s_do[j];
    d2 = s_a2[j] > 0.0f ? d2 : 0.0f;
    s_dh2[j] = d2;
    gb2 += d2;
#pragma unroll
    for (int k = 0; k < P_HID; ++k) gw2[k] = fmaf(d2, s_h1[k], gw2[k]);
    __syncthreads();
    float d1 = 0.0f;
#pragma unroll 8
    for (int r = 0; r < P_HID; ++r) d1 = fmaf(h2f(m->w2[r * P_HID + j]), s_dh2[r], d1);
    d1 = s_a1[j] > 0.0f ? d1 : 0.0f;
    gb1 += d1;
#pragma unroll
    for (int i = 0; i < P_IN; ++i) gw1[i] = fmaf(d1, s_x[i], gw1[i]);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < P_IN; ++i) atomicAdd(&grad[OFF_W1 + j * P_IN + i], gw1[i]);
  atomicAdd(&grad[OFF_B1 + j], gb1);
#pragma unroll
  for (int k = 0; k < P_HID; ++k) atomicAdd(&grad[OFF_W2 + j * P_HID + k], gw2[k]);
  atomicAdd(&grad[OFF_B2 + j], gb2);
#pragma unroll
  for (int o = 0; o < P_OUT; ++o) atomicAdd(&grad[OFF_W3 + o * P_HID + j], gw3[o]);
  if (j < P_OUT) {
    atomicAdd(&grad[OFF_B3 + j], gb3);
    atomicAdd(loss_sum, loss);
  }
}

// AdamW step t (1-based) on the flat fp32 parameters; decoupled weight
// decay on weights only.
__global__ void k_adam(float* p, const float* g, float* mo, float* ve, float lr, float b1, float b2, float eps,
                       float wd, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float m = fmaf(b1, mo[i], (1.0f - b1) * gi);
    const float v = fmaf(b2, ve[i], (1.0f - b2) * gi * gi);
    mo[i] = m;
    ve[i] = v;
    float w = p[i];
    if (!is_bias(i)) w -= lr * wd * w;
    p[i] = w - lr * (m / bc1) / (sqrtf(v / bc2) + eps);
  }
}

// Batched inference: one block of P_HID threads per input.
__global__ void __launch_bounds__(P_HID) k_mlp_predict(const grd_policy_model* m, const float* x, uint32_t n,
                                                       uint32_t allowed, float* out, int32_t* choice) {
  __shared__ float s_x[P_IN], s_h1[P_HID], s_h2[P_HID], s_out[P_OUT];
  MlpRegs r;
  mlp_load(m, r);
  for (uint32_t s = blockIdx.x; s < n; s += gridDim.x) {
    if (threadIdx.x < P_IN) s_x[threadIdx.x] = policy_input(m, threadIdx.x, x[(size_t)s * P_IN + threadIdx.x]);
    __syncthreads();
    mlp_eval(r, s_x, s_h1, s_h2, s_out);
    if (threadIdx.x == 0) {
      int best = -1;
      for (int o = 0; o < P_OUT; ++o) {
        out[(size_t)s * P_OUT + o] = s_out[o];
        if (((allowed >> o) & 1u) && (best < 0 || s_out[o] < s_out[best])) best = o;
      }
      choice[s] = best;
    }
    __syncthreads();
  }
}

// Device buffers of one policy call, freed on scope exit.
struct Scratch {
  std::vector<void*> ptrs;
  cudaStream_t stream = nullptr;
  ~Scratch() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : ptrs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t count) {
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(T) * std::max<size_t>(count, 1));
    if (e == cudaSuccess) ptrs.push_back(d);
    *p = static_cast<T*>(d);
    return e;
  }
};

#define PK(call)                                                             \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      g_policy_error = std::string(#call) + ": " + cudaGetErrorString(e_);   \
      (void)cudaGetLastError();                                              \
      return e_ == cudaErrorMemoryAllocation ? GRD_E_OOM : GRD_E_CUDA;       \
    }                                                                        \
  } while (0)

int grid_blocks(int device, uint32_t n, int per_sm) {
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return (int)std::max<uint32_t>(1, std::min<uint32_t>(n, (uint32_t)(sms * per_sm)));
}

// Masked count of the targets (the loss normaliser).
size_t masked_count(const uint8_t* mask, size_t n) {
  size_t c = 0;
  for (size_t i = 0; i < n * P_OUT; ++i) c += mask[i] ? 1 : 0;
  return c;
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

const char* grd_policy_error(void) { return g_policy_error.c_str(); }

int grd_policy_features(const uint64_t* frontier, const uint64_t* frontier_edges, const uint64_t* unvisited,
                        const uint64_t* max_degree, const uint32_t* round, uint32_t num_vertices, uint64_t num_edges,
                        size_t n, float* features) {
  if (n && (!frontier || !frontier_edges || !unvisited || !max_degree || !round || !features)) return GRD_E_INVALID;
  for (size_t i = 0; i < n; ++i)
    policy_features((double)frontier[i], (double)frontier_edges[i], (double)unvisited[i], (double)max_degree[i],
                    (double)round[i], (double)num_vertices, (double)num_edges, features + i * P_IN);
  return GRD_OK;
}

int grd_policy_grad(const grd_policy_model* model, const float* x, const float* y, const uint8_t* mask, size_t n,
                    int device, float* loss, float* grad) {
  g_policy_error.clear();
  if (!model || !x || !y || !mask || !grad || n == 0 || n > 0xFFFFFFFFull) {
    g_policy_error = "invalid arguments";
    return GRD_E_INVALID;
  }
  const size_t cnt = masked_count(mask, n);
  if (cnt == 0) {
    g_policy_error = "no measured targets";
    return GRD_E_INVALID;
  }
  PK(cudaSetDevice(device));
  Scratch sc;
  PK(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking));
  grd_policy_model* dm;
  float *dx, *dy, *dg, *dl;
  uint8_t* dmask;
  PK(sc.alloc(&dm, 1));
  PK(sc.alloc(&dx, n * P_IN));
  PK(sc.alloc(&dy, n * P_OUT));
  PK(sc.alloc(&dmask, n * P_OUT));
  PK(sc.alloc(&dg, NPARAM));
  PK(sc.alloc(&dl, 1));
  PK(cudaMemcpyAsync(dm, model, sizeof(*model), cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dx, x, sizeof(float) * n * P_IN, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dy, y, sizeof(float) * n * P_OUT, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dmask, mask, n * P_OUT, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemsetAsync(dg, 0, sizeof(float) * NPARAM, sc.stream));
  PK(cudaMemsetAsync(dl, 0, sizeof(float), sc.stream));
  k_mlp_grad<<<grid_blocks(device, (uint32_t)n, 4), P_HID, 0, sc.stream>>>(dm, dx, dy, dmask, (uint32_t)n,
                                                                          1.0f / (float)cnt, dg, dl);
  PK(cudaGetLastError());
  float lsum = 0.0f;
  PK(cudaMemcpyAsync(grad, dg, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, sc.stream));
  PK(cudaMemcpyAsync(&lsum, dl, sizeof(float), cudaMemcpyDeviceToHost, sc.stream));
  PK(cudaStreamSynchronize(sc.stream));
  if (loss) *loss = lsum / (float)cnt;
  return GRD_OK;
}

int grd_policy_train(const float* x, const float* y, const uint8_t* mask, size_t n, const grd_policy_train_cfg* cfg,
                     grd_policy_model* model, float* loss_curve) {
  g_policy_error.clear();
  if (!x || !y || !mask || !cfg || !model || n == 0 || n > 0xFFFFFFFFull || cfg->steps == 0) {
    g_policy_error = "invalid arguments";
    return GRD_E_INVALID;
  }
  const size_t cnt = masked_count(mask, n);
  if (cnt == 0) {
    g_policy_error = "no measured targets";
    return GRD_E_INVALID;
  }
  // Input normalisation from the data (mean 0, unit spread) and the
  // training range every input is clamped to.
  grd_policy_model host{};
  for (int i = 0; i < P_IN; ++i) {
    double s = 0.0, s2 = 0.0;
    float lo = x[i], hi = x[i];
    for (size_t k = 0; k < n; ++k) {
      const double v = x[k * P_IN + i];
      s += v;
      s2 += v * v;
      lo = std::min(lo, x[k * P_IN + i]);
      hi = std::max(hi, x[k * P_IN + i]);
    }
    const double mu = s / (double)n, var = std::max(0.0, s2 / (double)n - mu * mu);
    host.mean[i] = (float)mu;
    host.scale[i] = (float)(1.0 / std::max(std::sqrt(var), 1e-3));
    host.lo[i] = lo;
    host.hi[i] = hi;
  }
  // He-uniform weights, zero biases, output biases at the mean target.
  std::vector<float> p(NPARAM, 0.0f);
  uint64_t rs = cfg->seed;
  auto uni = [&](double lim) { return (float)(((double)(splitmix(rs) >> 11) * 0x1.0p-53 * 2.0 - 1.0) * lim); };
  for (int i = 0; i < P_HID * P_IN; ++i) p[OFF_W1 + i] = uni(std::sqrt(6.0 / P_IN));
  for (int i = 0; i < P_HID * P_HID; ++i) p[OFF_W2 + i] = uni(std::sqrt(6.0 / P_HID));
  for (int i = 0; i < P_OUT * P_HID; ++i) p[OFF_W3 + i] = uni(std::sqrt(6.0 / P_HID) * 0.1);
  for (int o = 0; o < P_OUT; ++o) {
    double s = 0.0;
    size_t c = 0;
    for (size_t k = 0; k < n; ++k)
      if (mask[k * P_OUT + o]) {
        s += y[k * P_OUT + o];
        ++c;
      }
    p[OFF_B3 + o] = c ? (float)(s / (double)c) : 0.0f;
  }
  PK(cudaSetDevice(cfg->device));
  Scratch sc;
  PK(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking));
  grd_policy_model* dm;
  float *dx, *dy, *dp, *dg, *dmo, *dve, *dl;
  uint8_t* dmask;
  PK(sc.alloc(&dm, 1));
  PK(sc.alloc(&dx, n * P_IN));
  PK(sc.alloc(&dy, n * P_OUT));
  PK(sc.alloc(&dmask, n * P_OUT));
  PK(sc.alloc(&dp, NPARAM));
  PK(sc.alloc(&dg, NPARAM));
  PK(sc.alloc(&dmo, NPARAM));
  PK(sc.alloc(&dve, NPARAM));
  PK(sc.alloc(&dl, cfg->steps));
  PK(cudaMemcpyAsync(dm, &host, sizeof(host), cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dx, x, sizeof(float) * n * P_IN, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dy, y, sizeof(float) * n * P_OUT, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dmask, mask, n * P_OUT, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dp, p.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemsetAsync(dmo, 0, sizeof(float) * NPARAM, sc.stream));
  PK(cudaMemsetAsync(dve, 0, sizeof(float) * NPARAM, sc.stream));
  PK(cudaMemsetAsync(dl, 0, sizeof(float) * cfg->steps, sc.stream));
  const int gb = grid_blocks(cfg->device, (uint32_t)n, 4);
  const float b1 = 0.9f, b2 = 0.999f;
  double bc1 = 1.0, bc2 = 1.0;
  for (uint32_t t = 1; t <= cfg->steps; ++t) {
    k_params_to_model<<<20, 256, 0, sc.stream>>>(dp, dm);
    PK(cudaMemsetAsync(dg, 0, sizeof(float) * NPARAM, sc.stream));
    k_mlp_grad<<<gb, P_HID, 0, sc.stream>>>(dm, dx, dy, dmask, (uint32_t)n, 1.0f / (float)cnt, dg, dl + (t - 1));
    bc1 *= b1;
    bc2 *= b2;
    k_adam<<<20, 256, 0, sc.stream>>>(dp, dg, dmo, dve, cfg->lr, b1, b2, 1e-8f, cfg->weight_decay,
                                      (float)(1.0 - bc1), (float)(1.0 - bc2));
    PK(cudaGetLastError());
  }
  k_params_to_model<<<20, 256, 0, sc.stream>>>(dp, dm);
  PK(cudaGetLastError());
  PK(cudaMemcpyAsync(model, dm, sizeof(*model), cudaMemcpyDeviceToHost, sc.stream));
  std::vector<float> curve(cfg->steps);
  PK(cudaMemcpyAsync(curve.data(), dl, sizeof(float) * cfg->steps, cudaMemcpyDeviceToHost, sc.stream));
  PK(cudaStreamSynchronize(sc.stream));
  if (loss_curve)
    for (uint32_t t = 0; t < cfg->steps; ++t) loss_curve[t] = curve[t] / (float)cnt;
  return GRD_OK;
}

int grd_policy_predict(const grd_policy_model* model, const float* x, size_t n, uint32_t allowed_mask, int device,
                       float* out, int32_t* choice) {
  g_policy_error.clear();
  if (!model || !x || !out || !choice || n == 0 || n > 0xFFFFFFFFull || (allowed_mask & 0xFu) == 0) {
    g_policy_error = "invalid arguments";
    return GRD_E_INVALID;
  }
  PK(cudaSetDevice(device));
  Scratch sc;
  PK(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking));
  grd_policy_model* dm;
  float *dx, *dout;
  int32_t* dc;
  PK(sc.alloc(&dm, 1));
  PK(sc.alloc(&dx, n * P_IN));
  PK(sc.alloc(&dout, n * P_OUT));
  PK(sc.alloc(&dc, n));
  PK(cudaMemcpyAsync(dm, model, sizeof(*model), cudaMemcpyHostToDevice, sc.stream));
  PK(cudaMemcpyAsync(dx, x, sizeof(float) * n * P_IN, cudaMemcpyHostToDevice, sc.stream));
  k_mlp_predict<<<grid_blocks(device, (uint32_t)n, 8), P_HID, 0, sc.stream>>>(dm, dx, (uint32_t)n, allowed_mask & 0xFu,
                                                                             dout, dc);
  PK(cudaGetLastError());
  PK(cudaMemcpyAsync(out, dout, sizeof(float) * n * P_OUT, cudaMemcpyDeviceToHost, sc.stream));
  PK(cudaMemcpyAsync(choice, dc, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, sc.stream));
  PK(cudaStreamSynchronize(sc.stream));
  return GRD_OK;
}

}  // extern "C"
