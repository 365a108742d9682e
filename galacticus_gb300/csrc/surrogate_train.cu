// surrogate_train.cu -- training and inference kernels of the cooling-function
// surrogate (3-64-64-64-1 SiLU MLP), and their C ABI.
//
// Training is plain mini-batch Adam on the mean squared error of the
// normalised log10 Lambda, in FP32 throughout: one kernel computes the
// forward and backward pass of a 64-sample slice per block and writes that
// block's gradient; a second sums the block gradients and applies the Adam
// update.  Inference comes in two forms: an FP32 reference kernel, and the
// warp-collective BF16 tensor-core path that the node integrator uses
// (surrogate.cuh), so the error map is measured on the deployed arithmetic.

#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <random>
#include <vector>
#include <numeric>
#include <algorithm>

#include "../../include/galnode_surrogate.h"
#include "surrogate.cuh"

using namespace gal;

namespace {

constexpr int kSlice = 64;      // samples per block in the training kernel
constexpr int kThreads = 256;

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_exact(float z) { return z * sigmoid(z); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = sigmoid(z);
  return s * (1.0f + z * (1.0f - s));
}

// Shared workspace of the training kernel.
struct TrainSmem {
  float p[kMlpParams];
  float x[kSlice][3];
  float y[kSlice];
  float z1[kSlice][kMlpWidth], a1[kSlice][kMlpWidth];
  float z2[kSlice][kMlpWidth], a2[kSlice][kMlpWidth];
  float z3[kSlice][kMlpWidth], a3[kSlice][kMlpWidth];
  float dout[kSlice];
};

// Forward and backward pass over samples idx[base .. base+count) (count <=
// 64) of (x, y); writes d(loss)/d(params) of this block to grad[blockIdx] and
// adds the block's sum of squared errors to *sse.  The loss is
// sum_s (out_s - y_s)^2 / lossNorm.
__global__ void __launch_bounds__(kThreads) mlp_forward_backward(const float* __restrict__ params,
                                                                 const float* __restrict__ xs, const float* __restrict__ ys,
                                                                 const int64_t* __restrict__ idx, int64_t base, int64_t total,
                                                                 float lossNorm, float* __restrict__ grad, float* sse) {
  extern __shared__ float smemRaw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smemRaw);
  const int tid = threadIdx.x;
  const int64_t first = base + (int64_t)blockIdx.x * kSlice;
  const int64_t remaining = base + total - first;
  const int count = remaining <= 0 ? 0 : (remaining < kSlice ? (int)remaining : kSlice);
  for (int i = tid; i < kMlpParams; i += kThreads) S.p[i] = params[i];
  for (int s = tid; s < kSlice; s += kThreads) {
    if (s < count) {
      const int64_t j = idx ? idx[first + s] : first + s;
      S.x[s][0] = xs[3 * j];
      S.x[s][1] = xs[3 * j + 1];
      S.x[s][2] = xs[3 * j + 2];
      S.y[s] = ys[j];
    } else {
      S.x[s][0] = S.x[s][1] = S.x[s][2] = 0.0f;
      S.y[s] = 0.0f;
    }
  }
  __syncthreads();
  const float* W1 = S.p + kW1;
  const float* W2 = S.p + kW2;
  const float* W3 = S.p + kW3;
  const float* W4 = S.p + kW4;
  // Forward.
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, u = e % kMlpWidth;
    const float z = S.p[kB1 + u] + W1[3 * u] * S.x[s][0] + W1[3 * u + 1] * S.x[s][1] + W1[3 * u + 2] * S.x[s][2];
    S.z1[s][u] = z;
    S.a1[s][u] = silu_exact(z);
  }
  __syncthreads();
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, u = e % kMlpWidth;
    float z = S.p[kB2 + u];
    for (int k = 0; k < kMlpWidth; ++k) z += W2[u * kMlpWidth + k] * S.a1[s][k];
    S.z2[s][u] = z;
    S.a2[s][u] = silu_exact(z);
  }
  __syncthreads();
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, u = e % kMlpWidth;
    float z = S.p[kB3 + u];
    for (int k = 0; k < kMlpWidth; ++k) z += W3[u * kMlpWidth + k] * S.a2[s][k];
    S.z3[s][u] = z;
    S.a3[s][u] = silu_exact(z);
  }
  __syncthreads();
  if (tid < kSlice) {
    const int s = tid;
    float out = S.p[kB4];
    for (int k = 0; k < kMlpWidth; ++k) out += W4[k] * S.a3[s][k];
    const float r = s < count ? out - S.y[s] : 0.0f;
    S.dout[s] = 2.0f * r / lossNorm;
    float sq = r * r;
    // Warp-reduce the squared errors of samples 0-31 and 32-63.
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_down_sync(0xffffffffu, sq, o);
    if ((tid & 31) == 0) atomicAdd(sse, sq);
  }
  __syncthreads();
  float* g = grad + (size_t)blockIdx.x * kMlpParams;
  // Output layer gradients; then dz3 = dout W4 silu'(z3), stored over z3.
  for (int k = tid; k < kMlpWidth; k += kThreads) {
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.dout[s] * S.a3[s][k];
    g[kW4 + k] = acc;
  }
  if (tid == 0) {
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.dout[s];
    g[kB4] = acc;
  }
  __syncthreads();
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, k = e % kMlpWidth;
    S.z3[s][k] = S.dout[s] * W4[k] * silu_grad(S.z3[s][k]);
  }
  __syncthreads();
  // Layer 3: gW3[u][k] = sum_s dz3[s][u] a2[s][k]; gb3; dz2 = (dz3 W3) silu'(z2) over z2.
  for (int e = tid; e < kMlpWidth * kMlpWidth; e += kThreads) {
    const int u = e / kMlpWidth, k = e % kMlpWidth;
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.z3[s][u] * S.a2[s][k];
    g[kW3 + e] = acc;
  }
  for (int u = tid; u < kMlpWidth; u += kThreads) {
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.z3[s][u];
    g[kB3 + u] = acc;
  }
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, k = e % kMlpWidth;
    float acc = 0.0f;
    for (int u = 0; u < kMlpWidth; ++u) acc += S.z3[s][u] * W3[u * kMlpWidth + k];
    S.a3[s][k] = acc * silu_grad(S.z2[s][k]);  // a3 is free now: holds dz2
  }
  __syncthreads();
  // Layer 2: gW2, gb2; dz1 = (dz2 W2) silu'(z1), stored over z2.
  for (int e = tid; e < kMlpWidth * kMlpWidth; e += kThreads) {
    const int u = e / kMlpWidth, k = e % kMlpWidth;
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.a3[s][u] * S.a1[s][k];
    g[kW2 + e] = acc;
  }
  for (int u = tid; u < kMlpWidth; u += kThreads) {
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.a3[s][u];
    g[kB2 + u] = acc;
  }
  for (int e = tid; e < kSlice * kMlpWidth; e += kThreads) {
    const int s = e / kMlpWidth, k = e % kMlpWidth;
    float acc = 0.0f;
    for (int u = 0; u < kMlpWidth; ++u) acc += S.a3[s][u] * W2[u * kMlpWidth + k];
    S.z2[s][k] = acc * silu_grad(S.z1[s][k]);
  }
  __syncthreads();
  // Layer 1: gW1[u][i] = sum_s dz1[s][u] x[s][i]; gb1.
  for (int e = tid; e < kMlpWidth * 3; e += kThreads) {
    const int u = e / 3, i = e % 3;
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.z2[s][u] * S.x[s][i];
    g[kW1 + e] = acc;
  }
  for (int u = tid; u < kMlpWidth; u += kThreads) {
    float acc = 0.0f;
    for (int s = 0; s < kSlice; ++s) acc += S.z2[s][u];
    g[kB1 + u] = acc;
  }
}

// Sum the block gradients; optionally apply one Adam step.
__global__ void mlp_reduce_adam(const float* __restrict__ grad, int blocks, float* params, float* m, float* v, float* gradOut,
                                int step, float lr, float beta1, float beta2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  float g = 0.0f;
  for (int b = 0; b < blocks; ++b) g += grad[(size_t)b * kMlpParams + i];
  if (gradOut) gradOut[i] = g;
  if (step > 0) {
    const float mi = beta1 * m[i] + (1.0f - beta1) * g;
    const float vi = beta2 * v[i] + (1.0f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(beta1, (float)step));
    const float vh = vi / (1.0f - powf(beta2, (float)step));
    params[i] -= lr * mh / (sqrtf(vh) + eps);
  }
}

// FP32 reference inference, one thread per sample.
__global__ void mlp_predict_fp32(const float* __restrict__ p, const float* __restrict__ xs, int64_t n, float* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float x0 = xs[3 * s], x1 = xs[3 * s + 1], x2 = xs[3 * s + 2];
  float a1[kMlpWidth], a2[kMlpWidth];
  for (int u = 0; u < kMlpWidth; ++u)
    a1[u] = silu_exact(p[kB1 + u] + p[kW1 + 3 * u] * x0 + p[kW1 + 3 * u + 1] * x1 + p[kW1 + 3 * u + 2] * x2);
  for (int u = 0; u < kMlpWidth; ++u) {
    float z = p[kB2 + u];
    for (int k = 0; k < kMlpWidth; ++k) z += p[kW2 + u * kMlpWidth + k] * a1[k];
    a2[u] = silu_exact(z);
  }
  float y = p[kB4];
  for (int u = 0; u < kMlpWidth; ++u) {
    float z = p[kB3 + u];
    for (int k = 0; k < kMlpWidth; ++k) z += p[kW3 + u * kMlpWidth + k] * a2[k];
    y += p[kW4 + u] * silu_exact(z);
  }
  out[s] = y;
}

// The integrator's BF16 tensor-core inference: each warp evaluates 32 samples.
// Inference with the integrator's tensor-core path (surrogate_eval): the
// packed parameter block (surrogate_pack) is staged into shared memory and
// each warp evaluates 32 samples at a time.
__global__ void mlp_predict_tensor(const float* __restrict__ small, const __nv_bfloat16* __restrict__ planes,
                                   const float* __restrict__ xs, int64_t n, float* __restrict__ out) {
  __shared__ float sSmall[(kSurrSmall + 3) & ~3];
  __shared__ __align__(16) __nv_bfloat16 sPlanes[4 * kSurrPlane];
  for (int i = threadIdx.x; i < kSurrSmall; i += blockDim.x) sSmall[i] = small[i];
  for (int i = threadIdx.x; i < 4 * kSurrPlane / 2; i += blockDim.x)
    reinterpret_cast<uint32_t*>(sPlanes)[i] = reinterpret_cast<const uint32_t*>(planes)[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const SurrogateSmem N = surrogate_view(sSmall, sPlanes);
  const int64_t warpsTotal = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t base = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * 32; base < n; base += warpsTotal * 32) {
    const int64_t s = base + lane;
    const bool ok = s < n;
    const float y = surrogate_eval(N, ok ? xs[3 * s] : 0.0f, ok ? xs[3 * s + 1] : 0.0f, ok ? xs[3 * s + 2] : 0.0f, lane,
                                   __ballot_sync(0xffffffffu, ok));
    if (ok) out[s] = y;
  }
}

int fail_code(cudaError_t e) { return e == cudaSuccess ? GAL_OK : GAL_ERR_CUDA; }

}  // namespace

extern "C" {

int gal_surrogate_param_count(void) { return kMlpParams; }

int gal_surrogate_gradient(const float* params, const float* x, const float* y, int64_t n, float* grad, float* loss) {
  if (!params || !x || !y || !grad || n < 1 || n > (1 << 20)) return GAL_ERR_ARGUMENT;
  const int blocks = (int)((n + kSlice - 1) / kSlice);
  float *dP = nullptr, *dX = nullptr, *dY = nullptr, *dG = nullptr, *dGo = nullptr, *dSse = nullptr;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&dP, kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dX, n * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dY, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dG, (size_t)blocks * kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dGo, kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dSse, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dP, params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, x, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dY, y, n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dSse, 0, sizeof(float));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(mlp_forward_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
  if (e == cudaSuccess) {
    mlp_forward_backward<<<blocks, kThreads, sizeof(TrainSmem)>>>(dP, dX, dY, nullptr, 0, n, (float)n, dG, dSse);
    mlp_reduce_adam<<<(kMlpParams + 255) / 256, 256>>>(dG, blocks, dP, nullptr, nullptr, dGo, 0, 0.f, 0.f, 0.f, 0.f);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(grad, dGo, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost);
  float sse = 0.0f;
  if (e == cudaSuccess) e = cudaMemcpy(&sse, dSse, sizeof(float), cudaMemcpyDeviceToHost);
  if (loss) *loss = sse / (float)n;
  cudaFree(dP); cudaFree(dX); cudaFree(dY); cudaFree(dG); cudaFree(dGo); cudaFree(dSse);
  return fail_code(e);
}

int gal_surrogate_train(const gal_surrogate_train_config* cfg, const float* xTrain, const float* yTrain, int64_t nTrain,
                        const float* xVal, const float* yVal, int64_t nVal, float* params, float* history) {
  if (!cfg || !xTrain || !yTrain || !params || nTrain < 1 || cfg->batch_size < 1 || cfg->batch_size % kSlice ||
      cfg->epochs < 1)
    return GAL_ERR_ARGUMENT;
  const int64_t batch = cfg->batch_size;
  const int blocks = (int)(batch / kSlice);
  float *dP = nullptr, *dM = nullptr, *dV = nullptr, *dX = nullptr, *dY = nullptr, *dG = nullptr, *dSse = nullptr;
  float *dXv = nullptr, *dYv = nullptr, *dOut = nullptr;
  int64_t* dIdx = nullptr;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes); };
  alloc((void**)&dP, kMlpParams * sizeof(float));
  alloc((void**)&dM, kMlpParams * sizeof(float));
  alloc((void**)&dV, kMlpParams * sizeof(float));
  alloc((void**)&dX, nTrain * 3 * sizeof(float));
  alloc((void**)&dY, nTrain * sizeof(float));
  alloc((void**)&dIdx, nTrain * sizeof(int64_t));
  alloc((void**)&dG, (size_t)blocks * kMlpParams * sizeof(float));
  alloc((void**)&dSse, sizeof(float));
  if (nVal > 0) {
    alloc((void**)&dXv, nVal * 3 * sizeof(float));
    alloc((void**)&dYv, nVal * sizeof(float));
    alloc((void**)&dOut, nVal * sizeof(float));
  }
  if (e == cudaSuccess) e = cudaMemcpy(dP, params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dM, 0, kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(dV, 0, kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dX, xTrain, nTrain * 3 * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dY, yTrain, nTrain * sizeof(float), cudaMemcpyHostToDevice);
  if (nVal > 0 && e == cudaSuccess) e = cudaMemcpy(dXv, xVal, nVal * 3 * sizeof(float), cudaMemcpyHostToDevice);
  if (nVal > 0 && e == cudaSuccess) e = cudaMemcpy(dYv, yVal, nVal * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(mlp_forward_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
  std::mt19937_64 rng((uint64_t)cfg->seed);
  std::vector<int64_t> perm(nTrain);
  std::vector<float> out((size_t)std::max<int64_t>(nVal, 1));
  int step = 0;
  const int64_t steps = nTrain / batch;  // the last partial batch of each epoch is dropped
  // Cosine decay from learning_rate to learning_rate_final over the run
  // (constant when the final rate is not positive or equals the initial one).
  const double lr0 = cfg->learning_rate, lr1 = cfg->learning_rate_final;
  const bool decay = lr1 > 0.0 && lr1 != lr0;
  const double totalSteps = (double)steps * cfg->epochs;
  auto rate = [&](int k) -> float {
    if (!decay || totalSteps <= 1.0) return (float)lr0;
    return (float)(lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(3.14159265358979323846 * (k - 1) / (totalSteps - 1.0))));
  };
  for (int epoch = 0; epoch < cfg->epochs && e == cudaSuccess; ++epoch) {
    std::iota(perm.begin(), perm.end(), 0);
    std::shuffle(perm.begin(), perm.end(), rng);
    e = cudaMemcpy(dIdx, perm.data(), nTrain * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dSse, 0, sizeof(float));
    for (int64_t b = 0; b < steps && e == cudaSuccess; ++b) {
      ++step;
      mlp_forward_backward<<<blocks, kThreads, sizeof(TrainSmem)>>>(dP, dX, dY, dIdx, b * batch, batch, (float)batch, dG, dSse);
      mlp_reduce_adam<<<(kMlpParams + 255) / 256, 256>>>(dG, blocks, dP, dM, dV, nullptr, step, rate(step), cfg->beta1,
                                                         cfg->beta2, cfg->epsilon);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    float sse = 0.0f;
    if (e == cudaSuccess) e = cudaMemcpy(&sse, dSse, sizeof(float), cudaMemcpyDeviceToHost);
    float valLoss = 0.0f;
    if (nVal > 0 && e == cudaSuccess) {
      mlp_predict_fp32<<<(unsigned)((nVal + 255) / 256), 256>>>(dP, dXv, nVal, dOut);
      e = cudaMemcpy(out.data(), dOut, nVal * sizeof(float), cudaMemcpyDeviceToHost);
      double acc = 0.0;
      for (int64_t i = 0; i < nVal; ++i) acc += (double)(out[i] - yVal[i]) * (out[i] - yVal[i]);
      valLoss = (float)(acc / nVal);
    }
    if (history) {
      history[2 * epoch] = sse / (float)(steps * batch);
      history[2 * epoch + 1] = valLoss;
    }
  }
  if (e == cudaSuccess) e = cudaMemcpy(params, dP, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dP); cudaFree(dM); cudaFree(dV); cudaFree(dX); cudaFree(dY); cudaFree(dIdx); cudaFree(dG); cudaFree(dSse);
  cudaFree(dXv); cudaFree(dYv); cudaFree(dOut);
  return fail_code(e);
}

int gal_surrogate_predict(const float* params, const float* x, int64_t n, float* y, int32_t tensorCores) {
  if (!params || !x || !y || n < 1) return GAL_ERR_ARGUMENT;
  std::vector<float> small(kSurrSmall);
  std::vector<__nv_bfloat16> planes(4 * kSurrPlane);
  surrogate_pack(params, small.data(), planes.data());
  float *dP = nullptr, *dX = nullptr, *dY = nullptr, *dSmall = nullptr;
  __nv_bfloat16* dPlanes = nullptr;
  cudaError_t e = cudaMalloc(&dP, kMlpParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dSmall, kSurrSmall * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dPlanes, planes.size() * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&dX, n * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dY, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dP, params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dSmall, small.data(), kSurrSmall * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(dPlanes, planes.data(), planes.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, x, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    if (tensorCores)
      mlp_predict_tensor<<<(unsigned)std::min<int64_t>((n + 127) / 128, 4096), 128>>>(dSmall, dPlanes, dX, n, dY);
    else mlp_predict_fp32<<<(unsigned)((n + 255) / 256), 256>>>(dP, dX, n, dY);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(y, dY, n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dP); cudaFree(dX); cudaFree(dY); cudaFree(dSmall); cudaFree(dPlanes);
  return fail_code(e);
}

}  // extern "C"
