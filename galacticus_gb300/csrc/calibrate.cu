// calibrate.cu -- FP64 peak measurement (DFMA throughput) for rooflines.
#include <cuda_runtime.h>
#include "../../include/galnode_calibrate.h"

namespace {
constexpr int CHAINS = 8;
constexpr int ITER = 4096;

__global__ void dfma_loop(double* out, double a, double b) {
  double x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x * 1.0e-3 + c;
  for (int i = 0; i < ITER; ++i) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the loop live
}
}  // namespace

extern "C" int gal_calibrate_fp64(double* flops, double* ms) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 2;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8;
  dfma_loop<<<blocks, threads>>>(out, 0.999999, 1.0e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    dfma_loop<<<blocks, threads>>>(out, 0.999999, 1.0e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    if (t < best) best = t;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return 2;
  const double total = 2.0 * CHAINS * (double)ITER * threads * blocks;
  if (flops) *flops = total / (best * 1.0e-3);
  if (ms) *ms = best;
  return 0;
}
