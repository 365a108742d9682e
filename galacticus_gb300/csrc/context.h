// context.h -- the evolution context shared by the host-side translation
// units (galnode.cu: batches and the surrogate; forest.cu: forests).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

#include "../../include/galnode.h"
#include "evolve_kernel.cuh"

using namespace gal;

struct gal_ctx {
  gal_params params;
  Globals globals;
  int device = 0;
  int smCount = 0;
  cudaStream_t stream = nullptr;
  double2* dTab = nullptr;
  double* dLnT = nullptr;
  double* dLnZ = nullptr;
  double2* dFastLog = nullptr;           // tables of the short FP64 log/exp
  double* dFastExp = nullptr;
  float2* dTabF = nullptr;               // FP32 copies of the tables (FP32-rate forms)
  float* dLnZF = nullptr;
  double* dKmt = nullptr;                // Krumholz (2009) tables: molecular fraction, then x^0.33
  float* dKmtF = nullptr;                // their FP32 copies
  unsigned long long* dQueue = nullptr;  // work-queue head
  // The surrogate forms' split launch: the two work lists [2][orderCap],
  // their lengths and queue heads (4 counters), a second stream, fork and
  // join events.
  int32_t* dOrder = nullptr;
  unsigned long long* dOrderCount = nullptr;
  int64_t orderCap = 0;
  cudaStream_t stream2 = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  int splitSurrogate = 1;
  void* dBuf = nullptr;                  // staging for the host-pointer API
  // Installed cooling-function surrogate (dSurrSmall == nullptr: none).
  float* dSurrSmall = nullptr;
  __nv_bfloat16* dSurrPlanes = nullptr;
  uint8_t* dSurrMap = nullptr;
  unsigned long long* dSurrStats = nullptr;
  SurrogateInfo surrInfo{};
  size_t bufBytes = 0;
  int threads = 128;
  int blocksPerSm = 1;
  int ratePrecision = GAL_RATES_FP64;
  int64_t launches = 0;
  int lastError = 0;
  char message[512] = {0};
};


namespace gal {
namespace host {

// Record an error (in the context, or thread-locally without one) and return code.
int fail(gal_ctx* ctx, int code, const char* fmt, const char* detail = "");
// The kernel form of the context: rate precision and surrogate.
int ctx_mode(const gal_ctx* ctx);
size_t ctx_shared_bytes(const gal_ctx* ctx, int mode);
// Block sizes each form is built for (evolve_*.cu).
bool mode_has_threads(int mode, int threads);
// The launch shape in use for a form.
void effective_shape(const gal_ctx* ctx, int mode, int& threads, int& blocksPerSm);
// The device tables of the context.
DeviceTables ctx_tables(const gal_ctx* ctx);

}  // namespace host
}  // namespace gal
