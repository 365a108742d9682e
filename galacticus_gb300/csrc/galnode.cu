// galnode.cu -- batched node evolution on GB300 (sm_103a) and its C ABI.
//
// Hot path: gal_gpu_evolve_batch[_device] -> evolve_kernel.  One thread owns
// one node at a time and integrates it with the Cash-Karp 4(5) stepper and
// the reference's scaled error controller, trial loop and post-step clamps
// (merger_trees/node_evolver/standard.F90:385-755, numerical/ODE_solver/
// solver.F90:492-691, external/gslODEInitVal2/driver2.c:148-250,
// cscal2.c:93-169).  The kernel is persistent: each warp loops over RK
// attempts, and a lane whose node has finished takes the next node from a
// device work queue (one atomic per warp), so lanes stay busy however uneven
// the per-node step counts are.  State, stages and step control are FP64 in
// registers; the CIE tables are staged in shared memory once per block.

#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <new>
#include <vector>
#include <algorithm>

#include "../../include/galnode.h"
#include "galnode_physics.cuh"

namespace gal {

constexpr unsigned FULL = 0xffffffffu;

// Cash-Karp 4(5) tableau (Cash & Karp 1990, ACM TOMS 16, 201).  The node
// right-hand side has no explicit time dependence (halo mass growth enters
// through the constant accretion rate), so the stage abscissae are unused.
namespace ck {
constexpr double b21 = 1.0 / 5.0;
constexpr double b31 = 3.0 / 40.0, b32 = 9.0 / 40.0;
constexpr double b41 = 3.0 / 10.0, b42 = -9.0 / 10.0, b43 = 6.0 / 5.0;
constexpr double b51 = -11.0 / 54.0, b52 = 5.0 / 2.0, b53 = -70.0 / 27.0, b54 = 35.0 / 27.0;
constexpr double b61 = 1631.0 / 55296.0, b62 = 175.0 / 512.0, b63 = 575.0 / 13824.0, b64 = 44275.0 / 110592.0,
                 b65 = 253.0 / 4096.0;
constexpr double c1 = 37.0 / 378.0, c3 = 250.0 / 621.0, c4 = 125.0 / 594.0, c6 = 512.0 / 1771.0;
constexpr double e1 = 37.0 / 378.0 - 2825.0 / 27648.0, e3 = 250.0 / 621.0 - 18575.0 / 48384.0,
                 e4 = 125.0 / 594.0 - 13525.0 / 55296.0, e5 = -277.0 / 14336.0, e6 = 512.0 / 1771.0 - 0.25;
constexpr double order = 5.0;  // order GSL's rkck reports to the step controller
}  // namespace ck

enum Phase : int { PH_NEED = 0, PH_TRIAL = 1, PH_STEP = 2, PH_DONE = 3 };

struct Batch {
  int64_t n;
  double* state;
  const double* param;
  const double* tStart;
  const double* tEnd;
  double* step;
  int32_t* status;
  uint32_t* counters;
  unsigned long long* queue;  // work-queue head (device scratch, zeroed before launch)
};

// Shared-memory layout: [nZ*nT] double2 tables, then ln T [nT], ln Z [nZ]
// and 1/(ln Z[i+1] - ln Z[i]) [nZ].
__host__ __device__ inline size_t shared_bytes(int nT, int nZ) {
  return (size_t)nZ * nT * sizeof(double2) + (size_t)(nT + 2 * nZ) * sizeof(double);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS, 1)
evolve_kernel(const __grid_constant__ Globals G, Batch b, const double2* __restrict__ gTab, const double* __restrict__ gLnT,
              const double* __restrict__ gLnZ) {
  extern __shared__ double2 smem[];
  const int nT = G.nT, nZ = G.nZ;
  double2* sTab = smem;
  double* sLnT = reinterpret_cast<double*>(sTab + nZ * nT);
  double* sLnZ = sLnT + nT;
  double* sInvDlnZ = sLnZ + nZ;
  for (int i = threadIdx.x; i < nZ * nT; i += blockDim.x) sTab[i] = gTab[i];
  for (int i = threadIdx.x; i < nT; i += blockDim.x) sLnT[i] = gLnT[i];
  for (int i = threadIdx.x; i < 2 * nZ; i += blockDim.x) sLnZ[i] = gLnZ[i];  // ln Z, then the reciprocal spacings
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int64_t n = b.n;
  const double epsAbs = G.p.ode_tolerance_absolute, epsRel = G.p.ode_tolerance_relative;
  const uint32_t budget = (uint32_t)max(G.p.step_budget, 0);

  int phase = PH_NEED;
  int64_t node = 0;
  NodeC c;
  double y[GAL_NY], s[GAL_NY], k1[GAL_NY], k2[GAL_NY], k3[GAL_NY], k4[GAL_NY], k5[GAL_NY], k6[GAL_NY], tmp[GAL_NY];
  double t = 0.0, t0 = 0.0, t1 = 0.0, h = 0.0, stepIn = -1.0;
  int trial = 0;
  uint32_t count = 0, nAcc = 0, nRej = 0, nRhs = 0;

  for (;;) {
    // ---- refill lanes whose node has finished (warp-aggregated queue pop)
    const unsigned need = __ballot_sync(FULL, phase == PH_NEED);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(b.queue, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (phase == PH_NEED) {
        node = (int64_t)(base + __popc(need & ((1u << lane) - 1u)));
        if (node >= n) {
          phase = PH_DONE;
        } else {
          double prm[GAL_NP];
#pragma unroll
          for (int v = 0; v < GAL_NP; ++v) prm[v] = b.param[v * n + node];
          node_setup(G, sLnT, prm, c);
#pragma unroll
          for (int v = 0; v < GAL_NY; ++v) y[v] = b.state[v * n + node];
          scales(y, c.massHalo, s);
          t0 = b.tStart[node];
          t1 = b.tEnd[node];
          stepIn = b.step[node];
          trial = 0;
          nAcc = nRej = nRhs = 0;
          phase = PH_TRIAL;
        }
      }
    }
    if (__all_sync(FULL, phase == PH_DONE)) break;

    // ---- start (or restart) an ODE trial: odeSolverSolve + driver reset
    if (phase == PH_TRIAL) {
      if (t0 == t1) {
        b.step[node] = -1.0;  // node%timeStepSet(-1) when there is nothing to do
        b.status[node] = GAL_STATUS_SUCCESS;
        if (b.counters) {
          b.counters[node] = 0; b.counters[n + node] = 0; b.counters[2 * n + node] = 0;
        }
        phase = PH_NEED;
      } else {
        const double stepSize = G.p.reuse_step_size ? stepIn / (double)(1u << trial) : -1.0;
        h = t1 - t0;
        if (stepSize > 0.0) h = fmin(stepSize, h);
        if (trial > 0) {
#pragma unroll
          for (int v = 0; v < GAL_NY; ++v) y[v] = b.state[v * n + node];
        }
        t = t0;
        count = 0;
        rhs(G, sTab, sLnZ, sInvDlnZ, c, y, k1);  // dydt_in of the first step
        ++nRhs;
        phase = PH_STEP;
      }
    }

    // ---- one attempted step (one pass of gsl_odeiv2_evolve_apply's try_step)
    if (phase == PH_STEP) {
      const double dt = t1 - t;
      const bool finalStep = (dt >= 0.0 && h > dt) || (dt < 0.0 && h < dt);
      const double hh = finalStep ? dt : h;
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i) tmp[i] = y[i] + ck::b21 * hh * k1[i];
      rhs(G, sTab, sLnZ, sInvDlnZ, c, tmp, k2);
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i) tmp[i] = y[i] + hh * (ck::b31 * k1[i] + ck::b32 * k2[i]);
      rhs(G, sTab, sLnZ, sInvDlnZ, c, tmp, k3);
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i) tmp[i] = y[i] + hh * (ck::b41 * k1[i] + ck::b42 * k2[i] + ck::b43 * k3[i]);
      rhs(G, sTab, sLnZ, sInvDlnZ, c, tmp, k4);
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i)
        tmp[i] = y[i] + hh * (ck::b51 * k1[i] + ck::b52 * k2[i] + ck::b53 * k3[i] + ck::b54 * k4[i]);
      rhs(G, sTab, sLnZ, sInvDlnZ, c, tmp, k5);
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i)
        tmp[i] = y[i] + hh * (ck::b61 * k1[i] + ck::b62 * k2[i] + ck::b63 * k3[i] + ck::b64 * k4[i] + ck::b65 * k5[i]);
      rhs(G, sTab, sLnZ, sInvDlnZ, c, tmp, k6);
      nRhs += 5;
      // 5th-order solution into tmp, scaled error ratio (sc2_control_hadjust, a_y=1, a_dydt=0).
      // The largest |err_i|/D_i is found by cross-multiplication and divided
      // once (max of the quotients = quotient of the maximal pair).
      double errMax = 0.0, dMax = 1.0;
#pragma unroll
      for (int i = 0; i < GAL_NY; ++i) {
        tmp[i] = y[i] + hh * (ck::c1 * k1[i] + ck::c3 * k3[i] + ck::c4 * k4[i] + ck::c6 * k6[i]);
        const double err = fabs(hh * (ck::e1 * k1[i] + ck::e3 * k3[i] + ck::e4 * k4[i] + ck::e5 * k5[i] + ck::e6 * k6[i]));
        const double D0 = fabs(epsRel * fabs(tmp[i]) + epsAbs * s[i]);
        if (err * dMax > errMax * D0 || !(err == err)) {
          errMax = err;
          dMax = D0;
        }
      }
      const double rmax = fmax(errMax / dMax, 2.2250738585072014e-308);  // floor DBL_MIN as cscal2.c
      ++count;
      const double tNew = finalStep ? t1 : t + hh;
      double hNew = hh;
      bool decrease = false;
      if (rmax > 1.1) {
        double r = 0.9 / pow(rmax, 1.0 / ck::order);
        if (r < 0.2) r = 0.2;
        hNew = r * hh;
        decrease = true;
      } else if (rmax < 0.5) {
        double r = 0.9 / pow(rmax, 1.0 / (ck::order + 1.0));
        if (r > 4.9) r = 4.9;
        if (r < 1.0) r = 1.0;
        hNew = r * hh;
      }
      bool finished = false;
      int finalStatus = GAL_STATUS_SUCCESS;
      if (decrease) {
        const double tNext = tNew + hNew;
        if (fabs(hNew) < fabs(hh) && tNext != tNew) {
          h = hNew;  // reject: retry from the same (t, y) with the smaller step
          ++nRej;
          if (budget && count >= budget) { finished = true; finalStatus = GAL_STATUS_XCPU; }
        } else {
          // The step cannot shrink any further: this trial fails
          // (GSL_FAILURE); the node evolver restarts with half the step.
          ++trial;
          if (trial >= G.p.trial_count_maximum) { finished = true; finalStatus = GAL_STATUS_UNDERFLOW; }
          else phase = PH_TRIAL;
        }
      } else {
        // Accept.
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) y[i] = tmp[i];
        t = tNew;
        h = hNew;
        ++nAcc;
        const bool reached = !(t1 - t > 0.0 || t1 - t < 0.0);
        if (!reached) {
          rhs(G, sTab, sLnZ, sInvDlnZ, c, y, k1);  // dydt_out, reused as the next dydt_in
          ++nRhs;
        }
        post_step(y);  // clamps return GSL_Continue: dydt_out is kept
        if (reached) {
          finished = true;
          bool finite = true;
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) finite = finite && isfinite(y[i]);
          finalStatus = finite ? GAL_STATUS_SUCCESS : GAL_STATUS_NOT_FINITE;
        } else if (budget && count >= budget) {
          finished = true;
          finalStatus = GAL_STATUS_XCPU;
        }
      }
      if (finished) {
        if (finalStatus == GAL_STATUS_SUCCESS) {
#pragma unroll
          for (int v = 0; v < GAL_NY; ++v) b.state[v * n + node] = y[v];
          b.step[node] = h;
        }
        b.status[node] = finalStatus;
        if (b.counters) {
          b.counters[node] = nAcc;
          b.counters[n + node] = nRej;
          b.counters[2 * n + node] = nRhs;
        }
        phase = PH_NEED;
      }
    }
  }
}

}  // namespace gal

// ===========================================================================
// Host side: context, C ABI.
// ===========================================================================
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
  unsigned long long* dQueue = nullptr;  // work-queue head
  void* dBuf = nullptr;                  // staging for the host-pointer API
  size_t bufBytes = 0;
  int threads = 128;
  int blocksPerSm = 1;
  int64_t launches = 0;
  int lastError = 0;
  char message[512] = {0};
};

namespace {
thread_local int gLibError = 0;
thread_local char gLibMessage[512] = {0};

int fail(gal_ctx* ctx, int code, const char* fmt, const char* detail = "") {
  char buf[512];
  snprintf(buf, sizeof buf, fmt, detail);
  if (ctx) {
    ctx->lastError = code;
    snprintf(ctx->message, sizeof ctx->message, "%s", buf);
  } else {
    gLibError = code;
    snprintf(gLibMessage, sizeof gLibMessage, "%s", buf);
  }
  return code;
}

#define CUDA_TRY(ctx, call)                                                  \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return fail((ctx), GAL_ERR_CUDA, "CUDA error: %s", cudaGetErrorString(e_)); \
  } while (0)

double sound_speed_host(double T) {
  return std::sqrt(5.0 * k::boltzmannsConstant * T / 3.0 / k::meanAtomicMassPrimordial / k::atomicMassUnit) / k::kilo;
}

template <int THREADS>
cudaError_t launch_evolve(gal_ctx* ctx, const Batch& b, cudaStream_t st) {
  const size_t shm = shared_bytes(ctx->globals.nT, ctx->globals.nZ);
  cudaError_t e = cudaFuncSetAttribute(evolve_kernel<THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  int64_t warps = (b.n + 31) / 32;
  int64_t blocks = (int64_t)ctx->smCount * ctx->blocksPerSm;
  blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (warps * 32 + THREADS - 1) / THREADS));
  evolve_kernel<THREADS><<<(unsigned)blocks, THREADS, shm, st>>>(ctx->globals, b, ctx->dTab, ctx->dLnT, ctx->dLnZ);
  return cudaGetLastError();
}

cudaError_t dispatch(gal_ctx* ctx, const Batch& b, cudaStream_t st) {
  switch (ctx->threads) {
    case 64: return launch_evolve<64>(ctx, b, st);
    case 128: return launch_evolve<128>(ctx, b, st);
    case 256: return launch_evolve<256>(ctx, b, st);
    case 512: return launch_evolve<512>(ctx, b, st);
    default: return cudaErrorInvalidConfiguration;
  }
}
}  // namespace

extern "C" {

const char* gal_version(void) { return "galnode-gb300 0.1 (sm_103a)"; }

void gal_params_default(gal_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->ode_tolerance_absolute = 0.01;
  p->ode_tolerance_relative = 0.01;
  p->reuse_step_size = 1;
  p->trial_count_maximum = 8;
  p->step_budget = 1000000;
  p->physics = GAL_PHYS_ALL;
  p->omega_matter = 0.3;
  p->omega_baryon = 0.045;
  p->omega_dark_energy = 0.7;
  p->hubble_constant = 70.0;
  p->core_radius_fraction = 0.3;
  p->cooling_velocity_cutoff = 1.0e4;
  p->cooling_degrees_of_freedom = 3.0;
  p->reincorporation_multiplier = 5.0;
  p->radius_factor_disk = p->radius_factor_spheroid = std::sqrt(0.5);
  for (gal_star_formation* sf : {&p->sf_disk, &p->sf_spheroid}) {
    sf->timescale_type = GAL_SF_TIMESCALE_DYNAMICAL;
    sf->efficiency = 0.01;
    sf->exponent_velocity = -1.5;
    sf->timescale_minimum = 1.0e-3;
    sf->timescale_fixed = 1.0;
  }
  p->recycled_fraction = 0.46;
  p->metal_yield = 0.035;
  p->outflow_disk.type = p->outflow_spheroid.type = GAL_OUTFLOW_POWER_LAW;
  p->outflow_disk.velocity_characteristic = 250.0;
  p->outflow_spheroid.velocity_characteristic = 100.0;
  p->outflow_disk.exponent = p->outflow_spheroid.exponent = 3.5;
  p->outflow_disk.fraction = p->outflow_spheroid.fraction = 1.0;
  p->outflow_disk.timescale_fractional_minimum = p->outflow_spheroid.timescale_fractional_minimum = 1.0e-3;
  p->bh_enhancement_spheroid = 5.0;
  p->bh_enhancement_hot_halo = 6.0;
  p->bh_temperature_spheroid = 100.0;
  p->bh_hot_mode_only = 1;
  p->bh_efficiency_radiative = 1.0 - std::sqrt(8.0 / 9.0);
  p->bh_efficiency_jet = 0.0;
}

int gal_gpu_last_error(const gal_ctx* ctx, char* buf, int len) {
  const char* msg = ctx ? ctx->message : gLibMessage;
  int code = ctx ? ctx->lastError : gLibError;
  if (buf && len > 0) snprintf(buf, (size_t)len, "%s", msg);
  return code;
}

int gal_gpu_init(const gal_params* p, const gal_cie_table* t, gal_ctx** out) {
  if (!out) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_init: out is NULL%s");
  *out = nullptr;
  if (!p || !t) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_init: params and table are required%s");
  if (!(p->ode_tolerance_absolute > 0.0 || p->ode_tolerance_relative > 0.0) || p->ode_tolerance_absolute < 0.0 ||
      p->ode_tolerance_relative < 0.0)
    return fail(nullptr, GAL_ERR_ARGUMENT, "at least one of absolute and relative tolerance must be greater than zero%s");
  if (p->trial_count_maximum < 1 || p->trial_count_maximum > 30)
    return fail(nullptr, GAL_ERR_ARGUMENT, "trial_count_maximum must be in 1..30%s");
  const int nT = t->n_temperature, nZ = t->n_metallicity;
  if (nT < 2 || nZ < 2 || !t->temperature || !t->metallicity || !t->cooling_rate || !t->electron_density)
    return fail(nullptr, GAL_ERR_TABLE, "CIE table: at least 2x2 entries and all arrays are required%s");
  if (shared_bytes(nT, nZ) > 200 * 1024) return fail(nullptr, GAL_ERR_TABLE, "CIE table too large for shared memory%s");
  for (int i = 0; i < nT * nZ; ++i)
    if (!(t->cooling_rate[i] > 0.0) || !(t->electron_density[i] > 0.0))
      return fail(nullptr, GAL_ERR_TABLE, "CIE table: cooling rates and electron densities must be positive%s");
  for (int i = 1; i < nT; ++i)
    if (!(t->temperature[i] > t->temperature[i - 1])) return fail(nullptr, GAL_ERR_TABLE, "CIE table: temperatures must increase%s");
  for (int i = 1; i < nZ; ++i)
    if (!(t->metallicity[i] > t->metallicity[i - 1])) return fail(nullptr, GAL_ERR_TABLE, "CIE table: metallicities must increase%s");
  if (!(t->temperature[0] > 0.0) || t->metallicity[0] < 0.0) return fail(nullptr, GAL_ERR_TABLE, "CIE table: bad grid origin%s");

  int device = 0, count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) return fail(nullptr, GAL_ERR_NO_DEVICE, "no CUDA device%s");
  cudaGetDevice(&device);
  gal_ctx* ctx = new (std::nothrow) gal_ctx();
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "out of host memory%s");
  ctx->params = *p;
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, device);

  // Tables as the reference reads them (cieFileReadFile): logs of T, Z, values.
  Globals& g = ctx->globals;
  std::memset(&g, 0, sizeof g);
  g.p = *p;
  g.nT = nT;
  g.nZ = nZ;
  g.Tmin = t->temperature[0];
  g.Tmax = t->temperature[nT - 1];
  g.Zmin = t->metallicity[0];
  g.Zmax = t->metallicity[nZ - 1];
  g.firstZero = t->metallicity[0] == 0.0;
  g.firstNonZero = t->metallicity[1];
  const double cs = sound_speed_host(p->bh_temperature_spheroid);
  g.soundSpeedSpheroid = cs;
  g.jeansPrefactor = cs / std::sqrt(k::gravitationalConstantInternal);
  g.bhSpheroidCoef = p->bh_enhancement_spheroid * k::bhlPrefactor * k::gravitationalConstantInternal *
                     k::gravitationalConstantInternal / (cs * cs * cs);
  g.bhRadiusSpheroidCoef = k::gravitationalConstantInternal / (cs * cs);
  g.coolingCoef = p->cooling_degrees_of_freedom / 2.0 * k::boltzmannsConstant / k::ergs / k::gigaYear / k::densityToHydrogenNumber;
  g.accretionFraction = p->omega_baryon / p->omega_matter;

  std::vector<double2> tab((size_t)nZ * nT);
  std::vector<double> lnT(nT), lnZ(2 * nZ, 0.0);
  for (int i = 0; i < nT; ++i) lnT[i] = std::log(t->temperature[i]);
  for (int j = 0; j < nZ; ++j) lnZ[j] = t->metallicity[j] > 0.0 ? std::log(t->metallicity[j]) : -999.0;
  for (int j = 0; j + 1 < nZ; ++j) lnZ[nZ + j] = 1.0 / (lnZ[j + 1] - lnZ[j]);
  g.invFirstNonZero = 1.0 / g.firstNonZero;
  for (int i = 0; i < nZ * nT; ++i) tab[i] = make_double2(std::log(t->cooling_rate[i]), std::log(t->electron_density[i]));

  auto cleanup = [&](int code) {
    gal_gpu_free(ctx);
    return code;
  };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&ctx->dTab, tab.size() * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&ctx->dLnT, nT * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dLnZ, 2 * nZ * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dQueue, sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    fail(nullptr, GAL_ERR_CUDA, "device allocation failed%s");
    return cleanup(GAL_ERR_CUDA);
  }
  if (cudaMemcpy(ctx->dTab, tab.data(), tab.size() * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dLnT, lnT.data(), nT * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dLnZ, lnZ.data(), 2 * nZ * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    fail(nullptr, GAL_ERR_CUDA, "table upload failed%s");
    return cleanup(GAL_ERR_CUDA);
  }
  *out = ctx;
  return GAL_OK;
}

void gal_gpu_free(gal_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->dTab);
  cudaFree(ctx->dLnT);
  cudaFree(ctx->dLnZ);
  cudaFree(ctx->dQueue);
  cudaFree(ctx->dBuf);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int gal_gpu_set_launch(gal_ctx* ctx, int32_t threads, int32_t blocksPerSm) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_set_launch: NULL context%s");
  if (threads) {
    if (threads != 64 && threads != 128 && threads != 256 && threads != 512)
      return fail(ctx, GAL_ERR_ARGUMENT, "threads per block must be 64, 128, 256 or 512%s");
    ctx->threads = threads;
  }
  if (blocksPerSm) {
    const size_t shm = shared_bytes(ctx->globals.nT, ctx->globals.nZ);
    if (blocksPerSm < 1 || (size_t)blocksPerSm * shm > 228 * 1024)
      return fail(ctx, GAL_ERR_ARGUMENT, "blocks per SM out of range for the shared-memory footprint%s");
    ctx->blocksPerSm = blocksPerSm;
  }
  return GAL_OK;
}

int gal_gpu_get_launch(const gal_ctx* ctx, int32_t* threads, int32_t* blocksPerSm) {
  if (!ctx) return GAL_ERR_ARGUMENT;
  if (threads) *threads = ctx->threads;
  if (blocksPerSm) *blocksPerSm = ctx->blocksPerSm;
  return GAL_OK;
}

int64_t gal_gpu_launch_count(const gal_ctx* ctx) { return ctx ? ctx->launches : -1; }

int gal_gpu_evolve_batch_device(gal_ctx* ctx, int64_t n, double* state, const double* param, const double* tStart,
                                const double* tEnd, double* step, int32_t* status, uint32_t* counters, void* stream) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "NULL context%s");
  if (n < 0) return fail(ctx, GAL_ERR_ARGUMENT, "negative node count%s");
  if (n == 0) return GAL_OK;
  if (!state || !param || !tStart || !tEnd || !step || !status) return fail(ctx, GAL_ERR_ARGUMENT, "NULL array%s");
  if ((unsigned long long)n * GAL_NY > (1ull << 62)) return fail(ctx, GAL_ERR_TOO_LARGE, "batch too large%s");
  cudaStream_t st = (cudaStream_t)stream;  // used as given: NULL is the legacy default stream
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  CUDA_TRY(ctx, cudaMemsetAsync(ctx->dQueue, 0, sizeof(unsigned long long), st));
  Batch b{n, state, param, tStart, tEnd, step, status, counters, ctx->dQueue};
  CUDA_TRY(ctx, dispatch(ctx, b, st));
  ++ctx->launches;
  return GAL_OK;
}

int gal_gpu_evolve_batch(gal_ctx* ctx, int64_t n, double* state, const double* param, const double* tStart,
                         const double* tEnd, double* step, int32_t* status, uint32_t* counters) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "NULL context%s");
  if (n < 0) return fail(ctx, GAL_ERR_ARGUMENT, "negative node count%s");
  if (n == 0) return GAL_OK;
  if (!state || !param || !tStart || !tEnd || !step || !status) return fail(ctx, GAL_ERR_ARGUMENT, "NULL array%s");
  // One device buffer: state, param, t0, t1, step (FP64), status, counters.
  const size_t nd = (size_t)n * (GAL_NY + GAL_NP + 3);
  const size_t bytes = nd * sizeof(double) + (size_t)n * sizeof(int32_t) + (size_t)n * 3 * sizeof(uint32_t) + 256;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  if (bytes > ctx->bufBytes) {
    cudaFree(ctx->dBuf);
    ctx->dBuf = nullptr;
    ctx->bufBytes = 0;
    CUDA_TRY(ctx, cudaMalloc(&ctx->dBuf, bytes));
    ctx->bufBytes = bytes;
  }
  double* dState = (double*)ctx->dBuf;
  double* dParam = dState + (size_t)n * GAL_NY;
  double* dT0 = dParam + (size_t)n * GAL_NP;
  double* dT1 = dT0 + n;
  double* dStep = dT1 + n;
  int32_t* dStatus = (int32_t*)(dStep + n);
  uint32_t* dCounters = (uint32_t*)(dStatus + n);
  cudaStream_t st = ctx->stream;
  CUDA_TRY(ctx, cudaMemcpyAsync(dState, state, (size_t)n * GAL_NY * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dParam, param, (size_t)n * GAL_NP * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dT0, tStart, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dT1, tEnd, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dStep, step, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  int rc = gal_gpu_evolve_batch_device(ctx, n, dState, dParam, dT0, dT1, dStep, dStatus, counters ? dCounters : nullptr,
                                       (void*)st);
  if (rc) return rc;
  CUDA_TRY(ctx, cudaMemcpyAsync(state, dState, (size_t)n * GAL_NY * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(step, dStep, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(status, dStatus, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  if (counters)
    CUDA_TRY(ctx, cudaMemcpyAsync(counters, dCounters, (size_t)n * 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return GAL_OK;
}

}  // extern "C"

// ===========================================================================
// Evolution without any allocation.
//
// Some callers cannot let a library allocate device memory: a host code that
// hands all device memory to its own pool allocator up front (so a library
// cudaMalloc fails or fragments the pool), or a scheduler that must not take
// the device-wide synchronisation that cudaMalloc/cudaFree can impose while
// its other work is in flight.  gal_gpu_evolve_batch_noalloc serves them: the
// caller passes every input and output in device memory it already owns, and
// the one piece of scratch the kernel needs besides them -- the work-queue
// head plus the log-converted CIE tables staged for the shared-memory copy --
// lives in the file-scope array below, which every GPU that loads this
// library holds until the process exits.
// ===========================================================================
#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = 128 * 1024;  // queue head + tables; see the size check below
constexpr int kNoAllocThreads = 128;                  // launch shape of this entry point (one block per SM)
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

std::mutex g_noallocMutex;
void* g_noallocScratchPtr[kNoAllocMaxDevices] = {nullptr};

// Scratch layout: [0,256) queue head; then the double2 table [nZ*nT];
// then ln T [nT]; then ln Z [nZ] and 1/(ln Z[i+1]-ln Z[i]) [nZ].
size_t noalloc_bytes(int nT, int nZ) { return 256 + shared_bytes(nT, nZ); }

// In-place conversion of the staged raw table to the layout the kernel
// reads (the logarithms of cieFileReadFile, CIE_file.F90:535-663).
__global__ void noalloc_prepare_tables(double2* tab, double* lnT, double* lnZ, int nT, int nZ) {
  const int stride = blockDim.x * gridDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nZ * nT; i += stride) {
    double2 v = tab[i];
    tab[i] = make_double2(log(v.x), log(v.y));
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nT; i += stride) lnT[i] = log(lnT[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int j = 0; j < nZ; ++j) lnZ[j] = lnZ[j] > 0.0 ? log(lnZ[j]) : -999.0;
    for (int j = 0; j + 1 < nZ; ++j) lnZ[nZ + j] = 1.0 / (lnZ[j + 1] - lnZ[j]);
    lnZ[2 * nZ - 1] = 0.0;
  }
}

}  // namespace

extern "C" int gal_gpu_evolve_batch_noalloc(const gal_params* p, const gal_cie_table* t, int64_t n, double* state,
                                            const double* param, const double* tStart, const double* tEnd, double* step,
                                            int32_t* status, uint32_t* counters, void* stream) {
  if (!p || !t) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_evolve_batch_noalloc: params and table are required%s");
  if (n < 0) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_evolve_batch_noalloc: negative node count%s");
  if (n == 0) return GAL_OK;
  if (!state || !param || !tStart || !tEnd || !step || !status)
    return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_evolve_batch_noalloc: NULL array%s");
  if (!(p->ode_tolerance_absolute > 0.0 || p->ode_tolerance_relative > 0.0) || p->ode_tolerance_absolute < 0.0 ||
      p->ode_tolerance_relative < 0.0 || p->trial_count_maximum < 1 || p->trial_count_maximum > 30)
    return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_evolve_batch_noalloc: invalid tolerances or trial count%s");
  const int nT = t->n_temperature, nZ = t->n_metallicity;
  if (nT < 2 || nZ < 2 || !t->temperature || !t->metallicity || !t->cooling_rate || !t->electron_density)
    return fail(nullptr, GAL_ERR_TABLE, "gal_gpu_evolve_batch_noalloc: CIE table needs at least 2x2 entries%s");
  if (noalloc_bytes(nT, nZ) > kNoAllocScratchBytes)
    return fail(nullptr, GAL_ERR_TOO_LARGE,
                "gal_gpu_evolve_batch_noalloc: CIE table too large for the fixed 128 KiB scratch "
                "(16 (n_metallicity*n_temperature) + 8 (n_temperature + 2 n_metallicity) + 256 bytes must not exceed 131072)%s");
  for (int i = 0; i < nT * nZ; ++i)
    if (!(t->cooling_rate[i] > 0.0) || !(t->electron_density[i] > 0.0))
      return fail(nullptr, GAL_ERR_TABLE, "gal_gpu_evolve_batch_noalloc: table values must be positive%s");
  for (int i = 1; i < nT; ++i)
    if (!(t->temperature[i] > t->temperature[i - 1])) return fail(nullptr, GAL_ERR_TABLE, "CIE table: temperatures must increase%s");
  for (int i = 1; i < nZ; ++i)
    if (!(t->metallicity[i] > t->metallicity[i - 1])) return fail(nullptr, GAL_ERR_TABLE, "CIE table: metallicities must increase%s");
  if (!(t->temperature[0] > 0.0) || t->metallicity[0] < 0.0) return fail(nullptr, GAL_ERR_TABLE, "CIE table: bad grid origin%s");

  // Once per device, with that device current: the device address of the
  // scratch array (its name is only a host-side stand-in in host code).
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kNoAllocMaxDevices)
    return fail(nullptr, GAL_ERR_NO_DEVICE, "gal_gpu_evolve_batch_noalloc: no usable current device%s");
  unsigned char* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocScratchPtr[device]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noallocScratch);
      if (e != cudaSuccess || !ptr)
        return fail(nullptr, GAL_ERR_CUDA, "gal_gpu_evolve_batch_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      g_noallocScratchPtr[device] = ptr;
    }
    scratch = (unsigned char*)g_noallocScratchPtr[device];
  }
  unsigned long long* queue = (unsigned long long*)scratch;
  double2* tab = (double2*)(scratch + 256);
  double* lnT = (double*)(tab + (size_t)nZ * nT);
  double* lnZ = lnT + nT;

  Globals g;
  std::memset(&g, 0, sizeof g);
  g.p = *p;
  g.nT = nT;
  g.nZ = nZ;
  g.Tmin = t->temperature[0];
  g.Tmax = t->temperature[nT - 1];
  g.Zmin = t->metallicity[0];
  g.Zmax = t->metallicity[nZ - 1];
  g.firstZero = t->metallicity[0] == 0.0;
  g.firstNonZero = t->metallicity[1];
  g.invFirstNonZero = 1.0 / g.firstNonZero;
  const double cs = sound_speed_host(p->bh_temperature_spheroid);
  g.soundSpeedSpheroid = cs;
  g.jeansPrefactor = cs / std::sqrt(k::gravitationalConstantInternal);
  g.bhSpheroidCoef = p->bh_enhancement_spheroid * k::bhlPrefactor * k::gravitationalConstantInternal *
                     k::gravitationalConstantInternal / (cs * cs * cs);
  g.bhRadiusSpheroidCoef = k::gravitationalConstantInternal / (cs * cs);
  g.coolingCoef = p->cooling_degrees_of_freedom / 2.0 * k::boltzmannsConstant / k::ergs / k::gigaYear / k::densityToHydrogenNumber;
  g.accretionFraction = p->omega_baryon / p->omega_matter;

  cudaStream_t st = (cudaStream_t)stream;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1)
    return fail(nullptr, GAL_ERR_CUDA, "gal_gpu_evolve_batch_noalloc: cannot query the SM count%s");
  cudaError_t e = cudaSuccess;
  // Stage the raw table: cooling rates into .x, electron densities into .y.
  const size_t cells = (size_t)nZ * nT;
  if (e == cudaSuccess) e = cudaMemcpy2DAsync(&tab[0].x, sizeof(double2), t->cooling_rate, sizeof(double), sizeof(double), cells,
                                              cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpy2DAsync(&tab[0].y, sizeof(double2), t->electron_density, sizeof(double), sizeof(double),
                                              cells, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lnT, t->temperature, nT * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lnZ, t->metallicity, nZ * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    noalloc_prepare_tables<<<32, 256, 0, st>>>(tab, lnT, lnZ, nT, nZ);
    e = cudaGetLastError();
  }
  // The queue head must start at zero: the array keeps the last call's contents.
  if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
  const size_t shm = shared_bytes(nT, nZ);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(evolve_kernel<kNoAllocThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e == cudaSuccess) {
    Batch b{n, state, param, tStart, tEnd, step, status, counters, queue};
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(sms, (n + kNoAllocThreads - 1) / kNoAllocThreads));
    evolve_kernel<kNoAllocThreads><<<(unsigned)blocks, kNoAllocThreads, shm, st>>>(g, b, tab, lnT, lnZ);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail(nullptr, GAL_ERR_CUDA, "gal_gpu_evolve_batch_noalloc: CUDA error: %s", cudaGetErrorString(e));
  return GAL_OK;
}
