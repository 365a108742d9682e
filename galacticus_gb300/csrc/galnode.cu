// galnode.cu -- batched node evolution on GB300 (sm_103a): context, C ABI.
//
// Hot path: gal_gpu_evolve_batch[_device] -> evolve_kernel (evolve_kernel.cuh,
// instantiated per form in evolve_*.cu).  This file owns the context: the
// tables uploaded once per context, the launch shape, the optional
// cooling-function surrogate and the rate precision, and the entry points of
// include/galnode.h and include/galnode_surrogate.h.

#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <new>
#include <vector>
#include <algorithm>

#include "../../include/galnode.h"
#include "../../include/galnode_surrogate.h"
#include "evolve_kernel.cuh"
#include "context.h"

namespace gal {

// The short-log/exp tables, computed once on the host from the C library.
struct HostFastTables {
  double2 log[kLogTableSize];
  double exp2[kExpTableSize];
  HostFastTables() { fast_tables_host(log, exp2); }
};
const HostFastTables& host_fast_tables() {
  static const HostFastTables tables;  // thread-safe one-time initialisation
  return tables;
}
const double2* host_fast_log_table() { return host_fast_tables().log; }
const double* host_fast_exp_table() { return host_fast_tables().exp2; }

}  // namespace gal

// ===========================================================================
// Host side: context, C ABI.
// ===========================================================================
using namespace gal;

namespace {
thread_local int gLibError = 0;
thread_local char gLibMessage[512] = {0};

}  // namespace

namespace gal {
namespace host {

int fail(gal_ctx* ctx, int code, const char* fmt, const char* detail) {
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

}  // namespace host
}  // namespace gal
using namespace gal::host;

namespace {

#define CUDA_TRY(ctx, call)                                                  \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return fail((ctx), GAL_ERR_CUDA, "CUDA error: %s", cudaGetErrorString(e_)); \
  } while (0)

double sound_speed_host(double T) {
  return std::sqrt(5.0 * k::boltzmannsConstant * T / 3.0 / k::meanAtomicMassPrimordial / k::atomicMassUnit) / k::kilo;
}

// Record whether the non-zero metallicity rows are evenly spaced in ln Z
// (the Cloudy grid is), so the kernel can find the cell arithmetically.
void set_uniform_metallicity_grid(Globals& g, const double* lnZ, int nZ) {
  const int first = g.firstZero ? 1 : 0;
  g.zFirstLog = first;
  g.lnZFirst = lnZ[first];
  g.zUniform = 0;
  if (nZ - first < 2) return;
  const double d = (lnZ[nZ - 1] - lnZ[first]) / (nZ - 1 - first);
  for (int j = first; j + 1 < nZ; ++j)
    if (std::fabs(lnZ[j + 1] - lnZ[j] - d) > 1.0e-9 * std::fabs(d)) return;
  g.invDlnZ = 1.0 / d;
  g.zUniform = 1;
}

// The same for the temperature rows (the Cloudy grid is evenly spaced in
// log T), for the FP32 node setup of the FP32-rate forms.
void set_uniform_temperature_grid(Globals& g, const double* lnT, int nT) {
  g.tUniform = 0;
  const double d = (lnT[nT - 1] - lnT[0]) / (nT - 1);
  for (int i = 0; i + 1 < nT; ++i)
    if (std::fabs(lnT[i + 1] - lnT[i] - d) > 1.0e-9 * std::fabs(d)) return;
  g.f.lnTFirst = (float)lnT[0];
  g.f.invDlnT = (float)(1.0 / d);
  g.tUniform = 1;
}

}  // namespace

namespace gal {
namespace host {

int ctx_mode(const gal_ctx* ctx) {
  return (ctx->ratePrecision == GAL_RATES_FP32 ? MODE_FAST : 0) | (ctx->dSurrSmall ? MODE_SURROGATE : 0);
}

size_t ctx_shared_bytes(const gal_ctx* ctx, int mode) {
  return evolve_shared_bytes(mode, ctx->globals.nT, ctx->globals.nZ,
                             surrogate_map_bytes(ctx->surrInfo.mapT, ctx->surrInfo.mapZ));
}

// Block sizes each form is built for (evolve_*.cu).
bool mode_has_threads(int mode, int threads) {
  switch (mode) {
    case MODE_PLAIN: return threads == 64 || threads == 128 || threads == 256 || threads == 512;
    case MODE_FAST: return threads == 128 || threads == 256 || threads == 512;
    default: return threads == 128 || threads == 256;
  }
}

DeviceTables ctx_tables(const gal_ctx* ctx) {
  return DeviceTables{ctx->dTab,     ctx->dLnT,     ctx->dLnZ,  ctx->dFastLog,
                      ctx->dFastExp, ctx->dTabF,    ctx->dLnZF,
                      KmtTables<double>{ctx->dKmt, ctx->dKmt + kmt::kFractionCount},
                      KmtTables<float>{ctx->dKmtF, ctx->dKmtF + kmt::kFractionCount}};
}

// The launch shape in use for a form: the requested one, moved to the
// nearest size the form is built for and to the blocks per SM that fit.
void effective_shape(const gal_ctx* ctx, int mode, int& threads, int& blocksPerSm) {
  threads = ctx->threads;
  if (!mode_has_threads(mode, threads)) threads = threads < 128 ? 128 : 256;
  if (ctx->params.sf_disk_rate == GAL_SF_RATE_KRUMHOLZ2009) threads = 128;  // its one instantiation
  const size_t shm = ctx_shared_bytes(ctx, mode);
  blocksPerSm = ctx->blocksPerSm;
  while (blocksPerSm > 1 && (size_t)blocksPerSm * shm > 228 * 1024) --blocksPerSm;
}

}  // namespace host
}  // namespace gal

namespace {

// Work estimate of a node for the order in which the table kernel of the
// split launch takes its nodes: the number of dynamical times in its
// interval times the disk's outflow mass loading (V_out/V_vir)^alpha_out.
// On the 65,536-halo isolated batch it tracks the right-hand-side count
// (mean 7, 15, 29 and 55 evaluations for estimates below 1, 1-10, 10-100
// and above 100; the batch's hardest halo, 1,061 evaluations, ranks 49th),
// and nodes at or above kFrontWork (about a fifth of that batch) are
// queued first, so that the long integrations start in the first wave of a
// kernel that shares the GPU with the network kernel.  It only orders the
// queue: a node's result does not depend on it.
constexpr float kFrontWork = 10.0f;

__device__ __forceinline__ float work_estimate(const Globals& G, const double* param, const double* tStart,
                                               const double* tEnd, int64_t n, int64_t i) {
  const float v = (float)param[GAL_P_VELOCITY_VIRIAL * n + i], r = (float)param[GAL_P_RADIUS_VIRIAL * n + i];
  const float dt = (float)(tEnd[i] - tStart[i]);
  const float tdyn = r / v * (float)k::MpcPerKmPerSToGyr;
  const float loading = G.p.outflow_disk.type == GAL_OUTFLOW_POWER_LAW
                            ? __powf((float)G.p.outflow_disk.velocity_characteristic / v, (float)G.p.outflow_disk.exponent)
                            : 1.0f;
  const float w = fabsf(dt) / tdyn * loading;
  return w == w ? w : 0.0f;
}

// The surrogate forms' split launch, step 1: sort the batch into the nodes
// the network may serve at their starting state (surrogate_open: a T row
// with network cells, hot gas, a metallicity in a cell the error map leaves
// to the network) and the others.  Lists in order of arrival (warp-
// aggregated atomics); in the table list the nodes with a work estimate at
// or above kFrontWork go to its front, the others fill it from its far end
// down.  A node's result does not depend on its place.
template <bool FAST>
__global__ void surrogate_classify(const __grid_constant__ Globals G, const __grid_constant__ SurrogateInfo I,
                                   const uint8_t* map, const double* param, const double* state, const double* tStart,
                                   const double* tEnd, int64_t n, int64_t cap, int32_t* orderTable, int32_t* orderNet,
                                   unsigned long long* counts) {
  const int lane = threadIdx.x & 31;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = i0 + threadIdx.x;
    bool open = false;
    if (i < n) {
      // The node's temperature as the kernel's node set-up forms it.
      const double vvir = param[GAL_P_VELOCITY_VIRIAL * n + i];
      float log10T;
      if (FAST) {
        const float v = (float)vvir, T = G.f.tempPerV2 * v * v;
        log10T = T > 0.0f ? log10f(T) : -1.0e30f;
      } else {
        const double T = 0.5 * k::atomicMassUnit * k::meanAtomicMassPrimordial * (k::kilo * vvir) * (k::kilo * vvir) /
                         k::boltzmannsConstant;
        log10T = T > 0.0 ? (float)log10(T) : -1.0e30f;
      }
      struct { int netRow; } c{surrogate_net_row(I, map, log10T, !(vvir > G.p.cooling_velocity_cutoff))};
      const double y[2] = {state[GAL_Y_HOT_MASS * n + i], state[GAL_Y_HOT_METALS * n + i]};
      open = surrogate_open(I, map, c, y);
    }
    const bool front = i < n && !open && work_estimate(G, param, tStart, tEnd, n, i) >= kFrontWork;
    const unsigned active = __ballot_sync(FULL, i < n);
    const unsigned net = __ballot_sync(FULL, open);
    const unsigned tabFront = __ballot_sync(FULL, front);
    const unsigned tabBack = active & ~net & ~tabFront;
    unsigned long long baseNet = 0, baseFront = 0, baseBack = 0;
    if (lane == 0) {
      if (net) baseNet = atomicAdd(&counts[1], (unsigned long long)__popc(net));
      if (tabFront) baseFront = atomicAdd(&counts[0], (unsigned long long)__popc(tabFront));
      if (tabBack) baseBack = atomicAdd(&counts[4], (unsigned long long)__popc(tabBack));
    }
    baseNet = __shfl_sync(FULL, baseNet, 0);
    baseFront = __shfl_sync(FULL, baseFront, 0);
    baseBack = __shfl_sync(FULL, baseBack, 0);
    const unsigned below = (1u << lane) - 1u;
    if (i < n) {
      if (open) orderNet[baseNet + __popc(net & below)] = (int32_t)i;
      else if (front) orderTable[baseFront + __popc(tabFront & below)] = (int32_t)i;
      else orderTable[cap - 1 - (int64_t)(baseBack + __popc(tabBack & below))] = (int32_t)i;
    }
  }
}

cudaError_t dispatch(gal_ctx* ctx, const Batch& b, cudaStream_t st) {
  const int mode = ctx_mode(ctx);
  if ((mode & MODE_SURROGATE) && ctx->splitSurrogate && b.n <= (int64_t)INT32_MAX) {
    // The split launch: the nodes the network may serve go to the surrogate
    // kernel, the others to the kernel of the same rates without it, the two
    // running at once on two streams.  The form without the network keeps
    // its own registers and code: in one kernel with the network path it ran
    // ~20% slower.
    if (b.n > ctx->orderCap) {
      cudaFree(ctx->dOrder);
      ctx->dOrder = nullptr;
      ctx->orderCap = 0;
      cudaError_t e = cudaMalloc(&ctx->dOrder, 2 * (size_t)b.n * sizeof(int32_t));
      if (e != cudaSuccess) return e;
      ctx->orderCap = b.n;
    }
    int32_t* orderTable = ctx->dOrder;
    int32_t* orderNet = ctx->dOrder + ctx->orderCap;
    // [0] table list (front), [1] network list, [2], [3] queue heads, [4] table list (back)
    unsigned long long* counts = ctx->dOrderCount;
    cudaError_t e = cudaMemsetAsync(counts, 0, 5 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const int cb = (int)std::min<int64_t>((b.n + 255) / 256, (int64_t)ctx->smCount * 8);
    if (mode & MODE_FAST)
      surrogate_classify<true><<<cb, 256, 0, st>>>(ctx->globals, ctx->surrInfo, ctx->dSurrMap, b.param, b.state,
                                                   b.tStart, b.tEnd, b.n, ctx->orderCap, orderTable, orderNet, counts);
    else
      surrogate_classify<false><<<cb, 256, 0, st>>>(ctx->globals, ctx->surrInfo, ctx->dSurrMap, b.param, b.state,
                                                    b.tStart, b.tEnd, b.n, ctx->orderCap, orderTable, orderNet, counts);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ctx->evFork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(ctx->stream2, ctx->evFork, 0)) != cudaSuccess) return e;
    int threads, blocksPerSm;
    effective_shape(ctx, mode, threads, blocksPerSm);
    const int tableMode = mode & ~MODE_SURROGATE;
    const int64_t blocksNet = std::max<int64_t>(1, std::min<int64_t>(ctx->smCount, (b.n + threads - 1) / threads));
    LaunchArgs a{};
    a.G = ctx->globals;
    a.tables = ctx_tables(ctx);
    a.b = b;
    a.b.order = orderNet;
    a.b.orderCount = counts + 1;
    a.b.queue = counts + 3;
    a.sd = SurrogateDev{ctx->dSurrSmall, ctx->dSurrPlanes, ctx->dSurrMap, ctx->surrInfo, ctx->dSurrStats};
    a.shm = ctx_shared_bytes(ctx, mode);
    a.blocks = blocksNet;
    a.stream = ctx->stream2;
    if ((e = evolve_launch(mode, threads, a)) != cudaSuccess) return e;
    const int tableThreads = mode_has_threads(tableMode, threads) ? threads : 128;
    LaunchArgs t = a;
    t.b.order = orderTable;
    t.b.orderCount = counts;
    t.b.orderBackCount = counts + 4;
    t.b.orderCap = ctx->orderCap;
    t.b.queue = counts + 2;
    t.sd = SurrogateDev{};
    t.sd.stats = ctx->dSurrStats;  // the table evaluations of these nodes
    t.shm = ctx_shared_bytes(ctx, tableMode);
    // The table kernel takes most of the nodes, the hardest among them: it
    // gets the context's blocks per SM, as the form alone does (a block
    // that does not fit beside the network kernel's starts when that one's
    // few nodes are done).
    int tableBlocksPerSm = blocksPerSm;
    while (tableBlocksPerSm > 1 && (size_t)tableBlocksPerSm * t.shm > 228 * 1024) --tableBlocksPerSm;
    t.blocks = std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->smCount * tableBlocksPerSm,
                                                      (b.n + tableThreads - 1) / tableThreads));
    t.stream = st;
    if ((e = evolve_launch(tableMode, tableThreads, t)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ctx->evJoin, ctx->stream2)) != cudaSuccess) return e;
    ctx->launches += 2;  // the classification and the second kernel (the caller counts one)
    return cudaStreamWaitEvent(st, ctx->evJoin, 0);
  }
  int threads, blocksPerSm;
  effective_shape(ctx, mode, threads, blocksPerSm);
  LaunchArgs a{};
  a.G = ctx->globals;
  a.b = b;
  a.tables = ctx_tables(ctx);
  if (mode & MODE_SURROGATE) a.sd = SurrogateDev{ctx->dSurrSmall, ctx->dSurrPlanes, ctx->dSurrMap, ctx->surrInfo, ctx->dSurrStats};
  a.shm = ctx_shared_bytes(ctx, mode);
  const int64_t warps = (b.n + 31) / 32;
  a.blocks = std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->smCount * blocksPerSm, (warps * 32 + threads - 1) / threads));
  a.stream = st;
  return evolve_launch(mode, threads, a);
}

void free_surrogate(gal_ctx* ctx) {
  cudaFree(ctx->dSurrSmall);
  cudaFree(ctx->dSurrPlanes);
  cudaFree(ctx->dSurrMap);
  cudaFree(ctx->dSurrStats);
  ctx->dSurrSmall = nullptr;
  ctx->dSurrPlanes = nullptr;
  ctx->dSurrMap = nullptr;
  ctx->dSurrStats = nullptr;
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
  p->timestep_relative = 0.1;
  p->timestep_absolute = 1.0;
  p->sf_disk_rate = GAL_SF_RATE_TIMESCALE;
  p->krumholz_fast = 0;
  p->krumholz_frequency = 0.385;
  p->krumholz_clumping = 5.0;
  p->merger_mass_ratio_major = 0.25;
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
  if (!(p->timestep_absolute > 0.0) || !(p->timestep_relative == p->timestep_relative))
    return fail(nullptr, GAL_ERR_ARGUMENT, "timestep_absolute must be positive%s");
  if (p->sf_disk_rate != GAL_SF_RATE_TIMESCALE && p->sf_disk_rate != GAL_SF_RATE_KRUMHOLZ2009)
    return fail(nullptr, GAL_ERR_ARGUMENT, "sf_disk_rate must be GAL_SF_RATE_TIMESCALE or GAL_SF_RATE_KRUMHOLZ2009%s");
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
  set_uniform_metallicity_grid(g, lnZ.data(), nZ);
  fill_fast_constants(g);
  set_uniform_temperature_grid(g, lnT.data(), nT);
  for (int i = 0; i < nZ * nT; ++i) tab[i] = make_double2(std::log(t->cooling_rate[i]), std::log(t->electron_density[i]));
  std::vector<float2> tabF(tab.size());
  std::vector<float> lnZF(2 * nZ);
  for (size_t i = 0; i < tab.size(); ++i) tabF[i] = make_float2((float)tab[i].x, (float)tab[i].y);
  for (int j = 0; j < 2 * nZ; ++j) lnZF[j] = (float)lnZ[j];

  // The Krumholz (2009) tables of the reference: the molecular fraction on
  // 1000 points of s in [0, 10] (Krumholz2009.F90:222-230) and x^0.33 on
  // [1, 1000] at 100 points per unit (math/exponentiation.F90).
  std::vector<double> kmtTab(kmt::kFractionCount + kmt::kPowerCount);
  for (int i = 0; i < kmt::kFractionCount; ++i)
    kmtTab[i] = kmt_fraction_formula<double>(kmt::kFractionMaximum * i / (kmt::kFractionCount - 1), p->krumholz_fast != 0);
  for (int i = 0; i < kmt::kPowerCount; ++i)
    kmtTab[kmt::kFractionCount + i] =
        std::pow(kmt::kPowerMinimum + (kmt::kPowerMaximum - kmt::kPowerMinimum) * i / (kmt::kPowerCount - 1), 0.33);
  std::vector<float> kmtTabF(kmtTab.begin(), kmtTab.end());
  auto cleanup = [&](int code) {
    gal_gpu_free(ctx);
    return code;
  };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&ctx->dTab, tab.size() * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&ctx->dLnT, nT * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dLnZ, 2 * nZ * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dFastLog, kLogTableSize * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&ctx->dFastExp, kExpTableSize * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dTabF, tab.size() * sizeof(float2)) != cudaSuccess ||
      cudaMalloc(&ctx->dLnZF, 2 * nZ * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&ctx->dKmt, (kmt::kFractionCount + kmt::kPowerCount) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ctx->dKmtF, (kmt::kFractionCount + kmt::kPowerCount) * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&ctx->dQueue, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&ctx->dOrderCount, 5 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->evFork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->evJoin, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    fail(nullptr, GAL_ERR_CUDA, "device allocation failed%s");
    return cleanup(GAL_ERR_CUDA);
  }
  if (cudaMemcpy(ctx->dTab, tab.data(), tab.size() * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dLnT, lnT.data(), nT * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dLnZ, lnZ.data(), 2 * nZ * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dFastLog, host_fast_log_table(), kLogTableSize * sizeof(double2), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dFastExp, host_fast_exp_table(), kExpTableSize * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dTabF, tabF.data(), tabF.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dLnZF, lnZF.data(), 2 * nZ * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dKmt, kmtTab.data(), kmtTab.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dKmtF, kmtTabF.data(), kmtTabF.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
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
  cudaFree(ctx->dFastLog);
  cudaFree(ctx->dFastExp);
  cudaFree(ctx->dTabF);
  cudaFree(ctx->dLnZF);
  cudaFree(ctx->dKmt);
  cudaFree(ctx->dKmtF);
  cudaFree(ctx->dQueue);
  cudaFree(ctx->dOrder);
  cudaFree(ctx->dOrderCount);
  if (ctx->stream2) {
    cudaStreamSynchronize(ctx->stream2);
    cudaStreamDestroy(ctx->stream2);
  }
  if (ctx->evFork) cudaEventDestroy(ctx->evFork);
  if (ctx->evJoin) cudaEventDestroy(ctx->evJoin);
  cudaFree(ctx->dBuf);
  free_surrogate(ctx);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int gal_gpu_set_launch(gal_ctx* ctx, int32_t threads, int32_t blocksPerSm) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_set_launch: NULL context%s");
  const int mode = ctx_mode(ctx);
  if (threads) {
    if (threads != 64 && threads != 128 && threads != 256 && threads != 512)
      return fail(ctx, GAL_ERR_ARGUMENT, "threads per block must be 64, 128, 256 or 512%s");
    if (!mode_has_threads(mode, threads))
      return fail(ctx, GAL_ERR_ARGUMENT, "this block size is not built for the current form (rate precision / surrogate)%s");
    ctx->threads = threads;
  }
  if (blocksPerSm) {
    if (blocksPerSm < 1 || (size_t)blocksPerSm * ctx_shared_bytes(ctx, mode) > 228 * 1024)
      return fail(ctx, GAL_ERR_ARGUMENT, "blocks per SM out of range for the shared-memory footprint%s");
    ctx->blocksPerSm = blocksPerSm;
  }
  return GAL_OK;
}

int gal_gpu_get_launch(const gal_ctx* ctx, int32_t* threads, int32_t* blocksPerSm) {
  if (!ctx) return GAL_ERR_ARGUMENT;
  int t, bps;
  effective_shape(ctx, ctx_mode(ctx), t, bps);
  if (threads) *threads = t;
  if (blocksPerSm) *blocksPerSm = bps;
  return GAL_OK;
}

int gal_gpu_set_rate_precision(gal_ctx* ctx, int32_t precision) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_set_rate_precision: NULL context%s");
  if (precision != GAL_RATES_FP64 && precision != GAL_RATES_FP32)
    return fail(ctx, GAL_ERR_ARGUMENT, "rate precision must be GAL_RATES_FP64 or GAL_RATES_FP32%s");
  ctx->ratePrecision = precision;
  return GAL_OK;
}

int gal_gpu_get_rate_precision(const gal_ctx* ctx) { return ctx ? ctx->ratePrecision : -1; }

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

int gal_gpu_evolve_batch_interrupt_device(gal_ctx* ctx, int64_t n, double* state, const double* param,
                                          const double* tStart, const double* tEnd, double* step,
                                          const int32_t* components, int32_t* status, uint32_t* counters,
                                          double* tReached, int32_t* task, void* stream) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "NULL context%s");
  if (n < 0) return fail(ctx, GAL_ERR_ARGUMENT, "negative node count%s");
  if (n == 0) return GAL_OK;
  if (!state || !param || !tStart || !tEnd || !step || !components || !status || !tReached || !task)
    return fail(ctx, GAL_ERR_ARGUMENT, "NULL array%s");
  if ((unsigned long long)n * GAL_NY > (1ull << 62)) return fail(ctx, GAL_ERR_TOO_LARGE, "batch too large%s");
  if (ctx_mode(ctx) != MODE_PLAIN || ctx->params.sf_disk_rate != GAL_SF_RATE_TIMESCALE)
    return fail(ctx, GAL_ERR_ARGUMENT,
                "interrupts are available in the FP64-rate form without a surrogate, with the timescale disk rate%s");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  CUDA_TRY(ctx, cudaMemsetAsync(ctx->dQueue, 0, sizeof(unsigned long long), st));
  int threads, blocksPerSm;
  effective_shape(ctx, MODE_PLAIN, threads, blocksPerSm);
  LaunchArgs a{};
  a.G = ctx->globals;
  a.b = Batch{n, state, param, tStart, tEnd, step, status, counters, ctx->dQueue, components, tReached, task};
  a.tables = ctx_tables(ctx);
  a.shm = ctx_shared_bytes(ctx, MODE_PLAIN);
  const int64_t warps = (n + 31) / 32;
  a.blocks = std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->smCount * blocksPerSm, (warps * 32 + 127) / 128));
  a.stream = st;
  CUDA_TRY(ctx, evolve_launch_plain_interrupt(a));
  ++ctx->launches;
  return GAL_OK;
}

int gal_gpu_evolve_batch_interrupt(gal_ctx* ctx, int64_t n, double* state, const double* param, const double* tStart,
                                   const double* tEnd, double* step, const int32_t* components, int32_t* status,
                                   uint32_t* counters, double* tReached, int32_t* task) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "NULL context%s");
  if (n < 0) return fail(ctx, GAL_ERR_ARGUMENT, "negative node count%s");
  if (n == 0) return GAL_OK;
  if (!state || !param || !tStart || !tEnd || !step || !components || !status || !tReached || !task)
    return fail(ctx, GAL_ERR_ARGUMENT, "NULL array%s");
  if (ctx_mode(ctx) != MODE_PLAIN)
    return fail(ctx, GAL_ERR_ARGUMENT, "interrupts are available in the FP64-rate form without a surrogate%s");
  // One device buffer: state, param, t0, t1, step, t_reached (FP64), then
  // components, status, task, counters.
  const size_t nd = (size_t)n * (GAL_NY + GAL_NP + 4);
  const size_t bytes = nd * sizeof(double) + (size_t)n * 3 * sizeof(int32_t) + (size_t)n * 3 * sizeof(uint32_t) + 256;
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
  double* dReached = dStep + n;
  int32_t* dComponents = (int32_t*)(dReached + n);
  int32_t* dStatus = dComponents + n;
  int32_t* dTask = dStatus + n;
  uint32_t* dCounters = (uint32_t*)(dTask + n);
  cudaStream_t st = ctx->stream;
  CUDA_TRY(ctx, cudaMemcpyAsync(dState, state, (size_t)n * GAL_NY * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dParam, param, (size_t)n * GAL_NP * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dT0, tStart, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dT1, tEnd, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dStep, step, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(dComponents, components, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  int rc = gal_gpu_evolve_batch_interrupt_device(ctx, n, dState, dParam, dT0, dT1, dStep, dComponents, dStatus,
                                                 counters ? dCounters : nullptr, dReached, dTask, (void*)st);
  if (rc) return rc;
  CUDA_TRY(ctx, cudaMemcpyAsync(state, dState, (size_t)n * GAL_NY * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(step, dStep, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(status, dStatus, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(tReached, dReached, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaMemcpyAsync(task, dTask, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  if (counters)
    CUDA_TRY(ctx, cudaMemcpyAsync(counters, dCounters, (size_t)n * 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(ctx, cudaStreamSynchronize(st));
  return GAL_OK;
}

int gal_gpu_set_surrogate(gal_ctx* ctx, const gal_surrogate* sg) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_set_surrogate: NULL context%s");
  CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  free_surrogate(ctx);
  if (!sg) return GAL_OK;
  if (ctx->params.sf_disk_rate != GAL_SF_RATE_TIMESCALE)
    return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_set_surrogate: the surrogate forms use the timescale disk star-formation rate%s");
  if (!sg->params || !sg->use_table || sg->map_t < 1 || sg->map_z < 1 || sg->map_t * sg->map_z > 4096 ||
      !(sg->map_dt > 0.0f) || !(sg->map_dz > 0.0f) || !(sg->y_scale > 0.0f))
    return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_set_surrogate: incomplete surrogate description%s");
  for (int i = 0; i < 3; ++i)
    if (!(sg->in_scale[i] > 0.0f) || !(sg->hi[i] > sg->lo[i]))
      return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_set_surrogate: bad normalisation or domain%s");
  std::vector<float> small(kSurrSmall);
  std::vector<__nv_bfloat16> planes(4 * kSurrPlane);
  surrogate_pack(sg->params, small.data(), planes.data());
  const int cells = sg->map_t * sg->map_z;
  SurrogateInfo& I = ctx->surrInfo;
  for (int i = 0; i < 3; ++i) {
    I.inMean[i] = sg->in_mean[i];
    I.inScale[i] = sg->in_scale[i];
    I.lo[i] = sg->lo[i];
    I.hi[i] = sg->hi[i];
  }
  I.yMean = sg->y_mean;
  I.yScale = sg->y_scale;
  I.mapT = sg->map_t;
  I.mapZ = sg->map_z;
  I.mapLoT = sg->map_lo_t;
  I.mapLoZ = sg->map_lo_z;
  I.mapInvDT = 1.0f / sg->map_dt;
  I.mapInvDZ = 1.0f / sg->map_dz;
  // The map followed by its row flags (1: some cell of the row uses the network).
  const int mapBytes = surrogate_map_bytes(sg->map_t, sg->map_z);
  std::vector<uint8_t> map(sg->use_table, sg->use_table + cells);
  for (int t = 0; t < sg->map_t; ++t) {
    uint8_t any = 0;
    for (int z = 0; z < sg->map_z; ++z) any |= sg->use_table[t * sg->map_z + z] == 0;
    map.push_back(any);
  }
  if (evolve_shared_bytes(MODE_SURROGATE, ctx->globals.nT, ctx->globals.nZ, mapBytes) > 227 * 1024)
    return fail(ctx, GAL_ERR_TOO_LARGE, "gal_gpu_set_surrogate: shared memory footprint too large%s");
  if (cudaMalloc(&ctx->dSurrSmall, small.size() * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&ctx->dSurrPlanes, planes.size() * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&ctx->dSurrMap, mapBytes) != cudaSuccess ||
      cudaMalloc(&ctx->dSurrStats, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    free_surrogate(ctx);
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_set_surrogate: device allocation failed%s");
  }
  if (cudaMemcpy(ctx->dSurrSmall, small.data(), small.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dSurrPlanes, planes.data(), planes.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->dSurrMap, map.data(), mapBytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(ctx->dSurrStats, 0, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    free_surrogate(ctx);
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_set_surrogate: upload failed%s");
  }
  return GAL_OK;
}

int gal_gpu_set_surrogate_split(gal_ctx* ctx, int32_t split) {
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_set_surrogate_split: NULL context%s");
  ctx->splitSurrogate = split ? 1 : 0;
  return GAL_OK;
}

int gal_gpu_surrogate_stats(const gal_ctx* ctx, uint64_t* network, uint64_t* table) {
  if (!ctx) return GAL_ERR_ARGUMENT;
  unsigned long long h[2] = {0, 0};
  if (ctx->dSurrStats) {
    cudaStreamSynchronize(ctx->stream);
    if (cudaMemcpy(h, ctx->dSurrStats, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return GAL_ERR_CUDA;
  }
  if (network) *network = h[0];
  if (table) *table = h[1];
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

// Scratch layout: [0,256) queue head; then the double2 table [nZ*nT]; the
// short-log table [128 double2]; ln T [nT]; ln Z [nZ] and
// 1/(ln Z[i+1]-ln Z[i]) [nZ]; the 2^(j/64) table [64] (the shared layout).
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

// The grid-spacing constants gal_gpu_init derives (evenly spaced rows in
// ln Z and ln T: the cell is found by arithmetic), computed from the raw
// grids one logarithm at a time so that nothing is allocated; then the FP32
// copies.  Same Globals as a context built from the same table.
void noalloc_uniform_grids(Globals& g, const double* temperature, const double* metallicity, int nT, int nZ) {
  auto lnZ = [&](int j) { return metallicity[j] > 0.0 ? std::log(metallicity[j]) : -999.0; };
  const int first = g.firstZero ? 1 : 0;
  g.zFirstLog = first;
  g.lnZFirst = lnZ(first);
  g.zUniform = 0;
  if (nZ - first >= 2) {
    const double d = (lnZ(nZ - 1) - lnZ(first)) / (nZ - 1 - first);
    bool even = true;
    for (int j = first; j + 1 < nZ && even; ++j) even = std::fabs(lnZ(j + 1) - lnZ(j) - d) <= 1.0e-9 * std::fabs(d);
    if (even) {
      g.invDlnZ = 1.0 / d;
      g.zUniform = 1;
    }
  }
  fill_fast_constants(g);
  g.tUniform = 0;
  const double lnT0 = std::log(temperature[0]);
  const double d = (std::log(temperature[nT - 1]) - lnT0) / (nT - 1);
  bool even = true;
  for (int i = 0; i + 1 < nT && even; ++i)
    even = std::fabs(std::log(temperature[i + 1]) - std::log(temperature[i]) - d) <= 1.0e-9 * std::fabs(d);
  if (even) {
    g.f.lnTFirst = (float)lnT0;
    g.f.invDlnT = (float)(1.0 / d);
    g.tUniform = 1;
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
  if ((unsigned long long)n * GAL_NY > (1ull << 62))
    return fail(nullptr, GAL_ERR_TOO_LARGE, "gal_gpu_evolve_batch_noalloc: batch too large%s");
  if (p->sf_disk_rate != GAL_SF_RATE_TIMESCALE)
    return fail(nullptr, GAL_ERR_ARGUMENT,
                "gal_gpu_evolve_batch_noalloc: only the timescale disk star-formation rate (its tables need memory)%s");
  const int nT = t->n_temperature, nZ = t->n_metallicity;
  if (nT < 2 || nZ < 2 || !t->temperature || !t->metallicity || !t->cooling_rate || !t->electron_density)
    return fail(nullptr, GAL_ERR_TABLE, "gal_gpu_evolve_batch_noalloc: CIE table needs at least 2x2 entries%s");
  // The cell count first, in 64-bit arithmetic, so that the int sizes below
  // cannot overflow for an absurd table.
  if ((uint64_t)nT * (uint64_t)nZ > kNoAllocScratchBytes / sizeof(double2) || noalloc_bytes(nT, nZ) > kNoAllocScratchBytes)
    return fail(nullptr, GAL_ERR_TOO_LARGE,
                "gal_gpu_evolve_batch_noalloc: CIE table too large for the fixed 128 KiB scratch "
                "(16 (n_metallicity*n_temperature + 128) + 8 (n_temperature + 2 n_metallicity + 64) + 256 bytes must not exceed 131072)%s");
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
  double2* fastLog = tab + (size_t)nZ * nT;
  double* lnT = (double*)(fastLog + kLogTableSize);
  double* lnZ = lnT + nT;
  double* fastExp = lnZ + 2 * nZ;

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
  noalloc_uniform_grids(g, t->temperature, t->metallicity, nT, nZ);

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
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(fastLog, host_fast_log_table(), kLogTableSize * sizeof(double2), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(fastExp, host_fast_exp_table(), kExpTableSize * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    noalloc_prepare_tables<<<32, 256, 0, st>>>(tab, lnT, lnZ, nT, nZ);
    e = cudaGetLastError();
  }
  // The queue head must start at zero: the array keeps the last call's contents.
  if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    LaunchArgs a{};
    a.G = g;
    a.b = Batch{n, state, param, tStart, tEnd, step, status, counters, queue};
    a.tables = DeviceTables{tab, lnT, lnZ, fastLog, fastExp, nullptr, nullptr};
    a.shm = shared_bytes(nT, nZ);
    a.blocks = std::max<int64_t>(1, std::min<int64_t>(sms, (n + kNoAllocThreads - 1) / kNoAllocThreads));
    a.stream = st;
    e = evolve_launch_plain(kNoAllocThreads, a);
  }
  if (e != cudaSuccess) return fail(nullptr, GAL_ERR_CUDA, "gal_gpu_evolve_batch_noalloc: CUDA error: %s", cudaGetErrorString(e));
  return GAL_OK;
}
