// evolve_kernel.cuh -- the persistent node-evolution kernel and its launch.
//
// One thread owns one node at a time and integrates it with the Cash-Karp
// 4(5) stepper and the reference's scaled error controller, trial loop and
// post-step clamps (merger_trees/node_evolver/standard.F90:385-755,
// numerical/ODE_solver/solver.F90:492-691, external/gslODEInitVal2/
// driver2.c:148-250, cscal2.c:93-169).  The kernel is persistent: each warp
// loops over RK attempts, and a lane whose node has finished takes the next
// node from a device work queue (one atomic per warp), so lanes stay busy
// however uneven the per-node step counts are.
//
// Four forms share the stepper (EvolveMode):
//   PLAIN          FP64 rates, CIE table (parity form: the reference's arithmetic)
//   SURROGATE      FP64 rates, cooling function from the MLP surrogate
//   FAST           FP32 rates (galnode_physics_fast.cuh), FP32 CIE table
//   FAST_SURROGATE FP32 rates, cooling function from the MLP surrogate
// In every form the state, the accepted-step update, the error norm and the
// step-size control are FP64.  The instantiations live in evolve_*.cu, one
// translation unit per form, so that they compile in parallel.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <type_traits>

#include "../../include/galnode.h"
#include "galnode_physics.cuh"
#include "galnode_physics_fast.cuh"
#include "surrogate.cuh"

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
// Stage abscissae (used only by the interrupt form, where evaluation times matter).
constexpr double a2 = 1.0 / 5.0, a3 = 3.0 / 10.0, a4 = 3.0 / 5.0, a5 = 1.0, a6 = 7.0 / 8.0;
}  // namespace ck

enum EvolveMode : int { MODE_PLAIN = 0, MODE_SURROGATE = 1, MODE_FAST = 2, MODE_FAST_SURROGATE = 3 };

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
  // Interrupt form only (gal_gpu_evolve_batch_interrupt): the GAL_COMPONENT_*
  // mask of each node, and the time reached and interrupt task.
  const int32_t* components;
  double* tReached;
  int32_t* task;
  // Optional work list (the surrogate forms' split launch): when set, the
  // queue walks order[0 .. *orderCount) instead of 0 .. n, and then, when
  // orderBackCount is set, the *orderBackCount entries written from the
  // list's far end down: order[orderCap - 1], order[orderCap - 2], ...
  const int32_t* order;
  const unsigned long long* orderCount;
  const unsigned long long* orderBackCount;
  int64_t orderCap;
};

// Device tables: the FP64 forms read gTab/gLnT/gLnZ/gFastLog/gFastExp, the
// FP32 forms gTabF/gLnZF (and gLnT for the temperature cell of each node).
struct DeviceTables {
  const double2* tab;     // (ln Lambda, ln n_e/n_H) [nZ][nT]
  const double* lnT;      // [nT]
  const double* lnZ;      // ln Z [nZ], then 1/(ln Z[i+1] - ln Z[i]) [nZ]
  const double2* fastLog; // short-log table [kLogTableSize]
  const double* fastExp;  // 2^(j/64) [kExpTableSize]
  const float2* tabF;     // FP32 copy of tab
  const float* lnZF;      // FP32 copy of lnZ (both halves)
  KmtTables<double> kmt;  // Krumholz (2009) disk tables (global memory)
  KmtTables<float> kmtF;
};

// Device copy of an installed cooling-function surrogate.
struct SurrogateDev {
  const float* small;          // kSurrSmall FP32 values
  const __nv_bfloat16* planes; // W2 hi, W2 lo, W3 hi, W3 lo, each [64][kMlpStride]
  const uint8_t* map;          // [mapT][mapZ] use-table flags, then [mapT] row flags (surrogate_map_bytes)
  SurrogateInfo info;
  unsigned long long* stats;   // [2]: network and table evaluations
};

// A forest resident on the device (gal_gpu_forest_*): topology, the
// pieces ("segments") each node's interval is cut into at the output times,
// and the per-node and per-snapshot results.  Progenitor-less nodes are the
// initial work; the last progenitor of a node to finish merges them into it
// and goes on with it.
struct ForestDev {
  int64_t n;                    // nodes
  int64_t nLeaves;
  const int32_t* leaves;        // [nLeaves] progenitor-less nodes
  const int32_t* parent;        // [n], -1 for a root
  const int32_t* childFirst;    // [n]
  const int32_t* childCount;    // [n]
  int32_t* pending;             // [n] progenitors not yet finished (reset before each evolution)
  const int32_t* segFirst;      // [n]
  const int32_t* segCount;      // [n]
  const int32_t* snapInitial;   // [n] snapshot slot of an output at the node's own time, or -1
  int64_t nSeg;
  const double* segParam;       // [GAL_NP][nSeg]
  const double* segT0;          // [nSeg]
  const double* segT1;          // [nSeg]
  const int32_t* segSnap;       // [nSeg] snapshot slot at the segment's end, or -1
  const double* state0;         // [GAL_NY][n] initial states (progenitor-less nodes)
  double* state;                // [GAL_NY][n] segment start states, then final states
  double* stepOut;              // [n] the step size on finishing (carried to the parent)
  int64_t nSnap;
  double* snapshots;            // [GAL_NY][nSnap]
  int32_t* status;              // [n]
  uint32_t* counters;           // [3][n]
  unsigned long long* head;     // next unclaimed leaf (zeroed before each evolution)
};

// Shared-memory layout.  FP64 forms: [nZ*nT] double2 tables, the short-log
// table [128 double2], ln T [nT], ln Z [nZ], 1/(ln Z[i+1] - ln Z[i]) [nZ],
// the 2^(j/64) table [64].  FP32 forms: [nZ*nT] float2 tables, ln Z and the
// reciprocal spacings [2 nZ, rounded up to even].  The surrogate forms
// append the network (kSurrSmall floats rounded up to a multiple of 4, then
// the four BF16 planes) and the error map.
__host__ __device__ inline size_t shared_bytes(int nT, int nZ) {
  return (size_t)(nZ * nT + kLogTableSize) * sizeof(double2) + (size_t)(nT + 2 * nZ + kExpTableSize) * sizeof(double);
}
__host__ __device__ inline size_t shared_bytes_fast(int nT, int nZ) {
  return (size_t)nZ * nT * sizeof(float2) + (size_t)((2 * nZ + 1) & ~1) * sizeof(float);
}
// The error map on the device: [mapT][mapZ] use-table flags, then one flag
// per T row: 1 when at least one cell of the row is served by the network.
__host__ __device__ inline int surrogate_map_bytes(int mapT, int mapZ) { return mapT * (mapZ + 1); }
__host__ __device__ inline size_t surrogate_shared_bytes(int mapCells) {
  return (size_t)((kSurrSmall + 3) & ~3) * sizeof(float) + 4 * (size_t)kSurrPlane * sizeof(__nv_bfloat16) +
         (size_t)((mapCells + 15) & ~15);
}
// The surrogate block starts on a 16-byte boundary (ldmatrix row addresses).
__host__ __device__ inline size_t surrogate_offset(int mode, int nT, int nZ) {
  const size_t base = (mode & MODE_FAST) ? shared_bytes_fast(nT, nZ) : shared_bytes(nT, nZ);
  return (base + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t evolve_shared_bytes(int mode, int nT, int nZ, int mapCells) {
  if (!(mode & MODE_SURROGATE)) return (mode & MODE_FAST) ? shared_bytes_fast(nT, nZ) : shared_bytes(nT, nZ);
  return surrogate_offset(mode, nT, nZ) + surrogate_shared_bytes(mapCells);
}

// Decrement a progenitor counter with acquire-release semantics at GPU
// scope; true for the decrement that takes it to zero.
__device__ __forceinline__ bool last_progenitor(int32_t* counter) {
  int32_t old;
  asm volatile("atom.acq_rel.gpu.add.s32 %0, [%1], -1;" : "=r"(old) : "l"(counter) : "memory");
  return old == 1;
}

// First error-map cell of the T row of a node at log10 T = lt, or -1 when
// the network can serve none of its evaluations (cooling cut off, T outside
// the training domain, or every cell of the row marked for the table).
__device__ __forceinline__ int surrogate_net_row(const SurrogateInfo& I, const uint8_t* map, float lt, bool cooling) {
  if (!cooling || !(lt >= I.lo[0] && lt <= I.hi[0])) return -1;
  const int it = min(max((int)((lt - I.mapLoT) * I.mapInvDT), 0), I.mapT - 1);
  return map[I.mapT * I.mapZ + it] ? it * I.mapZ : -1;
}

// Whether the network may serve the node of this lane at state y: its T
// row has network cells, it has hot gas, and its metallicity is inside the
// training domain in a cell the error map leaves to the network (the first
// tests of surrogate_cooling).  Decided once per attempted step, at the
// attempt's starting state: a warp none of whose lanes passes takes the
// step with the table alone, on the unrolled path of the forms without a
// surrogate.
template <class NodeT, class Real>
__device__ __forceinline__ bool surrogate_open(const SurrogateInfo& I, const uint8_t* map, const NodeT& c, const Real* y) {
  const float massHot = (float)y[GAL_Y_HOT_MASS];
  if (c.netRow < 0 || !(massHot > 0.0f)) return false;
  const float metals = (float)y[GAL_Y_HOT_METALS];
  const float zf = metals > massHot ? 1.0f : (metals <= 0.0f ? 0.0f : __fdividef(metals, massHot));
  const float zs = zf * (float)(1.0 / k::metallicitySolar);
  const float lz = zs > 0.0f ? __log10f(zs) : -1.0e30f;
  if (!(lz >= I.lo[1] && lz <= I.hi[1])) return false;
  const int iz = min(max((int)((lz - I.mapLoZ) * I.mapInvDZ), 0), I.mapZ - 1);
  return map[c.netRow + iz] == 0;
}

// Cooling function (without the n_H^2 factor) and n_e/n_H of one
// right-hand-side evaluation from the surrogate, for the node of this lane:
// the network gives log10 Lambda at the central hot-gas density and n_e/n_H
// is interpolated from the table in FP32.  use = false (the caller
// interpolates the table) outside the training domain, in error-map cells
// marked for the table, and when there is no hot gas.  Warp-collective.
template <class NodeT, class Real, class Tab2, class TabR>
__device__ __forceinline__ CoolingValuesF surrogate_cooling(const Globals& G, const Tab2* tab, const TabR* lnZTab,
                                                           const TabR* invDlnZTab, const SurrogateSmem& N,
                                                           const SurrogateInfo& I, const uint8_t* map, const NodeT& c,
                                                           const Real* y, bool active, int lane, uint32_t& nNet,
                                                           uint32_t& nTab) {
  const float massHot = (float)y[GAL_Y_HOT_MASS];
  const float metals = (float)y[GAL_Y_HOT_METALS];
  // The node's T row (its cooling cut-off, T domain and whether any cell of
  // the row uses the network) is fixed per node: c.netRow.  Then the Z
  // domain and the map cell, and last the n_H domain, so that a lane bound
  // for the table stops early.  The decision is the same as testing every
  // condition.
  const float lt = c.log10T;
  float zs = 0.0f, lz = -1.0e30f, ln = -1.0e30f;
  bool ok = active && c.netRow >= 0 && massHot > 0.0f;
  if (ok) {
    const float zf = metals > massHot ? 1.0f : (metals <= 0.0f ? 0.0f : __fdividef(metals, massHot));
    zs = zf * (float)(1.0 / k::metallicitySolar);
    lz = zs > 0.0f ? __log10f(zs) : -1.0e30f;
    ok = lz >= I.lo[1] && lz <= I.hi[1];
    if (ok) {
      const int iz = min(max((int)((lz - I.mapLoZ) * I.mapInvDZ), 0), I.mapZ - 1);
      ok = map[c.netRow + iz] == 0;
    }
    if (ok) {
      const float xH = fminf(fmaxf(zs * (float)(k::hydrogenByMassSolar - k::hydrogenByMassPrimordial) +
                                   (float)k::hydrogenByMassPrimordial, 0.7f), (float)k::hydrogenByMassPrimordial);
      const float nH = massHot * (float)c.rho0PerMass * xH * (float)k::densityToHydrogenNumber;
      ln = nH > 0.0f ? __log10f(nH) : -1.0e30f;
      ok = ln >= I.lo[2] && ln <= I.hi[2];
    }
  }
  CoolingValuesF cv{false, 0.0f, 0.0f};
  // The network runs only when some lane of the warp can use it.
  const unsigned need = __ballot_sync(FULL, ok);
  if (!need) {
    if (active) ++nTab;
    return cv;
  }
  const float x0 = ok ? (lt - I.inMean[0]) / I.inScale[0] : 0.0f;
  const float x1 = ok ? (lz - I.inMean[1]) / I.inScale[1] : 0.0f;
  const float x2 = ok ? (ln - I.inMean[2]) / I.inScale[2] : 0.0f;
  const float yn = surrogate_eval(N, x0, x1, x2, lane, need);
  if (ok) {
    // Lambda without its n_H^2 factor, as the table stores it: the network
    // output is log10 Lambda - 2 log10 n_H.
    cv.lambda = exp10f(fmaf(yn, I.yScale, I.yMean));
    // n_e/n_H: bilinear interpolation of the log table in FP32.
    int iZ;
    float hZ;
    if (G.firstZero && zs < G.f.firstNonZero) {
      iZ = 0;
      hZ = zs * G.f.invFirstNonZero;
    } else {
      const float lnZ = lz * 2.302585093f;
      const int last = G.nZ - 2;
      int j = G.zFirstLog + (int)floorf((lnZ - G.f.lnZFirst) * G.f.invDlnZ);
      j = min(max(j, G.zFirstLog), last);
      iZ = j;
      hZ = fminf(fmaxf((lnZ - (float)lnZTab[j]) * (float)invDlnZTab[j], 0.0f), 1.0f);
    }
    const int nT = G.nT;
    const float hT = (float)c.hT;
    const float a = (float)tab[iZ * nT + c.iT].y, b = (float)tab[(iZ + 1) * nT + c.iT].y;
    const float d = (float)tab[iZ * nT + c.iT + 1].y, e = (float)tab[(iZ + 1) * nT + c.iT + 1].y;
    cv.electrons = __expf((1.0f - hT) * ((1.0f - hZ) * a + hZ * b) + hT * ((1.0f - hZ) * d + hZ * e));
    cv.use = true;
    ++nNet;
  } else if (active) {
    ++nTab;
  }
  return cv;
}

template <int THREADS, int MODE, bool FOREST, bool INTR = false, bool KMT = false>
__global__ void __launch_bounds__(THREADS, 1)
evolve_kernel(const __grid_constant__ Globals G, Batch b, const __grid_constant__ DeviceTables T,
              const __grid_constant__ SurrogateDev sd, const __grid_constant__ ForestDev F) {
  static_assert(!INTR || (MODE == MODE_PLAIN && !FOREST), "interrupts: batches in the plain form only");
  static_assert(!KMT || !(MODE & MODE_SURROGATE), "krumholz2009 disks: the forms without a surrogate");
  constexpr bool SURR = (MODE & MODE_SURROGATE) != 0;
  constexpr bool FAST = (MODE & MODE_FAST) != 0;
  // Step control with few FP64 instructions (integer-pipe compares, seeded
  // reciprocal and roots): the FP32-rate batch forms.  The forest forms keep
  // the plain controller: there it measured 3-4% slower (registers).
  constexpr bool FASTCTL = FAST && !FOREST;
  using RateT = typename std::conditional<FAST, float, double>::type;
  extern __shared__ double2 smem[];
  const int nT = G.nT, nZ = G.nZ;
  const int lane = threadIdx.x & 31;

  // ---- stage the tables (and the network) into shared memory
  Smem S{};
  SmemF SF{};
  const double* sLnT = T.lnT;  // FAST: node_setup reads ln T from global memory
  unsigned char* tail;
  if constexpr (FAST) {
    float2* sTab = reinterpret_cast<float2*>(smem);
    float* sLnZ = reinterpret_cast<float*>(sTab + nZ * nT);
    for (int i = threadIdx.x; i < nZ * nT; i += blockDim.x) sTab[i] = T.tabF[i];
    for (int i = threadIdx.x; i < 2 * nZ; i += blockDim.x) sLnZ[i] = T.lnZF[i];
    SF = SmemF{sTab, sLnZ, sLnZ + nZ, T.kmtF};
    tail = reinterpret_cast<unsigned char*>(smem) + surrogate_offset(MODE, nT, nZ);
  } else {
    double2* sTab = smem;
    double2* sFastLog = sTab + nZ * nT;
    double* lnT = reinterpret_cast<double*>(sFastLog + kLogTableSize);
    double* sLnZ = lnT + nT;
    double* sInvDlnZ = sLnZ + nZ;
    double* sFastExp = sInvDlnZ + nZ;
    for (int i = threadIdx.x; i < nZ * nT; i += blockDim.x) sTab[i] = T.tab[i];
    for (int i = threadIdx.x; i < nT; i += blockDim.x) lnT[i] = T.lnT[i];
    for (int i = threadIdx.x; i < 2 * nZ; i += blockDim.x) sLnZ[i] = T.lnZ[i];  // ln Z, then the reciprocal spacings
    for (int i = threadIdx.x; i < kLogTableSize; i += blockDim.x) sFastLog[i] = T.fastLog[i];
    for (int i = threadIdx.x; i < kExpTableSize; i += blockDim.x) sFastExp[i] = T.fastExp[i];
    S = Smem{sTab, sLnZ, sInvDlnZ, FastTables{sFastLog, sFastExp}, T.kmt};
    sLnT = lnT;
    tail = reinterpret_cast<unsigned char*>(smem) + surrogate_offset(MODE, nT, nZ);
  }
  const float* sSmall = nullptr;
  const __nv_bfloat16* sPlanes = nullptr;
  const uint8_t* sMap = nullptr;
  if constexpr (SURR) {
    float* small = reinterpret_cast<float*>(tail);
    __nv_bfloat16* planes = reinterpret_cast<__nv_bfloat16*>(small + ((kSurrSmall + 3) & ~3));
    uint8_t* map = reinterpret_cast<uint8_t*>(planes + 4 * kSurrPlane);
    for (int i = threadIdx.x; i < kSurrSmall; i += blockDim.x) small[i] = sd.small[i];
    for (int i = threadIdx.x; i < 4 * kSurrPlane / 2; i += blockDim.x)
      reinterpret_cast<uint32_t*>(planes)[i] = reinterpret_cast<const uint32_t*>(sd.planes)[i];
    for (int i = threadIdx.x; i < surrogate_map_bytes(sd.info.mapT, sd.info.mapZ); i += blockDim.x) map[i] = sd.map[i];
    sSmall = small;
    sPlanes = planes;
    sMap = map;
  }
  __syncthreads();
  SurrogateSmem N{};
  if constexpr (SURR) N = surrogate_view(sSmall, sPlanes);

  const int64_t n = b.n;
  const int64_t nFront = (!FOREST && b.order) ? (int64_t)*b.orderCount : n;
  const int64_t nWork = nFront + ((!FOREST && b.order && b.orderBackCount) ? (int64_t)*b.orderBackCount : 0);
  const double epsAbs = G.p.ode_tolerance_absolute, epsRel = G.p.ode_tolerance_relative;
  const float epsAbsF = (float)epsAbs, epsRelF = (float)epsRel;
  const uint32_t budget = (uint32_t)max(G.p.step_budget, 0);

  int phase = PH_NEED;
  int64_t node = 0;
  NodeC c;
  NodeF cf;
  // y, s and the accepted solution are FP64 in every form; the stages k and
  // the stage arguments x are FP64 or FP32 with the rates.
  // In the FP64 forms yr is y itself and ynew shares the stage argument
  // array x, so those forms keep the register footprint of a plain stepper.
  // The tolerance scales s are FP64 in the FP64 forms; in the FP32-rate
  // forms they are kept in FP32 (coarse scales: 1e-3 of the halo mass and
  // the like) and the picked component's D is formed in FP64 from them.
  double y[GAL_NY];
  RateT s[GAL_NY];
  RateT k1[GAL_NY], k2[GAL_NY], k3[GAL_NY], k4[GAL_NY], k5[GAL_NY], k6[GAL_NY], x[GAL_NY];
  float yf[GAL_NY];
  double ynewF[GAL_NY];
  RateT* yr;
  double* ynew;
  if constexpr (FAST) {
    yr = yf;
    ynew = ynewF;
  } else {
    yr = y;
    ynew = x;
  }
  double t = 0.0, t0 = 0.0, t1 = 0.0, h = 0.0, stepIn = -1.0;
  double dtLeft = 0.0;  // t1 - t (FP32-rate forms: formed when t changes, not per attempt)
  int trial = 0;
  uint32_t count = 0, nAcc = 0, nRej = 0, nRhs = 0, nNet = 0, nTab = 0;
  // Lanes that never take a node still hold in-range table coordinates.
  c.log10T = 0.0f;
  cf.log10T = 0.0f;
  c.netRow = cf.netRow = -1;
  c.iT = cf.iT = 0;
  c.hT = 0.0;
  cf.hT = 0.0f;

  // One right-hand-side evaluation at xx for the lanes with `active`; with
  // the surrogate, every lane of the warp takes part in the network evaluation.
  // `net` (std::true_type / std::false_type) selects at compile time
  // whether this call site may use the network; without it the table is
  // interpolated as in the forms without a surrogate.
  auto eval = [&](const RateT* xx, RateT* d, bool active, auto net) {
    constexpr bool NET = SURR && decltype(net)::value;
    if constexpr (FAST) {
      if constexpr (NET) {
        const CoolingValuesF cv =
            surrogate_cooling(G, SF.tab, SF.lnZ, SF.invDlnZ, N, sd.info, sMap, cf, xx, active, lane, nNet, nTab);
        if (active) rhs_fast(G, SF, cf, xx, d, cv);
      } else {
        if (SURR && active) ++nTab;
        rhs_fast<KMT>(G, SF, cf, xx, d);
      }
    } else {
      if constexpr (NET) {
        const CoolingValuesF cv =
            surrogate_cooling(G, S.tab, S.lnZ, S.invDlnZ, N, sd.info, sMap, c, xx, active, lane, nNet, nTab);
        if (active) rhs(G, S, c, xx, d, CoolingValues{cv.use, (double)cv.lambda, (double)cv.electrons});
      } else {
        if (SURR && active) ++nTab;
        rhs<KMT>(G, S, c, xx, d);
      }
    }
  };
  // Whether the warp must enter a right-hand-side evaluation.
  auto any = [&](bool p) { return SURR ? __any_sync(FULL, p) : p; };
  // Per-node constants of the current evolve call (FP32 in the FP32-rate
  // forms, where the FP64 ones would only be rounded to FP32).
  auto setup = [&](const double* prm) {
    if constexpr (FAST) {
      node_setup_fast(G, sLnT, prm, cf);
      c.massHalo = prm[GAL_P_MASS];
      if constexpr (SURR) cf.netRow = surrogate_net_row(sd.info, sMap, cf.log10T, cf.coolingAllowed);
    } else {
      node_setup(G, sLnT, prm, c);
      if constexpr (SURR) c.netRow = surrogate_net_row(sd.info, sMap, c.log10T, c.coolingAllowed);
    }
  };
  // Absolute-tolerance scales of the current evolve call.
  auto set_scales = [&]() {
    if constexpr (FAST) {
      float yv[GAL_NY];
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) yv[v] = (float)y[v];
      scales_fast(yv, (float)c.massHalo, s);
    } else {
      double sd[GAL_NY];
      scales(y, c.massHalo, sd);
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) s[v] = (RateT)sd[v];
    }
  };
  // The FP32 copy of y in the FAST forms.
  auto sync_yr = [&]() {
    if constexpr (FASTCTL) {
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) yf[v] = d2f_int(y[v]);
    } else if constexpr (FAST) {
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) yf[v] = (float)y[v];
    }
  };
  // The post-step clamps; the FP32-rate forms test for a negative mass on
  // the integer pipe first (post_step's FP64 compares only when one is).
  auto post_step_any = [&](double* yy) -> bool {
    if constexpr (FASTCTL) return post_step_int(yy);
    else return post_step(yy);
  };

  // ---- work source and completion: a batch of independent nodes, or a forest
  int32_t seg = 0, segEnd = 0;
  // (forest) Set up the current segment of the node: its constants, tolerance
  // scales and interval; keep the starting state for trial restarts.
  auto start_segment = [&]() {
    double prm[GAL_NP];
#pragma unroll
    for (int v = 0; v < GAL_NP; ++v) prm[v] = F.segParam[v * F.nSeg + seg];
    setup(prm);
#pragma unroll
    for (int v = 0; v < GAL_NY; ++v) F.state[v * F.n + node] = y[v];
    set_scales();
    t0 = F.segT0[seg];
    t1 = F.segT1[seg];
    trial = 0;
    phase = PH_TRIAL;
  };
  // (forest) Finish the node with state y and status st; while this lane is
  // the last progenitor of the parent to finish, merge the progenitors into
  // the parent (the primary's state, then each other progenitor in index
  // order merged into it as a satellite, merge_satellite) and go on with
  // the parent.
  auto complete_node = [&](int st) {
    for (;;) {
      // The parent's fields are read-only during the evolution: read them
      // with the parent index, before the decrement, so that the merge
      // waits on no further lookup.
      const int32_t par = F.parent[node];
      int32_t c0 = 0, cn = 0, slot = -1, s0 = 0, sn = 0;
      if (par >= 0) {
        c0 = F.childFirst[par];
        cn = F.childCount[par];
        slot = F.snapInitial[par];
        s0 = F.segFirst[par];
        sn = F.segCount[par];
      }
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) F.state[v * F.n + node] = y[v];
      F.stepOut[node] = stepIn;
      F.status[node] = st;
      if (F.counters) {
        F.counters[node] = nAcc;
        F.counters[F.n + node] = nRej;
        F.counters[2 * F.n + node] = nRhs;
      }
      // One acquire-release decrement of the parent's counter: its release
      // half orders this lane's stores above before the decrement, and for
      // the lane that takes the counter to zero its acquire half orders the
      // other progenitors' stores (each released by their own decrement, in
      // the counter's release sequence) before the merge's loads below.
      if (par < 0 || !last_progenitor(&F.pending[par])) {
        phase = PH_NEED;
        return;
      }
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) y[v] = F.state[v * F.n + c0];
      for (int32_t j = 1; j < cn; ++j) {
        double sat[GAL_NY];
#pragma unroll
        for (int v = 0; v < GAL_NY; ++v) sat[v] = F.state[v * F.n + c0 + j];
        merge_satellite(y, sat, G.p.merger_mass_ratio_major);
      }
      stepIn = F.stepOut[c0];
      node = par;
      nAcc = nRej = nRhs = 0;
      if (slot >= 0) {
#pragma unroll
        for (int v = 0; v < GAL_NY; ++v) F.snapshots[v * F.nSnap + slot] = y[v];
      }
      seg = s0;
      segEnd = s0 + sn;
      if (seg < segEnd) {
        start_segment();
        return;
      }
      st = GAL_STATUS_SUCCESS;  // a node with nothing to evolve (a root at its own time)
    }
  };
  // Take work item idx of the queue.
  auto take = [&](unsigned long long idx) {
    if constexpr (FOREST) {
      if ((int64_t)idx >= F.nLeaves) {
        phase = PH_DONE;
        return;
      }
      node = F.leaves[idx];
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) y[v] = F.state0[v * F.n + node];
      stepIn = -1.0;
      nAcc = nRej = nRhs = 0;
      const int32_t slot = F.snapInitial[node];
      if (slot >= 0) {
#pragma unroll
        for (int v = 0; v < GAL_NY; ++v) F.snapshots[v * F.nSnap + slot] = y[v];
      }
      seg = F.segFirst[node];
      segEnd = seg + F.segCount[node];
      if (seg < segEnd) start_segment();
      else complete_node(GAL_STATUS_SUCCESS);
    } else {
      if ((int64_t)idx >= nWork) {
        phase = PH_DONE;
        return;
      }
      node = !b.order ? (int64_t)idx
                      : (int64_t)b.order[(int64_t)idx < nFront ? (int64_t)idx : b.orderCap - 1 - ((int64_t)idx - nFront)];
      double prm[GAL_NP];
#pragma unroll
      for (int v = 0; v < GAL_NP; ++v) prm[v] = b.param[v * n + node];
      setup(prm);
#pragma unroll
      for (int v = 0; v < GAL_NY; ++v) y[v] = b.state[v * n + node];
      set_scales();
      t0 = b.tStart[node];
      t1 = b.tEnd[node];
      stepIn = b.step[node];
      trial = 0;
      nAcc = nRej = nRhs = 0;
      phase = PH_TRIAL;
    }
  };
  unsigned long long* const queueHead = FOREST ? F.head : b.queue;
  // The state this evolve call started from (trial restarts, failures).
  auto restore_start = [&]() {
#pragma unroll
    for (int v = 0; v < GAL_NY; ++v) y[v] = FOREST ? F.state[v * F.n + node] : b.state[v * n + node];
  };
  // An interval of zero length: nothing to do (node%timeStepSet(-1) in the batch form).
  auto zero_interval = [&]() {
    if constexpr (FOREST) {
      h = stepIn;
      if (++seg < segEnd) start_segment();
      else complete_node(GAL_STATUS_SUCCESS);
    } else {
      b.step[node] = -1.0;
      b.status[node] = GAL_STATUS_SUCCESS;
      if (b.counters) {
        b.counters[node] = 0; b.counters[n + node] = 0; b.counters[2 * n + node] = 0;
      }
      if constexpr (INTR) {
        b.tReached[node] = t1;
        b.task[node] = 0;
      }
      phase = PH_NEED;
    }
  };
  // An evolve call ended with status st.
  auto finish = [&](int st) {
    if constexpr (FOREST) {
      if (st == GAL_STATUS_SUCCESS) {
        const int32_t slot = F.segSnap[seg];
        if (slot >= 0) {
#pragma unroll
          for (int v = 0; v < GAL_NY; ++v) F.snapshots[v * F.nSnap + slot] = y[v];
        }
        stepIn = h;  // node%timeStepSet: carried to the next piece
        if (++seg < segEnd) {
          start_segment();
          return;
        }
        complete_node(st);
      } else {
        restore_start();  // a failed call leaves the node as it started
        complete_node(st);
      }
    } else {
      if (st == GAL_STATUS_SUCCESS) {
#pragma unroll
        for (int v = 0; v < GAL_NY; ++v) b.state[v * n + node] = y[v];
        b.step[node] = h;
      }
      b.status[node] = st;
      if (b.counters) {
        b.counters[node] = nAcc;
        b.counters[n + node] = nRej;
        b.counters[2 * n + node] = nRhs;
      }
      if constexpr (!SURR) nTab += nRhs;  // table evaluations, for the split launch's statistics
      phase = PH_NEED;
    }
  };

  if constexpr (INTR) {
    // The plain form with interrupts (the reference's standardODEs,
    // node_evolver/standard.F90:895-945, with odeSolver%solve's
    // re-targeting, numerical/ODE_solver/solver.F90:608-620): an evaluation
    // that gives a rate to a component the node does not have returns zero
    // derivatives and, when it is the earliest so far, records its time and
    // task and abandons the attempt (GSL_EBADFUNC: the state stays at the
    // step's start); the integration then ends at that time, every
    // evaluation at or after it returning zero derivatives.  As GSL's rkck,
    // each attempt evaluates f(t+h, y_new), which can interrupt too and is
    // the next step's slope on acceptance.  The interrupt persists over the
    // trials of the call; a restarted trial integrates to the interrupt time.
    double kOut[GAL_NY];
    double tInt = 0.0, target = 0.0;
    bool found = false;
    int32_t task = 0;
    uint32_t comps = 0;
    // One evaluation at time ts; true when it sets the earliest interrupt.
    auto evalI = [&](const double* xx, double* d, double ts) -> bool {
      if (found && ts >= tInt) {
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) d[i] = 0.0;
        return false;
      }
      rhs(G, S, c, xx, d);
      ++nRhs;
      const int32_t req = interrupt_request(comps, d);
      if (req) {
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) d[i] = 0.0;
        if (!found || ts < tInt) {
          found = true;
          tInt = ts;
          task = req;
          return true;
        }
      }
      return false;
    };
    for (;;) {
      // ---- refill lanes whose node has finished (warp-aggregated queue pop)
      const unsigned need = __ballot_sync(FULL, phase == PH_NEED);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(queueHead, (unsigned long long)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if (phase == PH_NEED) {
          take(base + __popc(need & ((1u << lane) - 1u)));
          if (phase != PH_DONE) {
            found = false;
            task = 0;
            comps = (uint32_t)b.components[node];
          }
        }
      }
      if (__all_sync(FULL, phase == PH_DONE)) break;

      if (phase == PH_TRIAL && t0 == t1) zero_interval();
      bool finished = false;
      int finalStatus = GAL_STATUS_SUCCESS;
      if (phase == PH_TRIAL) {
        // odeSolverSolve from t0 toward the end (or the interrupt found by
        // an earlier trial); the slope at the start is evaluated first.
        target = found ? fmin(tInt, t1) : t1;
        const double stepSize = G.p.reuse_step_size ? stepIn / (double)(1u << trial) : -1.0;
        h = target - t0;
        if (stepSize > 0.0) h = fmin(stepSize, h);
        if (trial > 0) restore_start();
        t = t0;
        count = 0;
        phase = PH_STEP;
        if (target - t > 0.0 && evalI(y, k1, t)) target = tInt;
        if (!(target - t > 0.0)) finished = true;
      }
      if (phase == PH_STEP && !finished) {
        // ---- one attempted step (rkck with dydt_out, inside evolve_apply)
        const double dt = target - t;
        const bool finalStep = (dt >= 0.0 && h > dt) || (dt < 0.0 && h < dt);
        const double hh = finalStep ? dt : h;
        bool abandon;
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) x[i] = y[i] + ck::b21 * hh * k1[i];
        abandon = evalI(x, k2, t + ck::a2 * hh);
        if (!abandon) {
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) x[i] = y[i] + hh * (ck::b31 * k1[i] + ck::b32 * k2[i]);
          abandon = evalI(x, k3, t + ck::a3 * hh);
        }
        if (!abandon) {
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) x[i] = y[i] + hh * (ck::b41 * k1[i] + ck::b42 * k2[i] + ck::b43 * k3[i]);
          abandon = evalI(x, k4, t + ck::a4 * hh);
        }
        if (!abandon) {
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i)
            x[i] = y[i] + hh * (ck::b51 * k1[i] + ck::b52 * k2[i] + ck::b53 * k3[i] + ck::b54 * k4[i]);
          abandon = evalI(x, k5, t + ck::a5 * hh);
        }
        if (!abandon) {
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i)
            x[i] = y[i] + hh * (ck::b61 * k1[i] + ck::b62 * k2[i] + ck::b63 * k3[i] + ck::b64 * k4[i] + ck::b65 * k5[i]);
          abandon = evalI(x, k6, t + ck::a6 * hh);
        }
        if (!abandon) {
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) x[i] = y[i] + hh * (ck::c1 * k1[i] + ck::c3 * k3[i] + ck::c4 * k4[i] + ck::c6 * k6[i]);
          abandon = evalI(x, kOut, t + hh);
        }
        if (abandon) {
          // The attempt is abandoned: the integration now ends at the interrupt.
          target = tInt;
          if (!(target - t > 0.0)) finished = true;
        } else {
          double errMax = 0.0, dMax = 1.0;
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) {
            const double err = fabs(hh * (ck::e1 * k1[i] + ck::e3 * k3[i] + ck::e4 * k4[i] + ck::e5 * k5[i] + ck::e6 * k6[i]));
            const double D0 = fabs(epsRel * fabs(x[i]) + epsAbs * s[i]);
            if (err * dMax > errMax * D0 || !(err == err)) {
              errMax = err;
              dMax = D0;
            }
          }
          const double rmax = dmax(fast_div(errMax, dMax), 2.2250738585072014e-308);
          ++count;
          const double tNew = finalStep ? target : t + hh;
          double hNew = hh;
          bool decrease = false;
          if (rmax > 1.1) {
            double r = rmax > 1845.28125 ? 0.2 : 0.9 * inv_root<5>(rmax);
            if (r < 0.2) r = 0.2;
            hNew = r * hh;
            decrease = true;
          } else if (rmax < 0.5) {
            double r = rmax < 3.8394e-5 ? 4.9 : 0.9 * inv_root<6>(rmax);
            if (r > 4.9) r = 4.9;
            if (r < 1.0) r = 1.0;
            hNew = r * hh;
          }
          if (decrease) {
            const double tNext = tNew + hNew;
            if (fabs(hNew) < fabs(hh) && tNext != tNew) {
              h = hNew;
              ++nRej;
              if (budget && count >= budget) { finished = true; finalStatus = GAL_STATUS_XCPU; }
            } else {
              ++trial;
              if (trial >= G.p.trial_count_maximum) { finished = true; finalStatus = GAL_STATUS_UNDERFLOW; }
              else phase = PH_TRIAL;
            }
          } else {
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) {
              y[i] = x[i];
              k1[i] = kOut[i];
            }
            t = tNew;
            h = hNew;
            ++nAcc;
            post_step(y);
            if (!(target - t > 0.0 || target - t < 0.0)) {
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
        }
      }
      if (finished) {
        // evolve's results: an interrupted node reports the interrupt time
        // and task and node%timeStep = -1 (standard.F90:729-737).
        if (finalStatus == GAL_STATUS_SUCCESS) {
#pragma unroll
          for (int v = 0; v < GAL_NY; ++v) b.state[v * n + node] = y[v];
          b.step[node] = found ? -1.0 : h;
          b.tReached[node] = found ? tInt : t1;
          b.task[node] = found ? task : 0;
          b.status[node] = found ? GAL_STATUS_INTERRUPTED : GAL_STATUS_SUCCESS;
        } else {
          b.tReached[node] = t1;
          b.task[node] = 0;
          b.status[node] = finalStatus;
        }
        if (b.counters) {
          b.counters[node] = nAcc;
          b.counters[n + node] = nRej;
          b.counters[2 * n + node] = nRhs;
        }
        phase = PH_NEED;
      }
    }
  } else if constexpr (MODE == MODE_PLAIN) {
    // The FP64 parity form: every right-hand side inlined at its stage, the
    // stage arguments computed by the whole warp at once.
    for (;;) {
      // ---- refill lanes whose node has finished (warp-aggregated queue pop)
      const unsigned need = __ballot_sync(FULL, phase == PH_NEED);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(queueHead, (unsigned long long)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if (phase == PH_NEED) take(base + __popc(need & ((1u << lane) - 1u)));
      }
      if (__all_sync(FULL, phase == PH_DONE)) break;

      // ---- start (or restart) an ODE trial: odeSolverSolve + driver reset
      if (phase == PH_TRIAL && t0 == t1) zero_interval();
      const bool starting = phase == PH_TRIAL;
      if (starting) {
        const double stepSize = G.p.reuse_step_size ? stepIn / (double)(1u << trial) : -1.0;
        h = t1 - t0;
        if (stepSize > 0.0) h = fmin(stepSize, h);
        if (trial > 0) restore_start();
        sync_yr();
        t = t0;
        count = 0;
      }
      if (any(starting)) eval(yr, k1, starting, std::false_type{});  // dydt_in of the first step
      if (starting) {
        ++nRhs;
        phase = PH_STEP;
      }

      // ---- one attempted step (one pass of gsl_odeiv2_evolve_apply's try_step)
      const bool stepping = phase == PH_STEP;
      bool needOut = false;
      bool finished = false;
      int finalStatus = GAL_STATUS_SUCCESS;
      if (any(stepping)) {
        const double dt = t1 - t;
        const bool finalStep = (dt >= 0.0 && h > dt) || (dt < 0.0 && h < dt);
        const double hh = finalStep ? dt : h;
        const RateT hr = (RateT)hh;
        // Stage arguments: y + h sum_j b_ij k_j (in the rate precision).
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) x[i] = yr[i] + (RateT)ck::b21 * hr * k1[i];
        eval(x, k2, stepping, std::false_type{});
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) x[i] = yr[i] + hr * ((RateT)ck::b31 * k1[i] + (RateT)ck::b32 * k2[i]);
        eval(x, k3, stepping, std::false_type{});
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i)
          x[i] = yr[i] + hr * ((RateT)ck::b41 * k1[i] + (RateT)ck::b42 * k2[i] + (RateT)ck::b43 * k3[i]);
        eval(x, k4, stepping, std::false_type{});
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i)
          x[i] = yr[i] + hr * ((RateT)ck::b51 * k1[i] + (RateT)ck::b52 * k2[i] + (RateT)ck::b53 * k3[i] +
                               (RateT)ck::b54 * k4[i]);
        eval(x, k5, stepping, std::false_type{});
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i)
          x[i] = yr[i] + hr * ((RateT)ck::b61 * k1[i] + (RateT)ck::b62 * k2[i] + (RateT)ck::b63 * k3[i] +
                               (RateT)ck::b64 * k4[i] + (RateT)ck::b65 * k5[i]);
        eval(x, k6, stepping, std::false_type{});
        if (stepping) {
          nRhs += 5;
          // 5th-order solution, scaled error ratio (sc2_control_hadjust, a_y=1, a_dydt=0), FP64.
          // The largest |err_i|/D_i is found by cross-multiplication and divided
          // once (max of the quotients = quotient of the maximal pair).
          double errMax = 0.0, dMax = 1.0;
#pragma unroll
          for (int i = 0; i < GAL_NY; ++i) {
            const RateT inc = (RateT)ck::c1 * k1[i] + (RateT)ck::c3 * k3[i] + (RateT)ck::c4 * k4[i] + (RateT)ck::c6 * k6[i];
            const RateT est = (RateT)ck::e1 * k1[i] + (RateT)ck::e3 * k3[i] + (RateT)ck::e4 * k4[i] + (RateT)ck::e5 * k5[i] +
                              (RateT)ck::e6 * k6[i];
            ynew[i] = y[i] + hh * (double)inc;
            const double err = fabs(hh * (double)est);
            const double D0 = fabs(epsRel * fabs(ynew[i]) + epsAbs * s[i]);
            if (err * dMax > errMax * D0 || !(err == err)) {
              errMax = err;
              dMax = D0;
            }
          }
          const double rmax = dmax(fast_div(errMax, dMax), 2.2250738585072014e-308);  // floor DBL_MIN as cscal2.c
          ++count;
          const double tNew = finalStep ? t1 : t + hh;
          double hNew = hh;
          bool decrease = false;
          // 0.9 rmax^(-1/5), floored at 0.2 (reached for rmax >= 4.5^5 exactly),
          // and 0.9 rmax^(-1/6) capped at 4.9 (reached below (0.9/4.9)^6).
          if (rmax > 1.1) {
            double r = rmax > 1845.28125 ? 0.2 : 0.9 * inv_root<5>(rmax);
            if (r < 0.2) r = 0.2;
            hNew = r * hh;
            decrease = true;
          } else if (rmax < 0.5) {
            double r = rmax < 3.8394e-5 ? 4.9 : 0.9 * inv_root<6>(rmax);
            if (r > 4.9) r = 4.9;
            if (r < 1.0) r = 1.0;
            hNew = r * hh;
          }
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
            for (int i = 0; i < GAL_NY; ++i) y[i] = ynew[i];
            sync_yr();
            t = tNew;
            h = hNew;
            ++nAcc;
            const bool reached = !(t1 - t > 0.0 || t1 - t < 0.0);
            if (reached) {
              post_step(y);
              finished = true;
              bool finite = true;
#pragma unroll
              for (int i = 0; i < GAL_NY; ++i) finite = finite && isfinite(y[i]);
              finalStatus = finite ? GAL_STATUS_SUCCESS : GAL_STATUS_NOT_FINITE;
            } else {
              needOut = true;
            }
          }
        }
      }
      // dydt_out at the accepted point, reused as the next dydt_in; then the
      // post-step clamps (they return GSL_Continue: dydt_out is kept).
      if (any(needOut)) eval(yr, k1, needOut, std::false_type{});
      if (needOut) {
        ++nRhs;
        post_step(y);
        sync_yr();
        if (budget && count >= budget) {
          finished = true;
          finalStatus = GAL_STATUS_XCPU;
        }
      }
      if (finished) finish(finalStatus);
    }
  } else {
    // The other forms (FP32 rates, and the network with either rates): one
    // pass walks the stage index st = 0..5, the same for every lane of the
    // warp: st = 0 is f(y) for lanes that start a trial (dydt_in) or
    // accepted a step in the previous pass (dydt_out, reused as the next
    // dydt_in); st = 1..5 are the stage slopes k2..k6 of an attempt.  Lanes attempt steps together, so the FP64 error norm and
    // step control run once per attempt for the warp.  With the network the
    // stages are a rolled loop around one right-hand-side call site (the
    // network is compiled once); without it they are unrolled.
    bool needOut = false;
    for (;;) {
      // ---- refill lanes whose node has finished (warp-aggregated queue pop)
      const unsigned need = __ballot_sync(FULL, phase == PH_NEED);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(queueHead, (unsigned long long)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if (phase == PH_NEED) take(base + __popc(need & ((1u << lane) - 1u)));
      }
      if (__all_sync(FULL, phase == PH_DONE)) break;

      // ---- start (or restart) an ODE trial: odeSolverSolve + driver reset
      if (phase == PH_TRIAL && (FASTCTL ? !(d_isnan(t0) || d_isnan(t1)) && d_key(t0) == d_key(t1) : t0 == t1)) zero_interval();
      const bool starting = phase == PH_TRIAL;
      if (starting) {
        const double stepSize = G.p.reuse_step_size ? stepIn / (double)(1u << trial) : -1.0;
        h = t1 - t0;
        if (stepSize > 0.0) h = fmin(stepSize, h);
        if (trial > 0) restore_start();
        sync_yr();
        t = t0;
        dtLeft = t1 - t0;
        count = 0;
      }
      const bool atY = starting || needOut;
      bool finished = false;
      int finalStatus = GAL_STATUS_SUCCESS;
      bool stepping = false;
      bool finalStep = false;
      double hh = 0.0;
      RateT hr = (RateT)0;
      const bool anyY = any(atY);
      // With the surrogate: does any lane of the warp start this attempt in
      // a cell the network may serve?
      bool warpNet = false;
      if constexpr (SURR && !FOREST) {
        bool open = false;
        if (atY || phase == PH_STEP) {
          if constexpr (FAST) open = surrogate_open(sd.info, sMap, cf, yr);
          else open = surrogate_open(sd.info, sMap, c, yr);
        }
        warpNet = __any_sync(FULL, open);
      }
      // One stage: its argument, the evaluation and the slope's slot; false
      // when no lane of the warp steps (the attempt is over).
      auto stage = [&](const int st, auto net) -> bool {
        if (st == 1) {
          // ---- the slopes at y are in: begin one attempted step (a pass of
          // gsl_odeiv2_evolve_apply's try_step) for every lane that steps.
          if (starting) {
            ++nRhs;
            phase = PH_STEP;
          }
          if (needOut) {
            // The post-step clamps return GSL_Continue: dydt_out is kept.
            needOut = false;
            ++nRhs;
            if (post_step_any(y)) sync_yr();
            if (budget && count >= budget) {
              finished = true;
              finalStatus = GAL_STATUS_XCPU;
            }
          }
          stepping = phase == PH_STEP && !finished;
          if (!any(stepping)) return false;
          if constexpr (FASTCTL) {
            // The same last-step test with the compares on the integer pipe.
            const double dt = dtLeft;
            finalStep = (d_ge(dt, 0.0) && d_gt(h, dt)) || (d_lt(dt, 0.0) && d_lt(h, dt));
            hh = finalStep ? dt : h;
            hr = (RateT)d2f_int(hh);
          } else {
            const double dt = t1 - t;
            finalStep = (dt >= 0.0 && h > dt) || (dt < 0.0 && h < dt);
            hh = finalStep ? dt : h;
            hr = (RateT)hh;
          }
        }
        // Argument of this evaluation: y, or y + h sum_j b_ij k_j (in the rate precision).
        switch (st) {
          case 0:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) x[i] = yr[i];
            break;
          case 1:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) x[i] = yr[i] + (RateT)ck::b21 * hr * k1[i];
            break;
          case 2:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) x[i] = yr[i] + hr * ((RateT)ck::b31 * k1[i] + (RateT)ck::b32 * k2[i]);
            break;
          case 3:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i)
              x[i] = yr[i] + hr * ((RateT)ck::b41 * k1[i] + (RateT)ck::b42 * k2[i] + (RateT)ck::b43 * k3[i]);
            break;
          case 4:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i)
              x[i] = yr[i] + hr * ((RateT)ck::b51 * k1[i] + (RateT)ck::b52 * k2[i] + (RateT)ck::b53 * k3[i] +
                                   (RateT)ck::b54 * k4[i]);
            break;
          default:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i)
              x[i] = yr[i] + hr * ((RateT)ck::b61 * k1[i] + (RateT)ck::b62 * k2[i] + (RateT)ck::b63 * k3[i] +
                                   (RateT)ck::b64 * k4[i] + (RateT)ck::b65 * k5[i]);
            break;
        }
        RateT d[GAL_NY];
        eval(x, d, st == 0 ? atY : stepping, net);
        switch (st) {
          case 0:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) if (atY) k1[i] = d[i];
            break;
          case 1:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) k2[i] = d[i];
            break;
          case 2:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) k3[i] = d[i];
            break;
          case 3:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) k4[i] = d[i];
            break;
          case 4:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) k5[i] = d[i];
            break;
          default:
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) k6[i] = d[i];
            break;
        }
        return true;
      };
      if constexpr (SURR && FOREST) {
        // Forests keep the one path with the network (a second, unrolled
        // path for the table made the forest kernel slower: 0.276 -> 0.295 s
        // on the 4,096-tree forest, 1.52 -> 1.89 s at scale).
#pragma unroll 1
        for (int st = anyY ? 0 : 1; st <= 5; ++st)
          if (!stage(st, std::true_type{})) break;
      } else if (SURR && warpNet) {
        // One right-hand-side call site with the network, for its code size.
#pragma unroll 1
        for (int st = anyY ? 0 : 1; st <= 5; ++st)
          if (!stage(st, std::true_type{})) break;
      } else {
        // Without the network the stages are unrolled: no stage switch, and
        // the compiler schedules across stages.
        if (anyY) stage(0, std::false_type{});
#pragma unroll
        for (int st = 1; st <= 5; ++st)
          if (!stage(st, std::false_type{})) break;
      }
      if (stepping) {
        nRhs += 5;
        // 5th-order solution (FP64) and the scaled error ratio of
        // sc2_control_hadjust (a_y=1, a_dydt=0).  The component with the
        // largest |err_i|/D_i is picked by cross-multiplied FP32 comparisons;
        // the ratio of the picked component is then formed in FP64 from the
        // FP64 error and the FP64 D_i.  (Picking at FP32 precision can only
        // exchange two components whose ratios agree to ~1e-7.)
        float errMaxF = 0.0f, dMaxF = 1.0f;
        RateT estSel = (RateT)0, incSel = (RateT)0, sSel = (RateT)1;
        double ySel = 0.0;
#pragma unroll
        for (int i = 0; i < GAL_NY; ++i) {
          const RateT inc = (RateT)ck::c1 * k1[i] + (RateT)ck::c3 * k3[i] + (RateT)ck::c4 * k4[i] + (RateT)ck::c6 * k6[i];
          const RateT est = (RateT)ck::e1 * k1[i] + (RateT)ck::e3 * k3[i] + (RateT)ck::e4 * k4[i] + (RateT)ck::e5 * k5[i] +
                            (RateT)ck::e6 * k6[i];
          float ynf;
          if constexpr (FAST) {
            // The FP64 new state is formed only for the picked component and,
            // on acceptance, for all of them: here an FP32 estimate of it
            // serves the D_i of the pick, and the increment is kept (in the
            // free stage-argument array) for the update.
            x[i] = inc;
            ynf = yf[i] + hr * inc;
          } else {
            ynew[i] = y[i] + hh * (double)inc;
            ynf = (float)ynew[i];
          }
          const float errF = fabsf((float)hr * (float)est);
          const float dF = fabsf(epsRelF * fabsf(ynf) + epsAbsF * (float)s[i]);
          if (errF * dMaxF > errMaxF * dF || !(errF == errF)) {
            errMaxF = errF;
            dMaxF = dF;
            estSel = est;
            incSel = inc;
            ySel = FAST ? y[i] : ynew[i];
            sSel = s[i];
          }
        }
        // With nothing picked (every error zero) the ratio is 0, as in FP64.
        // (FP32-rate batch forms: the picked FP32 values are widened exactly
        // on the integer pipe, f2d_int.)
        double errMax, dMax;
        if constexpr (FASTCTL) {
          ySel = fma(hh, f2d_int(incSel), ySel);  // the picked component's new state, FP64
          errMax = fabs(hh * f2d_int(estSel));
          dMax = fabs(epsRel * fabs(ySel) + epsAbs * f2d_int(sSel));
        } else {
          if constexpr (FAST) ySel += hh * (double)incSel;  // the picked component's new state, FP64
          errMax = fabs(hh * (double)estSel);
          dMax = fabs(epsRel * fabs(ySel) + epsAbs * (double)sSel);
        }
        ++count;
        double hNew = hh;
        bool decrease = false;
        // 0.9 rmax^(-1/5), floored at 0.2 (reached for rmax >= 4.5^5 exactly),
        // and 0.9 rmax^(-1/6) capped at 4.9 (reached below (0.9/4.9)^6).
        if constexpr (FASTCTL) {
          // The same decisions and values with the FP64 pipe used only for
          // arithmetic: the comparisons of the (non-negative) ratio with the
          // thresholds on the integer pipe, and the roots from the FP32
          // ratio of the pick as seed (ctrl_root09).
          const double q = errMax * rcp_seeded(dMax, dMaxF);
          const double rmax = (d_isnan(q) || dpos_lt(q, 2.2250738585072014e-308)) ? 2.2250738585072014e-308 : q;
          const float rF = __fdividef(errMaxF, dMaxF);
          if (dpos_gt(rmax, 1.1)) {
            double r = 0.2;
            if (!dpos_gt(rmax, 1845.28125)) {
              r = ctrl_root09<5>(rmax, rF);
              if (__double2hiint(r) < 0) r = 0.9 * inv_root<5>(rmax);
              if (dpos_lt(r, 0.2)) r = 0.2;
            }
            hNew = r * hh;
            decrease = true;
          } else if (dpos_lt(rmax, 0.5)) {
            double r = 4.9;
            if (!dpos_lt(rmax, 3.8394e-5)) {
              r = ctrl_root09<6>(rmax, rF);
              if (__double2hiint(r) < 0) r = 0.9 * inv_root<6>(rmax);
              if (dpos_gt(r, 4.9)) r = 4.9;
              if (dpos_lt(r, 1.0)) r = 1.0;
            }
            hNew = r * hh;
          }
        } else {
          const double rmax = dmax(fast_div(errMax, dMax), 2.2250738585072014e-308);  // floor DBL_MIN as cscal2.c
          if (rmax > 1.1) {
            double r = rmax > 1845.28125 ? 0.2 : 0.9 * inv_root<5>(rmax);
            if (r < 0.2) r = 0.2;
            hNew = r * hh;
            decrease = true;
          } else if (rmax < 0.5) {
            double r = rmax < 3.8394e-5 ? 4.9 : 0.9 * inv_root<6>(rmax);
            if (r > 4.9) r = 4.9;
            if (r < 1.0) r = 1.0;
            hNew = r * hh;
          }
        }
        if (decrease) {
          // A smaller step that still moves t: |hNew| < |hh| and
          // t_new + hNew != t_new.  In the FP32-rate forms the second test is
          // settled by exponents when |hNew| is at least two ulps of every
          // time involved (|t_new| <= 2 max(|t|, |t1|, |hh|)), else in FP64.
          bool smaller, moves;
          if constexpr (FASTCTL) {
            const long long hb = __double_as_longlong(hNew) & 0x7fffffffffffffffLL;
            const long long hhb = __double_as_longlong(hh) & 0x7fffffffffffffffLL;
            smaller = hb < hhb && hhb <= 0x7ff0000000000000LL;
            const int eh = (int)(hb >> 52);
            const int eT = 1 + max(max((__double2hiint(t) >> 20) & 0x7ff, (__double2hiint(t1) >> 20) & 0x7ff),
                                   (int)(hhb >> 52));
            if (smaller && eh >= 1 && eT < 0x7ff && eh >= eT - 51) {
              moves = true;
            } else {
              const double tNew = finalStep ? t1 : t + hh;
              moves = tNew + hNew != tNew;
            }
          } else {
            const double tNew = finalStep ? t1 : t + hh;
            smaller = fabs(hNew) < fabs(hh);
            moves = tNew + hNew != tNew;
          }
          if (smaller && moves) {
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
          if constexpr (FAST) {
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) {
              // (The conversion instructions here: the integer-pipe ones of
              // the controller cost more registers than they save in this
              // twelve-fold loop -- measured.)
              y[i] += hh * (double)x[i];
              yf[i] = (float)y[i];
            }
          } else {
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) y[i] = ynew[i];
          }
          t = finalStep ? t1 : t + hh;
          h = hNew;
          ++nAcc;
          bool reached;
          if constexpr (FASTCTL) {
            // !(t1 - t > 0 || t1 - t < 0): t1 - t is zero or NaN.
            reached = d_isnan(t) || d_isnan(t1) || d_key(t) == d_key(t1);
            dtLeft = t1 - t;
          } else {
            reached = !(t1 - t > 0.0 || t1 - t < 0.0);
          }
          if (reached) {
            post_step_any(y);
            finished = true;
            bool finite = true;
#pragma unroll
            for (int i = 0; i < GAL_NY; ++i) finite = finite && isfinite(y[i]);
            finalStatus = finite ? GAL_STATUS_SUCCESS : GAL_STATUS_NOT_FINITE;
          } else {
            needOut = true;
          }
        }
      }
      if (finished) finish(finalStatus);
    }
  }
  if (sd.stats) {
    // One atomic pair per warp for the network/table evaluation counts
    // (a form without the network counts its table evaluations when it
    // runs the table half of a surrogate form's split launch).
    for (int o = 16; o > 0; o >>= 1) {
      nNet += __shfl_down_sync(FULL, nNet, o);
      nTab += __shfl_down_sync(FULL, nTab, o);
    }
    if (lane == 0) {
      atomicAdd(&sd.stats[0], (unsigned long long)nNet);
      atomicAdd(&sd.stats[1], (unsigned long long)nTab);
    }
  }
}

// Everything one launch needs.
struct LaunchArgs {
  Globals G;
  Batch b;
  DeviceTables tables;
  SurrogateDev sd;
  ForestDev forest;
  size_t shm;
  int64_t blocks;
  cudaStream_t stream;
};

template <int THREADS, int MODE, bool FOREST = false, bool INTR = false, bool KMT = false>
cudaError_t launch_evolve(const LaunchArgs& a) {
  cudaError_t e = cudaFuncSetAttribute(evolve_kernel<THREADS, MODE, FOREST, INTR, KMT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.shm);
  if (e != cudaSuccess) return e;
  evolve_kernel<THREADS, MODE, FOREST, INTR, KMT><<<(unsigned)a.blocks, THREADS, a.shm, a.stream>>>(a.G, a.b, a.tables,
                                                                                                    a.sd, a.forest);
  return cudaGetLastError();
}

// The krumholz2009 disk rate is its own instantiation, 128 threads per block.
inline bool krumholz(const LaunchArgs& a) { return a.G.p.sf_disk_rate == GAL_SF_RATE_KRUMHOLZ2009; }

// Per-form launchers (evolve_plain.cu, evolve_surrogate.cu, evolve_fast.cu,
// evolve_fast_surrogate.cu); cudaErrorInvalidConfiguration for a block size
// the form is not built for.
cudaError_t evolve_launch_plain(int threads, const LaunchArgs& a);
// The plain form with interrupts (128 threads per block).
cudaError_t evolve_launch_plain_interrupt(const LaunchArgs& a);
cudaError_t evolve_launch_surrogate(int threads, const LaunchArgs& a);
cudaError_t evolve_launch_fast(int threads, const LaunchArgs& a);
cudaError_t evolve_launch_fast_surrogate(int threads, const LaunchArgs& a);
// Forest forms (evolve_forest_*.cu); cudaErrorInvalidConfiguration for a
// form or block size not built.
cudaError_t evolve_launch_forest(int mode, int threads, const LaunchArgs& a);

inline cudaError_t evolve_launch(int mode, int threads, const LaunchArgs& a) {
  switch (mode) {
    case MODE_PLAIN: return evolve_launch_plain(threads, a);
    case MODE_SURROGATE: return evolve_launch_surrogate(threads, a);
    case MODE_FAST: return evolve_launch_fast(threads, a);
    case MODE_FAST_SURROGATE: return evolve_launch_fast_surrogate(threads, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace gal
