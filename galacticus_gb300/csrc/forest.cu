// forest.cu -- whole-forest evolution on the GPU (include/galnode_forest.h).
//
// The tree evolver of the reference walks each tree node by node: a node is
// evolved from its own time to its parent's, the evolve calls being cut at
// the output times, and on reaching its parent it is promoted (the primary
// progenitor) or merged (merger_trees/evolver/standard.F90:762-1035,
// threaded.F90:418-840).  Here a forest is uploaded once -- its topology, the
// dependency counter of every node, and a segment table with the halo
// constants of every evolve call -- and each evolution is one CUDA graph:
// reset the counters and the leaf queue, then one persistent kernel
// (evolve_kernel with FOREST = true) in which the last progenitor of each
// node to finish merges the progenitors and carries on with the node.  No
// lane ever waits on another.
//
// The segment constants are computed on the host in FP64 without
// contraction (the file is compiled with -ffp-contract=off), from the
// analytic flat matter + Lambda time-redshift relation and the Bryan &
// Norman (1998) virial contrast relative to the mean density
// (structure_formation/virial_density_contrast/Bryan_Norman.F90:172-196).
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>
#include <algorithm>
#include <memory>
#include <type_traits>

#include "../../include/galnode_forest.h"
#include "context.h"

using namespace gal::host;

namespace {

constexpr double kMpc = 1.0e6 * 3.08567758135e16;
constexpr double kGyr = 1.0e9 * 3.15581497635456e7;
constexpr double kG = 6.673e-11 * 1.98892e30 / 1.0e6 / kMpc;  // km^2 s^-2 Mpc / Msun

struct HostCosmology {
  double om, ol, h0;
  __host__ __device__ double redshift(double t) const {
    const double hubbleGyr = h0 / (kMpc / 1.0e3 / kGyr);
    const double x = sinh(1.5 * hubbleGyr * sqrt(ol) * t);
    return 1.0 / pow(x / sqrt(ol / om), 2.0 / 3.0) - 1.0;
  }
  // The longest evolve call from a time at redshift z: min(relative / H,
  // absolute) (mergerTreeEvolveTimestepSimple, timesteps/simple.F90:124-161),
  // H the expansion rate of cosmologyFunctionsMatterLambda in 1/Gyr.
  __host__ __device__ double step_limit_z(double z, double relative, double absolute) const {
    if (!(relative > 0.0)) return absolute;
    const double hubbleGyr = h0 / (kMpc / 1.0e3 / kGyr);
    const double zp = 1.0 + z;
    const double rate = hubbleGyr * sqrt(om * zp * zp * zp + ol);
    return fmin(relative / rate, absolute);
  }
  __host__ __device__ void virial(double M, double z, double& r, double& v) const {
    const double zp = (1.0 + z) * (1.0 + z) * (1.0 + z);
    const double omz = om * zp / (om * zp + ol);
    const double x = omz - 1.0;
    const double contrast = (18.0 * M_PI * M_PI + 82.0 * x - 39.0 * x * x) / (x + 1.0);
    const double rhoMean = om * 3.0 * h0 * h0 / (8.0 * M_PI * kG) * zp;
    r = cbrt(3.0 * M / (4.0 * M_PI * contrast * rhoMean));
    v = sqrt(kG * M / r);
  }
};

template <class T>
cudaError_t upload(T** dst, const T* src, size_t n) {
  *dst = nullptr;
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)dst, n * sizeof(T));
  if (e == cudaSuccess) e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}
template <class T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  return upload(dst, src.data(), src.size());
}

// ---------------------------------------------------------------- segment table on the GPU
//
// The segment table (one row per evolve call) built on the device, one
// thread per node: a first kernel counts each node's evolve calls and
// snapshots, a scan turns the counts into offsets, and a second kernel
// writes each node's rows at its offsets.  The rules are those of the tree
// evolver (merger_trees/evolver/standard.F90:762-1035): a node evolves from
// its time to its parent's in calls that end at the first of the next
// output time, the parent's time and the mergerTreeEvolveTimestepSimple
// limit (merger_trees/evolve/timesteps/simple.F90:124-161); each call's
// halo mass follows the node's mass line and its virial scales are those of
// its start (a satellite's, those of its infall).
struct SegmentInputs {
  HostCosmology cos;
  double relative, absolute;
  int64_t n;
  int32_t nOut;
  const double* tOut;
  const double* time;
  const double* mass;
  const double* spin;
  const double* massIn;
  const int32_t* parent;
  const int32_t* childFirst;
  const int32_t* childCount;
  const int32_t* satHost;  // may be null
};

// Calls per node are bounded (a node past the bound is flagged, not looped).
constexpr int64_t kMaxCallsPerNode = 1 << 24;

__device__ __forceinline__ int32_t first_output_after(const SegmentInputs& in, double t) {
  int32_t lo = 0, hi = in.nOut;  // first k with tOut[k] > t
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (in.tOut[mid] > t)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// The output at the node's own time, if any (a non-root only if it has an
// interval to evolve).
__device__ __forceinline__ int32_t initial_output_dev(const SegmentInputs& in, int64_t i) {
  const int32_t par = in.parent[i];
  const double t0 = in.time[i];
  if (!(par < 0 || t0 < in.time[par])) return -1;
  int32_t lo = 0, hi = in.nOut;  // first k with tOut[k] >= t0
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (in.tOut[mid] >= t0)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo < in.nOut && in.tOut[lo] == t0 ? lo : -1;
}

// seg(a, b, k, z) for each evolve call of node i (k the output it ends at
// or -1, z the redshift at a or NaN); returns false past the bound.
template <class F>
__device__ __forceinline__ bool node_calls(const SegmentInputs& in, int64_t i, F&& seg) {
  const int32_t par = in.parent[i];
  const double t0 = in.time[i], t1 = par >= 0 ? in.time[par] : t0;
  double a = t0;
  int32_t k = first_output_after(in, t0);
  const bool relative = in.relative > 0.0;
  int64_t calls = 0;
  while (a < t1) {
    if (++calls > kMaxCallsPerNode) return false;
    const double z = relative ? in.cos.redshift(a) : __longlong_as_double(0x7ff8000000000000ll);
    const double limit = a + in.cos.step_limit_z(z, in.relative, in.absolute);
    const bool atOutput = k < in.nOut && in.tOut[k] < t1 && !(limit < in.tOut[k]);
    const double b = atOutput ? in.tOut[k] : fmin(limit, t1);
    seg(a, b, atOutput ? k : -1, z);
    if (atOutput) ++k;
    a = b;
  }
  return true;
}

__global__ void count_calls_kernel(SegmentInputs in, int32_t* segCount, int32_t* snapCount, int* flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < in.n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t ns = 0, nsnap = initial_output_dev(in, i) >= 0 ? 1 : 0;
    const bool ok = node_calls(in, i, [&](double, double, int32_t k, double) {
      ++ns;
      if (k >= 0) ++nsnap;
    });
    if (!ok || ns > INT32_MAX) {
      atomicExch(flag, 1);
      ns = nsnap = 0;
    }
    segCount[i] = (int32_t)ns;
    snapCount[i] = (int32_t)nsnap;
  }
}

// Exclusive scan of two count arrays, 1,024 entries per block; the block
// totals are scanned on the host and added by add_offsets_kernel.
__global__ void __launch_bounds__(1024) scan_blocks_kernel(const int32_t* a, const int32_t* b, int64_t n, int64_t* oa,
                                                           int64_t* ob, int64_t* totals) {
  __shared__ int64_t sa[1024], sb[1024];
  const int64_t i = blockIdx.x * 1024ll + threadIdx.x;
  const int64_t va = i < n ? a[i] : 0, vb = i < n ? b[i] : 0;
  sa[threadIdx.x] = va;
  sb[threadIdx.x] = vb;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int64_t ta = threadIdx.x >= off ? sa[threadIdx.x - off] : 0;
    const int64_t tb = threadIdx.x >= off ? sb[threadIdx.x - off] : 0;
    __syncthreads();
    sa[threadIdx.x] += ta;
    sb[threadIdx.x] += tb;
    __syncthreads();
  }
  if (i < n) {
    oa[i] = sa[threadIdx.x] - va;
    ob[i] = sb[threadIdx.x] - vb;
  }
  if (threadIdx.x == 1023) {
    totals[2 * blockIdx.x] = sa[1023];
    totals[2 * blockIdx.x + 1] = sb[1023];
  }
}

__global__ void add_offsets_kernel(int64_t* oa, int64_t* ob, int64_t n, const int64_t* blockOffsets) {
  const int64_t i = blockIdx.x * 1024ll + threadIdx.x;
  if (i < n) {
    oa[i] += blockOffsets[2 * blockIdx.x];
    ob[i] += blockOffsets[2 * blockIdx.x + 1];
  }
}

struct SegmentOutputs {
  int64_t nSeg, nSnap;
  const int64_t* segBase;
  const int64_t* snapBase;
  const int32_t* segCount;
  int32_t* segFirst;
  int32_t* snapInitial;
  int32_t* snapNode;
  int32_t* snapOutput;
  double* segParam;  // [GAL_NP][nSeg]
  double* segT0;
  double* segT1;
  int32_t* segSnap;
};

__global__ void fill_calls_kernel(SegmentInputs in, SegmentOutputs out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < in.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t par = in.parent[i];
    const double t0 = in.time[i], t1 = par >= 0 ? in.time[par] : t0;
    const bool satellite = in.satHost && in.satHost[i] >= 0;
    // The primary progenitor grows by its parent's unresolved mass (the
    // parent's mass beyond its progenitors' and the satellites falling in);
    // other progenitors and satellites keep theirs and accrete nothing.
    double massEnd = in.mass[i], accretion = 0.0;
    if (par >= 0 && in.childFirst[par] == (int32_t)i && t1 > t0 && !satellite) {
      double brought = in.massIn[par];
      for (int32_t c = 0; c < in.childCount[par]; ++c) {
        const int32_t s = in.childFirst[par] + c;
        if (!(in.satHost && in.satHost[s] >= 0)) brought += in.mass[s];
      }
      accretion = fmax(in.mass[par] - brought, 0.0) / (t1 - t0);
      massEnd = in.mass[i] + accretion * (t1 - t0);
    }
    // A satellite's virial scales are those of its infall time.
    const double zFrozen = satellite ? in.cos.redshift(t0) : 0.0;
    int64_t slot = out.snapBase[i];
    const int64_t slotEnd = i + 1 < in.n ? out.snapBase[i + 1] : out.nSnap;
    const int32_t k0 = initial_output_dev(in, i);
    out.snapInitial[i] = -1;
    if (k0 >= 0 && slot < slotEnd) {
      out.snapInitial[i] = (int32_t)slot;
      out.snapNode[slot] = (int32_t)i;
      out.snapOutput[slot] = k0;
      ++slot;
    }
    int64_t sg = out.segBase[i];
    const int64_t sgEnd = sg + out.segCount[i];
    out.segFirst[i] = (int32_t)sg;
    const double m0 = in.mass[i], sp = in.spin[i];
    node_calls(in, i, [&](double a, double b, int32_t k, double z) {
      if (sg >= sgEnd) return;  // (the count pass made room for exactly these)
      const double M = m0 + (massEnd - m0) * (a - t0) / (t1 - t0);
      double r, v;
      in.cos.virial(M, satellite ? zFrozen : (z == z ? z : in.cos.redshift(a)), r, v);
      out.segParam[(size_t)GAL_P_MASS * out.nSeg + sg] = M;
      out.segParam[(size_t)GAL_P_MASS_RATE * out.nSeg + sg] = accretion;
      out.segParam[(size_t)GAL_P_RADIUS_VIRIAL * out.nSeg + sg] = r;
      out.segParam[(size_t)GAL_P_VELOCITY_VIRIAL * out.nSeg + sg] = v;
      out.segParam[(size_t)GAL_P_SPIN * out.nSeg + sg] = sp;
      out.segT0[sg] = a;
      out.segT1[sg] = b;
      if (k >= 0 && slot < slotEnd) {
        out.segSnap[sg] = (int32_t)slot;
        out.snapNode[slot] = (int32_t)i;
        out.snapOutput[slot] = k;
        ++slot;
      } else {
        out.segSnap[sg] = -1;
      }
      ++sg;
    });
  }
}

}  // namespace

struct gal_forest_dev {
  int64_t n = 0, nLeaves = 0, nSeg = 0, nSnap = 0;
  // device arrays
  int32_t *dLeaves = nullptr, *dParent = nullptr, *dChildFirst = nullptr, *dChildCount = nullptr;
  int32_t *dPending = nullptr, *dPending0 = nullptr, *dSegFirst = nullptr, *dSegCount = nullptr, *dSnapInitial = nullptr;
  int32_t* dSegSnap = nullptr;
  double *dSegParam = nullptr, *dSegT0 = nullptr, *dSegT1 = nullptr;
  double *dState0 = nullptr, *dState = nullptr, *dStepOut = nullptr, *dSnap = nullptr;
  int32_t* dStatus = nullptr;
  uint32_t* dCounters = nullptr;
  unsigned long long* dHead = nullptr;
  // snapshot labels: node and output index of each slot
  int32_t *dSnapNode = nullptr, *dSnapOutput = nullptr;
  // the captured evolution and the form/shape it was captured for
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graphMode = -1, graphThreads = 0, graphBlocks = 0;
  cudaEvent_t done = nullptr;
};

namespace {

void release(gal_forest_dev* f) {
  if (!f) return;
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  if (f->done) cudaEventDestroy(f->done);
  void* ptrs[] = {f->dLeaves, f->dParent, f->dChildFirst, f->dChildCount, f->dPending, f->dPending0, f->dSegFirst,
                  f->dSegCount, f->dSnapInitial, f->dSegSnap, f->dSegParam, f->dSegT0, f->dSegT1, f->dState0,
                  f->dState, f->dStepOut, f->dSnap, f->dStatus, f->dCounters, f->dHead, f->dSnapNode, f->dSnapOutput};
  for (void* p : ptrs) cudaFree(p);
  delete f;
}

// The launch arguments of one forest evolution in the context's current form and shape.
LaunchArgs forest_args(gal_ctx* ctx, gal_forest_dev* f, int mode, int threads, int blocksPerSm) {
  LaunchArgs a{};
  a.G = ctx->globals;
  a.tables = ctx_tables(ctx);
  if (mode & MODE_SURROGATE)
    a.sd = SurrogateDev{ctx->dSurrSmall, ctx->dSurrPlanes, ctx->dSurrMap, ctx->surrInfo, ctx->dSurrStats};
  ForestDev& F = a.forest;
  F.n = f->n;
  F.nLeaves = f->nLeaves;
  F.leaves = f->dLeaves;
  F.parent = f->dParent;
  F.childFirst = f->dChildFirst;
  F.childCount = f->dChildCount;
  F.pending = f->dPending;
  F.segFirst = f->dSegFirst;
  F.segCount = f->dSegCount;
  F.snapInitial = f->dSnapInitial;
  F.nSeg = f->nSeg;
  F.segParam = f->dSegParam;
  F.segT0 = f->dSegT0;
  F.segT1 = f->dSegT1;
  F.segSnap = f->dSegSnap;
  F.state0 = f->dState0;
  F.state = f->dState;
  F.stepOut = f->dStepOut;
  F.nSnap = f->nSnap;
  F.snapshots = f->dSnap;
  F.status = f->dStatus;
  F.counters = f->dCounters;
  F.head = f->dHead;
  a.shm = ctx_shared_bytes(ctx, mode);
  const int64_t lanes = (f->nLeaves + 31) / 32 * 32;
  a.blocks = std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->smCount * blocksPerSm, (lanes + threads - 1) / threads));
  a.stream = ctx->stream;
  return a;
}

// (Re)capture the evolution graph when the form or the launch shape changed.
int ensure_graph(gal_ctx* ctx, gal_forest_dev* f) {
  const int mode = ctx_mode(ctx);
  int threads, blocksPerSm;
  effective_shape(ctx, mode, threads, blocksPerSm);
  if (f->exec && f->graphMode == mode && f->graphThreads == threads && f->graphBlocks == blocksPerSm) return GAL_OK;
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  f->exec = nullptr;
  f->graph = nullptr;
  const LaunchArgs a = forest_args(ctx, f, mode, threads, blocksPerSm);
  cudaStream_t st = ctx->stream;
  // The kernel attribute (dynamic shared memory) is set by an empty-forest
  // launch outside the capture: with no leaves every block returns at once.
  LaunchArgs warm = a;
  warm.forest.nLeaves = 0;
  warm.blocks = 1;
  cudaError_t e = cudaMemsetAsync(f->dHead, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = evolve_launch_forest(mode, threads, warm);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "forest kernel set-up failed: %s", cudaGetErrorString(e));
  e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaError_t e1 = cudaMemcpyAsync(f->dPending, f->dPending0, f->n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    if (e1 == cudaSuccess) e1 = cudaMemsetAsync(f->dHead, 0, sizeof(unsigned long long), st);
    if (e1 == cudaSuccess) e1 = evolve_launch_forest(mode, threads, a);
    cudaError_t e2 = cudaStreamEndCapture(st, &f->graph);
    e = e1 != cudaSuccess ? e1 : e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&f->exec, f->graph, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, GAL_ERR_CUDA, "forest graph capture failed: %s", cudaGetErrorString(e));
  }
  f->graphMode = mode;
  f->graphThreads = threads;
  f->graphBlocks = blocksPerSm;
  return GAL_OK;
}

}  // namespace

extern "C" {

int gal_gpu_forest_create(gal_ctx* ctx, int64_t n, const int32_t* parent, const int32_t* childFirst,
                          const int32_t* childCount, const double* time, const double* mass, const double* spin,
                          const int32_t* satHost, const double* state0, int32_t nOut, const double* tOut,
                          gal_forest_dev** out) {
  if (!out) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_create: out is NULL%s");
  *out = nullptr;
  if (!ctx) return fail(nullptr, GAL_ERR_ARGUMENT, "gal_gpu_forest_create: NULL context%s");
  if (n < 1 || n > (int64_t)INT32_MAX || !parent || !childFirst || !childCount || !time || !mass || !spin || !state0 ||
      nOut < 0 || (nOut > 0 && !tOut))
    return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_create: bad arguments%s");
  for (int32_t k = 1; k < nOut; ++k)
    if (!(tOut[k] > tOut[k - 1])) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_create: output times must increase%s");
  // Topology checks (parents in range and later, progenitors contiguous,
  // satellite hosts at the infall time), parallel over nodes; the first
  // failing node is reported.
  auto node_error = [&](int64_t i) -> int {
    const int32_t p = parent[i];
    if (p >= n || p < -1 || (p >= 0 && !(time[p] > time[i])) || childCount[i] < 0 ||
        (childCount[i] > 0 && (childFirst[i] < 0 || (int64_t)childFirst[i] + childCount[i] > n)))
      return 1;
    for (int32_t c = 0; c < childCount[i]; ++c)
      if (parent[childFirst[i] + c] != (int32_t)i) return 2;
    if (p >= 0 && !(childFirst[p] <= i && i < (int64_t)childFirst[p] + childCount[p])) return 2;
    if (satHost && (satHost[i] < -1 || satHost[i] >= n || (satHost[i] >= 0 && time[satHost[i]] != time[i]))) return 3;
    return 0;
  };
  int64_t firstBad = n;
#pragma omp parallel for schedule(static) reduction(min : firstBad)
  for (int64_t i = 0; i < n; ++i)
    if (node_error(i) && i < firstBad) firstBad = i;
  if (firstBad < n) {
    const int code = node_error(firstBad);
    return fail(ctx, GAL_ERR_ARGUMENT,
                code == 1   ? "gal_gpu_forest_create: inconsistent forest topology%s"
                : code == 2 ? "gal_gpu_forest_create: progenitors must be contiguous%s"
                            : "gal_gpu_forest_create: a satellite's host must be a node of its infall time%s");
  }
  // The mass each node gains at its own time from the satellites that fall
  // into it (their halos join its halo there).
  std::vector<double> massIn((size_t)n, 0.0);
  if (satHost)
    for (int64_t i = 0; i < n; ++i)
      if (satHost[i] >= 0) massIn[(size_t)satHost[i]] += mass[i];
  const gal_params& p = ctx->params;
  const HostCosmology cos{p.omega_matter, p.omega_dark_energy, p.hubble_constant};
  gal_forest_dev* f = new (std::nothrow) gal_forest_dev();
  if (!f) return fail(ctx, GAL_ERR_ARGUMENT, "out of host memory%s");
  f->n = n;
  // The segment table on the GPU: the node arrays the kernels read, the
  // counts and their offsets (freed at the end), then the table itself.
  cudaStream_t st = ctx->stream;
  double *dTime = nullptr, *dMass = nullptr, *dSpin = nullptr, *dMassIn = nullptr, *dTOut = nullptr;
  int32_t *dSatHost = nullptr, *dSnapCount = nullptr;
  int64_t *dSegBase = nullptr, *dSnapBase = nullptr, *dTotals = nullptr;
  int* dFlag = nullptr;
  auto cleanup = [&]() {
    void* tmp[] = {dTime, dMass, dSpin, dMassIn, dTOut, dSatHost, dSnapCount, dSegBase, dSnapBase, dTotals, dFlag};
    for (void* q : tmp) cudaFree(q);
  };
  auto put = [&](auto** dst, const auto* src, size_t count) {
    using T = std::remove_const_t<std::remove_pointer_t<decltype(src)>>;
    cudaError_t r = cudaMalloc((void**)dst, std::max<size_t>(count, 1) * sizeof(T));
    if (r == cudaSuccess && count) r = cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, st);
    return r;
  };
  auto give_up = [&](cudaError_t err) {
    cudaGetLastError();
    cleanup();
    release(f);
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_create: segment table on the GPU failed: %s", cudaGetErrorString(err));
  };
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = put(&f->dParent, parent, (size_t)n);
  if (e == cudaSuccess) e = put(&f->dChildFirst, childFirst, (size_t)n);
  if (e == cudaSuccess) e = put(&f->dChildCount, childCount, (size_t)n);
  if (e == cudaSuccess) e = put(&dTime, time, (size_t)n);
  if (e == cudaSuccess) e = put(&dMass, mass, (size_t)n);
  if (e == cudaSuccess) e = put(&dSpin, spin, (size_t)n);
  if (e == cudaSuccess) e = put(&dMassIn, massIn.data(), (size_t)n);
  if (e == cudaSuccess) e = put(&dTOut, tOut, (size_t)nOut);
  if (e == cudaSuccess && satHost) e = put(&dSatHost, satHost, (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&f->dSegCount, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&dSnapCount, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&dSegBase, (size_t)n * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&dSnapBase, (size_t)n * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&dFlag, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(dFlag, 0, sizeof(int), st);
  if (e != cudaSuccess) return give_up(e);
  const SegmentInputs in{cos,   p.timestep_relative, p.timestep_absolute, n,       nOut,           dTOut,
                         dTime, dMass,               dSpin,              dMassIn, f->dParent,     f->dChildFirst,
                         f->dChildCount, dSatHost};
  const int threads = 256;
  const int grid = (int)std::min<int64_t>((n + threads - 1) / threads, (int64_t)std::max(ctx->smCount, 1) * 16);
  count_calls_kernel<<<grid, threads, 0, st>>>(in, f->dSegCount, dSnapCount, dFlag);
  const int64_t nb = (n + 1023) / 1024;
  if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaMalloc(&dTotals, (size_t)2 * nb * sizeof(int64_t))) != cudaSuccess)
    return give_up(e);
  scan_blocks_kernel<<<(unsigned)nb, 1024, 0, st>>>(f->dSegCount, dSnapCount, n, dSegBase, dSnapBase, dTotals);
  std::vector<int64_t> totals((size_t)2 * nb);
  int flag = 0;
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(totals.data(), dTotals, totals.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&flag, dFlag, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return give_up(e);
  if (flag) {
    cleanup();
    release(f);
    return fail(ctx, GAL_ERR_TOO_LARGE, "gal_gpu_forest_create: a node needs more than 2^24 evolve calls%s");
  }
  int64_t nSeg = 0, nSnap = 0;
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t ts = totals[(size_t)(2 * b)], tn = totals[(size_t)(2 * b + 1)];
    totals[(size_t)(2 * b)] = nSeg;
    totals[(size_t)(2 * b + 1)] = nSnap;
    nSeg += ts;
    nSnap += tn;
  }
  if (nSeg > (int64_t)INT32_MAX || nSnap > (int64_t)INT32_MAX) {
    cleanup();
    release(f);
    return fail(ctx, GAL_ERR_TOO_LARGE, "gal_gpu_forest_create: more than 2^31 evolve calls or snapshots%s");
  }
  if ((e = cudaMemcpyAsync(dTotals, totals.data(), totals.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return give_up(e);
  add_offsets_kernel<<<(unsigned)nb, 1024, 0, st>>>(dSegBase, dSnapBase, n, dTotals);
  if ((e = cudaGetLastError()) != cudaSuccess) return give_up(e);
  if ((e = cudaMalloc(&f->dSegFirst, (size_t)n * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSnapInitial, (size_t)n * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSnapNode, (size_t)std::max<int64_t>(nSnap, 1) * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSnapOutput, (size_t)std::max<int64_t>(nSnap, 1) * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSegParam, (size_t)GAL_NP * std::max<int64_t>(nSeg, 1) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSegT0, (size_t)std::max<int64_t>(nSeg, 1) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSegT1, (size_t)std::max<int64_t>(nSeg, 1) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&f->dSegSnap, (size_t)std::max<int64_t>(nSeg, 1) * sizeof(int32_t))) != cudaSuccess)
    return give_up(e);
  const SegmentOutputs outs{nSeg,          nSnap,         dSegBase,        dSnapBase,       f->dSegCount,
                            f->dSegFirst,  f->dSnapInitial, f->dSnapNode,  f->dSnapOutput,  f->dSegParam,
                            f->dSegT0,     f->dSegT1,     f->dSegSnap};
  fill_calls_kernel<<<grid, threads, 0, st>>>(in, outs);
  if ((e = cudaGetLastError()) != cudaSuccess) return give_up(e);
  ctx->launches += 4;
  std::vector<int32_t> leaves;
  for (int64_t i = 0; i < n; ++i)
    if (childCount[i] == 0) leaves.push_back((int32_t)i);
  // Longest chains first: a leaf's chain to its root is the sequence of
  // nodes that can only run one after another, so leaves are queued by the
  // number of their ancestors, largest first (ties in index order).  The
  // deep branches of the largest trees then start at once instead of
  // setting the end of the evolution.  Depths by a walk down from each
  // root, the order by a stable counting sort.
  {
    std::vector<int32_t> depth((size_t)n, 0), roots;
    for (int64_t i = 0; i < n; ++i)
      if (parent[i] < 0) roots.push_back((int32_t)i);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t r = 0; r < (int64_t)roots.size(); ++r) {
      std::vector<int32_t> stack{roots[(size_t)r]};
      while (!stack.empty()) {
        const int32_t i = stack.back();
        stack.pop_back();
        for (int32_t c = 0; c < childCount[i]; ++c) {
          depth[(size_t)(childFirst[i] + c)] = depth[(size_t)i] + 1;
          stack.push_back(childFirst[i] + c);
        }
      }
    }
    int32_t maxDepth = 0;
    for (int32_t l : leaves) maxDepth = std::max(maxDepth, depth[(size_t)l]);
    std::vector<int64_t> at((size_t)maxDepth + 2, 0);
    for (int32_t l : leaves) ++at[(size_t)(maxDepth - depth[(size_t)l]) + 1];
    for (size_t d = 1; d < at.size(); ++d) at[d] += at[d - 1];
    std::vector<int32_t> sorted(leaves.size());
    for (int32_t l : leaves) sorted[(size_t)at[(size_t)(maxDepth - depth[(size_t)l])]++] = l;
    leaves.swap(sorted);
  }
  f->nLeaves = (int64_t)leaves.size();
  f->nSeg = nSeg;
  f->nSnap = nSnap;
  if (e == cudaSuccess) e = put(&f->dLeaves, leaves.data(), leaves.size());
  if (e == cudaSuccess) e = cudaMalloc(&f->dPending0, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&f->dPending, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(f->dPending0, f->dChildCount, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(f->dPending, f->dChildCount, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = put(&f->dState0, state0, (size_t)GAL_NY * n);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e == cudaSuccess) e = cudaMalloc(&f->dState, (size_t)GAL_NY * n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&f->dStepOut, (size_t)n * sizeof(double));
  if (e == cudaSuccess && f->nSnap > 0) e = cudaMalloc(&f->dSnap, (size_t)GAL_NY * f->nSnap * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&f->dStatus, (size_t)n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&f->dCounters, (size_t)3 * n * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&f->dHead, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaGetLastError();
    release(f);
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_create: device allocation or upload failed: %s", cudaGetErrorString(e));
  }
  *out = f;
  return GAL_OK;
}

int gal_gpu_forest_evolve(gal_ctx* ctx, gal_forest_dev* f) {
  if (!ctx || !f) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_evolve: NULL argument%s");
  if (ctx_mode(ctx) == MODE_SURROGATE)
    return fail(ctx, GAL_ERR_ARGUMENT,
                "gal_gpu_forest_evolve: forests are built for the FP64 form, the FP32-rate form and the FP32-rate "
                "form with the surrogate; with a surrogate installed, set GAL_RATES_FP32%s");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "CUDA error: %s", cudaGetErrorString(e));
  int rc = ensure_graph(ctx, f);
  if (rc) return rc;
  e = cudaGraphLaunch(f->exec, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(f->done, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "forest graph launch failed: %s", cudaGetErrorString(e));
  ++ctx->launches;
  return GAL_OK;
}

int gal_gpu_forest_sync(gal_ctx* ctx, gal_forest_dev* f) {
  if (!ctx || !f) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_sync: NULL argument%s");
  const cudaError_t e = cudaEventSynchronize(f->done);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "forest evolution failed: %s", cudaGetErrorString(e));
  return GAL_OK;
}

int64_t gal_gpu_forest_snapshot_count(const gal_forest_dev* f) { return f ? f->nSnap : -1; }

int gal_gpu_forest_results(gal_ctx* ctx, gal_forest_dev* f, double* state, int32_t* status, uint32_t* counters,
                           double* snapshot, int32_t* snapNode, int32_t* snapOutput) {
  if (!ctx || !f) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_results: NULL argument%s");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  const int64_t n = f->n;
  if (e == cudaSuccess && state) e = cudaMemcpy(state, f->dState, (size_t)GAL_NY * n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && status) e = cudaMemcpy(status, f->dStatus, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && counters)
    e = cudaMemcpy(counters, f->dCounters, (size_t)3 * n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && snapshot && f->nSnap > 0)
    e = cudaMemcpy(snapshot, f->dSnap, (size_t)GAL_NY * f->nSnap * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && snapNode && f->nSnap > 0)
    e = cudaMemcpy(snapNode, f->dSnapNode, (size_t)f->nSnap * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && snapOutput && f->nSnap > 0)
    e = cudaMemcpy(snapOutput, f->dSnapOutput, (size_t)f->nSnap * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_results: %s", cudaGetErrorString(e));
  return GAL_OK;
}

int64_t gal_gpu_forest_accepted_steps(gal_ctx* ctx, gal_forest_dev* f) {
  if (!ctx || !f) return -1;
  std::vector<uint32_t> acc((size_t)f->n);
  if (cudaSetDevice(ctx->device) != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
      cudaMemcpy(acc.data(), f->dCounters, acc.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  int64_t total = 0;
  for (uint32_t a : acc) total += a;
  return total;
}

int gal_gpu_forest_autotune(gal_ctx* ctx, gal_forest_dev* f, int32_t repeats, double* timesMs) {
  if (!ctx || !f || repeats < 1) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_autotune: bad arguments%s");
  static const int shapes[6][2] = {{64, 1}, {128, 1}, {128, 2}, {256, 1}, {256, 2}, {512, 1}};
  const int mode = ctx_mode(ctx);
  const int keepThreads = ctx->threads, keepBlocks = ctx->blocksPerSm;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_autotune: event creation failed%s");
  double best = 1e300;
  int bestI = -1;
  int rc = GAL_OK;
  for (int i = 0; i < 6 && rc == GAL_OK; ++i) {
    if (timesMs) timesMs[i] = -1.0;
    const int t = shapes[i][0], b = shapes[i][1];
    if (!mode_has_threads(mode, t) || (size_t)b * ctx_shared_bytes(ctx, mode) > 228 * 1024) continue;
    ctx->threads = t;
    ctx->blocksPerSm = b;
    rc = gal_gpu_forest_evolve(ctx, f);  // warm-up (and graph capture)
    if (rc) break;
    cudaEventRecord(e0, ctx->stream);
    for (int r = 0; r < repeats && rc == GAL_OK; ++r) rc = gal_gpu_forest_evolve(ctx, f);
    cudaEventRecord(e1, ctx->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_autotune: evolution failed%s");
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double mean = ms / repeats;
    if (timesMs) timesMs[i] = mean;
    if (mean < best) {
      best = mean;
      bestI = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (bestI >= 0) {
    ctx->threads = shapes[bestI][0];
    ctx->blocksPerSm = shapes[bestI][1];
  } else {
    ctx->threads = keepThreads;
    ctx->blocksPerSm = keepBlocks;
  }
  return rc;
}

void gal_gpu_forest_free(gal_forest_dev* f) {
  if (!f) return;
  if (f->done) cudaEventSynchronize(f->done);  // the last evolution has finished with the arrays
  release(f);
}

}  // extern "C"
