// trees_gpu.cu -- the Cole et al. (2000) tree builder's branching on the GPU
// (gal_gpu_forest_build, include/galnode_forest.h): the walk of
// Builder::grow in trees.cpp (merger_trees/construct/builder/Cole2000/
// _class.F90:360-913 with the Parkinson, Cole & Helly (2008) rates of
// merger_trees/branching_probability/Parkinson_Cole_Helly.F90:265-634),
// one branch per thread, with keyed random streams (trees_internal.h).
//
// Work is grown in generations.  A thread takes a node, walks its branch
// back in w until it splits or ends, and on a split numbers the two
// progenitors, hands the smaller to the next generation and walks on along
// the larger: a main branch stays in one thread from the root to its
// earliest halo, and the number of generations is the largest number of
// times a path from a root turns into a smaller progenitor (tens), not the
// number of splits along it.  Nodes are numbered by an atomic counter, so
// their device order depends on the schedule; the host renumbers each tree
// into the host builder's order, which the keyed streams make a function
// of the tree alone.
//
// One lane's walk is the critical path: the main branch of a 1e14 Msun
// tree at a 1e8 Msun resolution is ~1e5 dependent steps, and GB300 issues
// FP64 at one warp instruction per ~64 cycles per SM sub-partition, so the
// host builder's FP64 step (two logarithms, three exponentials, a power, a
// square root and three divisions, ~200 FP64 instructions) would take
// seconds in one lane.  The walk here evaluates the rates in FP32 from FP32
// copies of the tables in shared memory, with its own logarithm and
// exponential (ln_pos, exp_f: Cody & Waite (1980) argument reduction and
// the series of atanh and exp, with explicit fmaf), compares positive
// doubles as integers, and keeps FP64 only where it accumulates: the mass
// and w along the branch.  Every operation is IEEE-defined (fmaf, FP32
// division and square root, exact float<->double conversions), and the file
// is compiled without FMA contraction, so the oracle's restatement on the
// CPU gives the same trees bit for bit.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "../../include/galnode_forest.h"
#include "context.h"
#include "galnode_fastmath.cuh"
#include "trees_internal.h"

namespace gal {
namespace trees {
namespace {

// ln 2 split for the Cody & Waite reduction: kLn2Hi = 355/512 (exact in 9
// bits, so e kLn2Hi is exact for |e| < 2^15), kLn2Lo = ln 2 - kLn2Hi; the
// same split of ln 2 / 32 for the exponential.
constexpr float kLn2Hi = 0.693359375f;
constexpr float kLn2Lo = -2.12194440e-4f;
constexpr float kLn2By32Hi = 0.0216674805f;   // 355/16384
constexpr float kLn2By32Lo = -6.63107626e-6f;  // (ln 2 - 355/512)/32
constexpr float k32ByLn2 = 46.1662445f;

// The walk's function tables (shared memory): for the logarithm, ln c_j and
// 1/c_j at c_j = 1 + (j + 1/2)/128; for the exponential, 2^(j/32).
struct FnTables {
  const float* lnc;
  const float* invc;
  const float* pow2;
};

// ln x in FP32 for a positive normal double x, after Tang (1990, ACM TOMS
// 16, 378): x = 2^e f, f in [1, 2) (its top 23 mantissa bits, truncated),
// c_j the centre of f's 1/128 interval, r = f/c_j - 1 (|r| < 2^-8), and
// ln x = e ln 2 + ln c_j + ln(1 + r), ln(1 + r) = r - r^2/2 + r^3/3
// (truncation < 1e-10).
__device__ __forceinline__ float ln_pos(double x, const FnTables& t) {
  const long long b = __double_as_longlong(x);
  const int e = (int)(b >> 52) - 1023;
  const int j = (int)((b >> 45) & 127);
  const float f = __int_as_float(0x3f800000 | (int)((b >> 29) & 0x7fffff));
  const float r = fmaf(f, t.invc[j], -1.0f);
  const float p = fmaf(fmaf(r, 1.0f / 3.0f, -0.5f), r * r, r);
  const float ef = (float)e;
  return fmaf(ef, kLn2Hi, fmaf(ef, kLn2Lo, t.lnc[j] + p));
}

// e^x in FP32 for |x| < 80, after Tang (1989, ACM TOMS 15, 144): x =
// (32 k + j) ln 2/32 + r, |r| <= ln 2/64, e^x = 2^k 2^(j/32) e^r with
// e^r = 1 + r + r^2/2 + r^3/6 (truncation < 6e-10).
__device__ __forceinline__ float exp_f(float x, const FnTables& t) {
  x = fminf(fmaxf(x, -80.0f), 80.0f);
  const float n = rintf(x * k32ByLn2);
  const int ni = (int)n;
  const int j = ni & 31;
  const int k = ni >> 5;
  const float r = fmaf(-n, kLn2By32Lo, fmaf(-n, kLn2By32Hi, x));
  const float p = fmaf(fmaf(fmaf(r, 1.0f / 6.0f, 0.5f), r, 1.0f), r, 1.0f);
  return (t.pow2[j] * p) * __int_as_float((k + 127) << 23);
}

struct DevTables {
  // FP32 copies of ln sigma, R and F and the function tables (staged in
  // shared memory), the FP64 split tables (read on splits only) and the
  // walk's constants.
  const float* fn;  // [128 ln c_j][128 1/c_j][32 2^(j/32)]
  const float* lnSigma;
  const float* R;
  const float* F;
  const float* lnqA;  // per rate row: ln q of its first point and the spacing in ln q
  const float* lnqD;
  const float* cdf;   // [rows][kNq]
  int32_t nSigma, rows;
  float sigLnMin, sigInv, halfShift, rtLnMin, rtInv, gamma2, accuracyFirst, accuracySecond;
  double mRes, mRes2, wMax;
};

struct DevNodes {
  double* mass;
  double* w;
  int32_t* childFirst;
  int32_t* childCount;
  uint64_t* key;
  int64_t capacity;
};

// Counters of one growth: [0] nodes numbered (may run past the capacity),
// [1] length of the next generation, [2] capacity overflow flag.
enum { kNodes = 0, kNext = 1, kOverflow = 2, kCounters = 4 };

// Positive doubles order as their bit patterns (signed 64-bit integers):
// the walk's comparisons of masses and w run on the integer pipe.
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }

__device__ __forceinline__ float interp(const float* t, int n, float x) {
  x = fminf(fmaxf(x, 0.0f), (float)(n - 1));
  const int i = min((int)x, n - 2);
  const float f = x - (float)i;
  return t[i] + f * (t[i + 1] - t[i]);
}

// Number c consecutive new nodes; -1 (and the overflow flag) when the
// arrays are full.
__device__ __forceinline__ int64_t take_nodes(unsigned long long* counters, int64_t capacity, int c) {
  const unsigned long long base = atomicAdd(&counters[kNodes], (unsigned long long)c);
  if ((int64_t)base + c > capacity) {
    atomicExch(reinterpret_cast<unsigned int*>(&counters[kOverflow]), 1u);
    return -1;
  }
  return (int64_t)base;
}

__device__ __forceinline__ void put_node(const DevNodes& nd, int64_t i, double mass, double w, uint64_t key) {
  nd.mass[i] = mass;
  nd.w[i] = w;
  nd.childFirst[i] = 0;
  nd.childCount[i] = 0;
  nd.key[i] = key;
}

__global__ void __launch_bounds__(128) grow_kernel(DevTables tab, DevNodes nd, const int32_t* __restrict__ frontier,
                                                   int32_t nFrontier, int32_t* __restrict__ next,
                                                   unsigned long long* counters) {
  extern __shared__ float smem[];
  float* fn = smem;
  float* lnSigma = fn + kFnTable;
  float* Rt = lnSigma + tab.nSigma;
  float* Ft = Rt + tab.rows;
  float* qA = Ft + tab.rows;
  float* qD = qA + tab.rows;
  for (int k = threadIdx.x; k < kFnTable; k += blockDim.x) fn[k] = tab.fn[k];
  for (int k = threadIdx.x; k < tab.nSigma; k += blockDim.x) lnSigma[k] = tab.lnSigma[k];
  for (int k = threadIdx.x; k < tab.rows; k += blockDim.x) {
    Rt[k] = tab.R[k];
    Ft[k] = tab.F[k];
    qA[k] = tab.lnqA[k];
    qD[k] = tab.lnqD[k];
  }
  __syncthreads();
  const FnTables ft{fn, fn + 128, fn + 256};
  const int32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nFrontier) return;
  int64_t i = frontier[slot];
  const long long bMax = bits(tab.wMax), bRes = bits(tab.mRes), bRes2 = bits(tab.mRes2);
  while (i >= 0) {
    const uint64_t key = nd.key[i];
    double m = nd.mass[i], w = nd.w[i];
    const double w0 = w;
    double mPrev = m, wPrev = w;
    uint32_t k = 0;  // draws taken from this node's stream
    int64_t cont = -1;
    bool split = false;
    int guard = 0;
    while (bits(w) < bMax && bits(m) >= bRes && ++guard < 100000) {
      const float lm = ln_pos(m, ft);
      const float x = (lm - tab.rtLnMin) * tab.rtInv;
      const float xs = (lm - tab.sigLnMin) * tab.sigInv;
      const float lns2 = interp(lnSigma, tab.nSigma, xs);
      const float S2 = exp_f(2.0f * lns2, ft);
      const float Sh = exp_f(2.0f * interp(lnSigma, tab.nSigma, xs - tab.halfShift), ft);
      const float wf = exp_f(tab.gamma2 * (ln_pos(w, ft) - lns2), ft);
      const float xc = fminf(fmaxf(x, 0.0f), (float)(tab.rows - 1));
      const int j = min((int)xc, tab.rows - 2);
      const float fx = xc - (float)j;
      const float R = bits(m) <= bRes2 ? 0.0f : wf * (Rt[j] + fx * (Rt[j + 1] - Rt[j]));
      const float F = wf * (Ft[j] + fx * (Ft[j + 1] - Ft[j]));
      // min(dw_sigma, acc/R, acc/F) with one division (acc/max(R, F) is the
      // smaller quotient, rounding being monotone).
      float dwf = tab.accuracySecond * sqrtf(2.0f * fmaxf(Sh - S2, 0.0f));
      const float RF = fmaxf(R, F);
      if (RF > 0.0f) dwf = fminf(dwf, tab.accuracyFirst / RF);
      if (!(dwf > 0.0f)) dwf = 1.0e-3f;
      double dw = f2d_int(dwf);
      const double wStep = w + dw;
      const bool last = bits(wStep) >= bMax;
      if (last) {
        dw = tab.wMax - w;
        dwf = (float)dw;
      }
      const double wNext = last ? tab.wMax : wStep;
      // The mass kept over the step (the rest falls below the resolution).
      const double keep = f2d_int(1.0f - F * dwf);
      mPrev = m;
      wPrev = w;
      if (R > 0.0f && draw24(key, k++) < R * dwf) {
        // q from the split's distribution in ln q of the nearest row with
        // a resolved split (its q range is that row's): the first point of
        // the cumulative distribution above a second draw, and linear
        // interpolation in ln q (the row's points are evenly spaced).
        int row = fx < 0.5f ? j : j + 1;
        if (!(Rt[row] > 0.0f)) row = j + 1;
        const float* cdf = tab.cdf + (size_t)row * kNq;
        const float target = draw24(key, k++);
        int lo = 0, hi = kNq;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (target < cdf[mid])
            hi = mid;
          else
            lo = mid + 1;
        }
        const int k1 = min(max(lo, 1), kNq - 1);
        const float c0 = cdf[k1 - 1];
        const float f = (target - c0) / fmaxf(cdf[k1] - c0, 1e-30f);
        const double q = f2d_int(exp_f(fmaf((float)(k1 - 1) + f, qD[row], qA[row]), ft));
        const double m1 = q * m;
        const double m2 = m * keep - m1;
        const double big = fmax(m1, m2), small = fmin(m1, m2);
        const int count = (big >= tab.mRes) + (small >= tab.mRes);
        if (count > 0) {
          const int64_t first = take_nodes(counters, nd.capacity, count);
          if (first < 0) return;
          put_node(nd, first, big, wNext, child_key(key, 0));
          if (count == 2) {
            put_node(nd, first + 1, small, wNext, child_key(key, 1));
            const unsigned long long at = atomicAdd(&counters[kNext], 1ull);
            next[at] = (int32_t)(first + 1);
          }
          nd.childFirst[i] = (int32_t)first;
          nd.childCount[i] = count;
          cont = first;
        }
        split = true;
        break;
      }
      m *= keep;
      w = wNext;
      if (last) break;
    }
    if (!split) {
      // The branch ends: its earliest resolved halo is a leaf progenitor.
      double lm = m, lw = w;
      if (bits(m) < bRes) {
        lm = mPrev;
        lw = wPrev;
      }
      if (bits(lw) > bits(w0) && bits(lm) >= bRes) {
        const int64_t c = take_nodes(counters, nd.capacity, 1);
        if (c < 0) return;
        put_node(nd, c, lm, lw, child_key(key, 0));
        nd.childFirst[i] = (int32_t)c;
        nd.childCount[i] = 1;
      }
    }
    i = cont;
  }
}

template <typename T>
cudaError_t upload(T** dst, const T* src, size_t n) {
  cudaError_t e = cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(T));
  if (e == cudaSuccess && n) e = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

struct Buffers {
  std::vector<void*> ptrs;
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
  template <typename T>
  cudaError_t put(T** p, const T* src, size_t n) {
    cudaError_t e = upload(p, src, n);
    if (*p) ptrs.push_back(*p);
    return e;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
  ~Buffers() { release(); }
};

}  // namespace

int record_error(gal_ctx* ctx, int code, const char* message) { return gal::host::fail(ctx, code, "%s", message); }

int grow_forest_gpu(gal_ctx* ctx, const BranchTables& tab, const double* rootMass, int64_t n, double rootW,
                    uint64_t seed, std::vector<std::vector<GrownNode>>& trees, double* stats) {
  using gal::host::fail;
  trees.assign((size_t)n, {});
  if (n == 0) return GAL_OK;
  if (n > INT32_MAX / 2) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_build: too many trees%s");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: %s", cudaGetErrorString(e));
  Buffers tb;
  DevTables dt{};
  {
    std::vector<float> ls(tab.lnSigma, tab.lnSigma + tab.nSigma), rf(tab.R, tab.R + tab.rows),
        ff(tab.F, tab.F + tab.rows);
    const std::vector<float> fnt = function_tables();
    std::vector<float> qa((size_t)tab.rows), qd((size_t)tab.rows), cdff((size_t)tab.rows * kNq);
    split_tables(tab, qa.data(), qd.data(), cdff.data());
    float *fnd = nullptr, *a = nullptr, *c = nullptr, *d = nullptr, *pa = nullptr, *pd = nullptr, *cf = nullptr;
    if ((e = tb.put(&fnd, fnt.data(), fnt.size())) != cudaSuccess || (e = tb.put(&a, ls.data(), ls.size())) != cudaSuccess ||
        (e = tb.put(&c, rf.data(), rf.size())) != cudaSuccess || (e = tb.put(&d, ff.data(), ff.size())) != cudaSuccess ||
        (e = tb.put(&pa, qa.data(), qa.size())) != cudaSuccess || (e = tb.put(&pd, qd.data(), qd.size())) != cudaSuccess ||
        (e = tb.put(&cf, cdff.data(), cdff.size())) != cudaSuccess)
      return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: table upload failed: %s", cudaGetErrorString(e));
    dt.fn = fnd;
    dt.lnSigma = a;
    dt.R = c;
    dt.F = d;
    dt.lnqA = pa;
    dt.lnqD = pd;
    dt.cdf = cf;
  }
  const WalkConstants wc = walk_constants(tab);
  dt.nSigma = tab.nSigma;
  dt.rows = tab.rows;
  dt.sigLnMin = wc.sigLnMin;
  dt.sigInv = wc.sigInv;
  dt.halfShift = wc.halfShift;
  dt.rtLnMin = wc.rtLnMin;
  dt.rtInv = wc.rtInv;
  dt.gamma2 = wc.gamma2;
  dt.accuracyFirst = wc.accuracyFirst;
  dt.accuracySecond = wc.accuracySecond;
  dt.mRes = tab.mRes;
  dt.mRes2 = 2.0 * tab.mRes;
  dt.wMax = tab.wMax;
  const size_t smem = (size_t)(kFnTable + tab.nSigma + 4 * tab.rows) * sizeof(float);
  if (tab.nSigma < 2 || tab.rows < 2 || smem > 200 * 1024)
    return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_build: branching tables too large for shared memory%s");
  if ((e = cudaFuncSetAttribute(grow_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
    return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: %s", cudaGetErrorString(e));
  // Roots: node t is the root of tree t.
  std::vector<double> w0((size_t)n, rootW);
  std::vector<uint64_t> key0((size_t)n);
  std::vector<int32_t> first((size_t)n);
  for (int64_t t = 0; t < n; ++t) {
    key0[(size_t)t] = root_key(seed, t);
    first[(size_t)t] = (int32_t)t;
  }
  // Capacity: a first guess from the roots' masses in resolution units,
  // doubled and the growth repeated while it overflows.
  double guess = 0.0;
  for (int64_t t = 0; t < n; ++t) guess += 4.0 + 2.0 * std::pow(rootMass[t] / tab.mRes, 0.85);
  int64_t cap = (int64_t)std::min(std::max(guess, 1.0e6), (double)INT32_MAX);
  // GALNODE_BRANCH_CAPACITY sets the first capacity instead (at least the
  // roots): tests use it to run the overflow-and-repeat path.
  if (const char* env = std::getenv("GALNODE_BRANCH_CAPACITY")) {
    const long long c = std::atoll(env);
    if (c > 0) cap = std::min<int64_t>(std::max<int64_t>(c, n), INT32_MAX);
  }
  cudaStream_t s = ctx->stream;
  std::vector<unsigned long long> counters(kCounters);
  for (int attempt = 0; attempt < 16; ++attempt) {
    Buffers nb;
    DevNodes dn{nullptr, nullptr, nullptr, nullptr, nullptr, cap};
    int32_t *fa = nullptr, *fb = nullptr;
    unsigned long long* dc = nullptr;
    if ((e = nb.alloc(&dn.mass, (size_t)cap)) != cudaSuccess || (e = nb.alloc(&dn.w, (size_t)cap)) != cudaSuccess ||
        (e = nb.alloc(&dn.childFirst, (size_t)cap)) != cudaSuccess ||
        (e = nb.alloc(&dn.childCount, (size_t)cap)) != cudaSuccess ||
        (e = nb.alloc(&dn.key, (size_t)cap)) != cudaSuccess || (e = nb.alloc(&fa, (size_t)cap)) != cudaSuccess ||
        (e = nb.alloc(&fb, (size_t)cap)) != cudaSuccess || (e = nb.alloc(&dc, (size_t)kCounters)) != cudaSuccess)
      return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: device allocation failed: %s", cudaGetErrorString(e));
    counters.assign(kCounters, 0);
    counters[kNodes] = (unsigned long long)n;
    if ((e = cudaMemcpyAsync(dn.mass, rootMass, n * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dn.w, w0.data(), n * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(dn.childFirst, 0, n * sizeof(int32_t), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(dn.childCount, 0, n * sizeof(int32_t), s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dn.key, key0.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(fa, first.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dc, counters.data(), kCounters * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                             s)) != cudaSuccess)
      return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: upload failed: %s", cudaGetErrorString(e));
    const auto t0 = std::chrono::steady_clock::now();
    int64_t nFrontier = n;
    int generations = 0;
    bool overflow = false;
    while (nFrontier > 0) {
      ++generations;
      const int threads = 128;
      const int blocks = (int)((nFrontier + threads - 1) / threads);
      grow_kernel<<<blocks, threads, smem, s>>>(dt, dn, fa, (int32_t)nFrontier, fb, dc);
      ctx->launches++;
      if ((e = cudaGetLastError()) != cudaSuccess ||
          (e = cudaMemcpyAsync(counters.data(), dc, kCounters * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: branching kernel failed: %s", cudaGetErrorString(e));
      if (counters[kOverflow]) {
        overflow = true;
        break;
      }
      nFrontier = (int64_t)counters[kNext];
      std::swap(fa, fb);
      if ((e = cudaMemsetAsync(dc + kNext, 0, sizeof(unsigned long long), s)) != cudaSuccess)
        return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: %s", cudaGetErrorString(e));
    }
    if (overflow) {
      if (cap >= INT32_MAX) return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_build: forest too large%s");
      cap = std::min<int64_t>(std::max<int64_t>(2 * cap, (int64_t)counters[kNodes] + cap / 4), INT32_MAX);
      continue;
    }
    const auto t1 = std::chrono::steady_clock::now();
    const int64_t total = (int64_t)counters[kNodes];
    std::vector<double> mass((size_t)total), w((size_t)total);
    std::vector<int32_t> cf((size_t)total), cc((size_t)total);
    if ((e = cudaMemcpyAsync(mass.data(), dn.mass, total * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(w.data(), dn.w, total * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cf.data(), dn.childFirst, total * sizeof(int32_t), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(cc.data(), dn.childCount, total * sizeof(int32_t), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail(ctx, GAL_ERR_CUDA, "gal_gpu_forest_build: download failed: %s", cudaGetErrorString(e));
    nb.release();
    tb.release();
    // Renumber each tree as the host builder numbers it: depth first, the
    // larger progenitor first, a node's progenitors numbered together when
    // the node is taken.
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < n; ++t) {
      std::vector<GrownNode>& out = trees[(size_t)t];
      std::vector<std::pair<int32_t, int32_t>> stack{{(int32_t)t, 0}};  // (device index, tree index)
      out.push_back(GrownNode{mass[(size_t)t], w[(size_t)t], -1, 0, 0});
      while (!stack.empty()) {
        const auto [d, ti] = stack.back();
        stack.pop_back();
        const int32_t count = cc[(size_t)d];
        if (count == 0) continue;
        const int32_t base = (int32_t)out.size();
        out[(size_t)ti].childFirst = base;
        out[(size_t)ti].childCount = count;
        for (int32_t c = 0; c < count; ++c) {
          const int32_t dc2 = cf[(size_t)d] + c;
          out.push_back(GrownNode{mass[(size_t)dc2], w[(size_t)dc2], ti, 0, 0});
        }
        for (int32_t c = count - 1; c >= 0; --c) stack.push_back({cf[(size_t)d] + c, base + c});
      }
    }
    stats[0] = std::chrono::duration<double>(t1 - t0).count();
    stats[1] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    stats[2] = generations;
    return GAL_OK;
  }
  return fail(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_build: forest too large%s");
}

}  // namespace trees
}  // namespace gal
