// trees_internal.h -- what the host tree builder (trees.cpp) and the device
// branching (trees_gpu.cu) share: the grown-node record, the builder's
// tables as flat arrays, and the keyed random streams of the device
// branching.
//
// Keyed streams.  The host builder draws every tree from one sequential
// stream, so the order in which branches are grown fixes the tree.  On the
// GPU thousands of branches grow at once, so each branch draws from its
// own stream: a node's key is a function of its tree and of its path from
// the root (child_key of its parent's key and its rank among the
// progenitors), and the k-th number drawn while growing that node's branch
// is SplitMix64 (Steele, Lea & Flood 2014) at key + (k + 1) gamma.  A tree
// is then a function of (seed, tree index, root mass) alone, whatever the
// schedule.
#ifndef GALNODE_TREES_INTERNAL_H
#define GALNODE_TREES_INTERNAL_H

#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define GAL_HD __host__ __device__ __forceinline__
#else
#define GAL_HD inline
#endif

struct gal_ctx;

namespace gal {
namespace trees {

// One node of a grown tree: halo mass, w = delta_c0/D(z), and its links
// (progenitors contiguous, the larger first).
struct GrownNode {
  double mass, w;
  int32_t parent, childFirst, childCount;
};

// Points of the tabulated split distribution in ln q per rate row.
constexpr int kNq = 96;

// The builder's tables and step parameters as flat host arrays.
struct BranchTables {
  // ln sigma(M) at z = 0 on a grid in ln M.
  double sigLnMin, sigDlnM;
  int32_t nSigma;
  const double* lnSigma;
  // Split rate R, sub-resolution accretion rate F (both without their
  // (w/sigma)^gamma2 factor) and the split's cumulative distribution in
  // ln q, per row of a grid in ln M.
  double rtLnMin, rtDlnM;
  int32_t rows;
  const double* R;
  const double* F;
  const double* lnq;  // [rows][kNq]
  const double* cdf;  // [rows][kNq], normalised to 1 where R > 0
  double mRes, wMax, gamma2, accuracyFirst, accuracySecond;
};

constexpr uint64_t kGamma = 0x9e3779b97f4a7c15ull;

GAL_HD uint64_t mix64(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
// The root's key of tree t.
GAL_HD uint64_t root_key(uint64_t seed, int64_t tree) {
  return mix64(seed + kGamma) ^ mix64((uint64_t)tree * 0xd1b54a32d192ed03ull + 0x5851f42d4c957f2dull);
}
// The key of progenitor c (0 the larger) of the node with key k.
GAL_HD uint64_t child_key(uint64_t k, int c) { return mix64(k ^ (0xa0761d6478bd642full * (uint64_t)(c + 1))); }
// The k-th uniform draw in [0, 1) of the stream with key `key`, to 53 bits
// (draw) or to 24 bits as a float (draw24).
GAL_HD double draw(uint64_t key, uint32_t k) {
  return (double)(mix64(key + (uint64_t)(k + 1) * kGamma) >> 11) * 0x1.0p-53;
}
GAL_HD float draw24(uint64_t key, uint32_t k) {
  return (float)(uint32_t)(mix64(key + (uint64_t)(k + 1) * kGamma) >> 40) * 0x1.0p-24f;
}

// The walk's function tables, as floats: ln c_j [128], 1/c_j [128] at
// c_j = 1 + (j + 1/2)/128, then 2^(j/32) [32], rounded from FP64.
constexpr int kFnTable = 128 + 128 + 32;
inline std::vector<float> function_tables() {
  std::vector<float> t(kFnTable);
  for (int j = 0; j < 128; ++j) {
    const double c = 1.0 + (j + 0.5) / 128.0;
    t[(size_t)j] = (float)std::log(c);
    t[(size_t)(128 + j)] = (float)(1.0 / c);
  }
  for (int j = 0; j < 32; ++j) t[(size_t)(256 + j)] = (float)std::exp2(j / 32.0);
  return t;
}

// The FP32 split tables of the GPU walk: per rate row, ln q at its first
// point and the spacing of its (evenly spaced) points in ln q, and the
// cumulative distribution [rows][kNq], rounded from the FP64 tables.
inline void split_tables(const BranchTables& t, float* lnqA, float* lnqD, float* cdf) {
  for (int32_t r = 0; r < t.rows; ++r) {
    const double* q = t.lnq + (size_t)r * kNq;
    lnqA[r] = (float)q[0];
    lnqD[r] = (float)((q[kNq - 1] - q[0]) / (kNq - 1));
    for (int k = 0; k < kNq; ++k) cdf[(size_t)r * kNq + k] = (float)t.cdf[(size_t)r * kNq + k];
  }
}

// The FP32 constants of the GPU walk, rounded from the FP64 tables' grid:
// ln M of the first rows, the inverse spacings, the shift of the sigma row
// coordinate from M to M/2 (ln 2 / spacing), gamma2 and the accuracies.
struct WalkConstants {
  float sigLnMin, sigInv, halfShift, rtLnMin, rtInv, gamma2, accuracyFirst, accuracySecond;
};
inline WalkConstants walk_constants(const BranchTables& t) {
  return WalkConstants{(float)t.sigLnMin, (float)(1.0 / t.sigDlnM), (float)(0.6931471805599453 / t.sigDlnM),
                       (float)t.rtLnMin, (float)(1.0 / t.rtDlnM), (float)t.gamma2, (float)t.accuracyFirst,
                       (float)t.accuracySecond};
}

// Grow the branches of n trees on the context's GPU from their roots
// (root masses rootMass[n] at w = rootW), with the keyed streams of seed;
// trees[t] receives tree t in the host builder's order (depth first, the
// larger progenitor first, a node's progenitors numbered when it splits).
// Returns a GAL_* code (errors recorded in the context).
// Record an error in the context (its message for gal_gpu_last_error) and
// return code.
int record_error(gal_ctx* ctx, int code, const char* message);

// stats[3] receives the seconds of the device growth (its generations), of
// the nodes' download and renumbering on the host, and the number of
// generations.
int grow_forest_gpu(gal_ctx* ctx, const BranchTables& tab, const double* rootMass, int64_t n, double rootW,
                    uint64_t seed, std::vector<std::vector<GrownNode>>& trees, double* stats);

}  // namespace trees
}  // namespace gal

#endif
