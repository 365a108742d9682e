// surrogate.cuh -- the cooling-function surrogate: a 3-64-64-64-1 SiLU MLP
// from (log10 T, log10 Z/Zsun, log10 n_H) to log10 Lambda, evaluated by one
// warp for the 32 nodes of its lanes.  The CIE cooling function scales
// exactly as n_H^2 (cieFileCoolingFunctionDensityLogSlope = 2,
// CIE_file.F90:514-533), so that dependence enters as a fixed term:
// log10 Lambda = (network output) y_scale + y_mean + 2 log10 n_H, and the
// network learns the temperature and metallicity dependence.
//
// Layers 2 and 3 (64 -> 64) run on the tensor cores (mma.sync m16n8k16,
// BF16 x BF16 with FP32 accumulation; the warp's nodes that need the
// network are packed into one or two 16-row tiles).  Each FP32 operand is
// split into a BF16 high part and a BF16 remainder, v = hi + lo, and a
// product is taken as hi*hi + hi*lo + lo*hi
// (three MMAs), which keeps about 16 significant bits -- plain BF16 operands
// (8 bits) put up to 0.03 dex of rounding error on the output, three times
// the fallback tolerance.  The activations never leave registers: layer 1
// (3 -> 64, FP32) is computed directly in the A-fragment layout of layer 2,
// the accumulator fragments of layer 2 are the A fragments of layer 3 (the
// column pairs of an m16n8 accumulator are the column pairs of an m16k16 A
// fragment), and the output layer (64 -> 1, FP32) reduces layer 3's
// accumulators across the four lanes of a row group.  Only the weights live
// in shared memory.
//
// Every lane of the warp must call surrogate_eval together (mma.sync is a
// warp-collective instruction); lanes outside `need` get no row and ignore
// the result, and lanes in it must feed finite inputs.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace gal {

constexpr int kMlpWidth = 64;
constexpr int kMlpStride = 72;  // padded row length (BF16 elements) of the weight rows: conflict-free fragment loads

// Parameter layout of the trained network (FP32, the order the trainer writes):
// W1[64][3], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[64], b4.
constexpr int kW1 = 0, kB1 = kW1 + 64 * 3, kW2 = kB1 + 64, kB2 = kW2 + 64 * 64, kW3 = kB2 + 64,
              kB3 = kW3 + 64 * 64, kW4 = kB3 + 64, kB4 = kW4 + 64, kMlpParams = kB4 + 1;

// The FP32 parameters kept in shared memory: w1[192], b1, b2, b3, w4 [64
// each], b4 (449 values), and the BF16 weight planes W2 hi, W2 lo, W3 hi,
// W3 lo, each [64][kMlpStride] with row n holding W[n][k].
constexpr int kSurrSmall = 64 * 3 + 4 * 64 + 1;
constexpr int kSurrPlane = 64 * kMlpStride;

// Input normalisation and output scaling (x_n = (x - mean)/scale, log10
// Lambda = y_n * yScale + yMean + 2 log10 n_H), the training domain, and
// the cells of the (log10 T, log10 Z) plane where the deployed network
// misses the table by more than the tolerance (the table is used there).
struct SurrogateInfo {
  float inMean[3], inScale[3];
  float yMean, yScale;
  float lo[3], hi[3];          // training domain of the three inputs
  int mapT, mapZ;              // error-map cells in log10 T and log10 Z
  float mapLoT, mapLoZ, mapInvDT, mapInvDZ;
};

// Shared-memory view of the network.
struct SurrogateSmem {
  const float* w1;              // [64][3]
  const float* b1;              // [64]
  const float* b2;
  const float* b3;
  const float* w4;              // [64]
  float b4;
  const __nv_bfloat16* w2hi;    // [64][kMlpStride]
  const __nv_bfloat16* w2lo;
  const __nv_bfloat16* w3hi;
  const __nv_bfloat16* w3lo;
};

// View of the packed parameter block [small FP32 | 4 BF16 planes].
__device__ __forceinline__ SurrogateSmem surrogate_view(const float* small, const __nv_bfloat16* planes) {
  return SurrogateSmem{small, small + 192, small + 256, small + 320, small + 384, small[448],
                       planes, planes + kSurrPlane, planes + 2 * kSurrPlane, planes + 3 * kSurrPlane};
}

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// Lane of the (q+1)-th set bit of mask (q < popc(mask)): PTX fns.
__device__ __forceinline__ int nth_set_lane(unsigned mask, int q) {
  unsigned r;
  asm("fns.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(mask), "r"(q + 1));
  return (int)r;
}

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat162 v) { return *reinterpret_cast<const uint32_t*>(&v); }

// (a, b) -> BF16 pairs hi and lo with a = hi.x + lo.x, b = hi.y + lo.y to ~2^-16.
__device__ __forceinline__ void split_bf16(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  hi = bf16_bits(h);
  lo = bf16_bits(__floats2bfloat162_rn(a - hf.x, b - hf.y));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four 8x8 BF16 matrices from shared memory (ldmatrix): lanes 8m..8m+7 give
// the row addresses of matrix m; each lane receives, of every matrix, the
// pair of row (lane/4), columns 2 (lane%4), +1 -- a B fragment when the
// matrix rows are rows of W.
__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const __nv_bfloat16* rowAddress) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(rowAddress);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// One 64 -> 64 layer for one 16-row tile: acc[nt] (columns nt*8 + 2t, +1 of
// rows g and g+8) = bias + A W^T with the split products.  The B fragments
// of one (n-tile, k-step) -- hi and lo planes, k 0-7 and 8-15 -- come from one
// ldmatrix: lane l addresses row l%8 of the n-tile in the hi (l < 16) or lo
// plane, at k offset 8 ((l/8) % 2).
__device__ __forceinline__ void mlp_layer_tile(const uint32_t (&ahi)[4][4], const uint32_t (&alo)[4][4],
                                               const __nv_bfloat16* whi, const __nv_bfloat16* wlo, const float* bias,
                                               float (&acc)[8][4], int g, int t, int lane) {
  const __nv_bfloat16* laneRow = (lane < 16 ? whi : wlo) + (lane & 7) * kMlpStride + ((lane >> 3) & 1) * 8;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int col = nt * 8 + 2 * t;
    acc[nt][0] = bias[col];
    acc[nt][1] = bias[col + 1];
    acc[nt][2] = bias[col];
    acc[nt][3] = bias[col + 1];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      uint32_t b[4];  // hi k0-7, hi k8-15, lo k0-7, lo k8-15
      ldmatrix_x4(b, laneRow + nt * 8 * kMlpStride + ks * 16);
      mma_bf16(acc[nt], alo[ks], b[0], b[1]);
      mma_bf16(acc[nt], ahi[ks], b[2], b[3]);
      mma_bf16(acc[nt], ahi[ks], b[0], b[1]);
    }
  }
}

// One 16-row tile of the network.  Lane group g = lane/4 holds rows g
// (inputs u) and g + 8 (inputs v); `upper` (warp-uniform) says whether rows
// 8-15 carry nodes -- otherwise their element-wise work is skipped and their
// A rows are zero.  No row's output depends on another row.  On return
// every lane of group g holds in p0 and p1 the normalised outputs of rows g
// and g + 8 without the output bias.  Warp-collective.
__device__ __forceinline__ void mlp_tile(const SurrogateSmem& N, float u0, float u1, float u2, float v0, float v1,
                                         float v2, bool upper, int lane, float& p0, float& p1) {
  const unsigned FULLMASK = 0xffffffffu;
  const int g = lane >> 2, t = lane & 3;
  // Layer 1 (FP32) straight into layer 2's A fragments: for k-step ks the
  // lane holds columns ks*16 + 2t, +1 (regs 0, 1) and ks*16 + 8 + 2t, +1
  // (regs 2, 3) of rows g (regs 0, 2) and g + 8 (regs 1, 3).
  uint32_t ahi[4][4], alo[4][4];
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int c = ks * 16 + half * 8 + 2 * t;
      const float* wa = N.w1 + 3 * c;
      const float h00 = silu(fmaf(wa[2], u2, fmaf(wa[1], u1, fmaf(wa[0], u0, N.b1[c]))));
      const float h01 = silu(fmaf(wa[5], u2, fmaf(wa[4], u1, fmaf(wa[3], u0, N.b1[c + 1]))));
      split_bf16(h00, h01, ahi[ks][2 * half], alo[ks][2 * half]);
    }
  }
  if (upper) {
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int c = ks * 16 + half * 8 + 2 * t;
        const float* wa = N.w1 + 3 * c;
        const float h10 = silu(fmaf(wa[2], v2, fmaf(wa[1], v1, fmaf(wa[0], v0, N.b1[c]))));
        const float h11 = silu(fmaf(wa[5], v2, fmaf(wa[4], v1, fmaf(wa[3], v0, N.b1[c + 1]))));
        split_bf16(h10, h11, ahi[ks][2 * half + 1], alo[ks][2 * half + 1]);
      }
    }
  } else {
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) ahi[ks][1] = alo[ks][1] = ahi[ks][3] = alo[ks][3] = 0u;
  }
  float acc[8][4];
  mlp_layer_tile(ahi, alo, N.w2hi, N.w2lo, N.b2, acc, g, t, lane);
  // Layer 2's accumulators (n-tiles 2ks and 2ks+1) are layer 3's A fragments for k-step ks.
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    split_bf16(silu(acc[2 * ks][0]), silu(acc[2 * ks][1]), ahi[ks][0], alo[ks][0]);
    split_bf16(silu(acc[2 * ks + 1][0]), silu(acc[2 * ks + 1][1]), ahi[ks][2], alo[ks][2]);
  }
  if (upper) {
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      split_bf16(silu(acc[2 * ks][2]), silu(acc[2 * ks][3]), ahi[ks][1], alo[ks][1]);
      split_bf16(silu(acc[2 * ks + 1][2]), silu(acc[2 * ks + 1][3]), ahi[ks][3], alo[ks][3]);
    }
  }
  mlp_layer_tile(ahi, alo, N.w3hi, N.w3lo, N.b3, acc, g, t, lane);
  // Output layer (FP32): this lane's 16 columns of rows g and g + 8, then the
  // sum over the four lanes of the row group.
  p0 = 0.0f;
  p1 = 0.0f;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int col = nt * 8 + 2 * t;
    p0 = fmaf(N.w4[col], silu(acc[nt][0]), fmaf(N.w4[col + 1], silu(acc[nt][1]), p0));
  }
  p0 += __shfl_xor_sync(FULLMASK, p0, 1);
  p0 += __shfl_xor_sync(FULLMASK, p0, 2);
  if (upper) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + 2 * t;
      p1 = fmaf(N.w4[col], silu(acc[nt][2]), fmaf(N.w4[col + 1], silu(acc[nt][3]), p1));
    }
    p1 += __shfl_xor_sync(FULLMASK, p1, 1);
    p1 += __shfl_xor_sync(FULLMASK, p1, 2);
  }
}

// Normalised output of the network for this lane's input (x0, x1, x2):
// returns y_n.  `need` is the warp's ballot of lanes that use the result;
// they are packed into consecutive rows in lane order, so that
// ceil(count/16) tiles run.  The lane of rank q is row (q & 7) of half
// (q >> 3) & 1 of tile q >> 4; its sum ends up in lane 4 (q & 7) of that
// tile's pass.  Warp-collective.
__device__ __forceinline__ float surrogate_eval(const SurrogateSmem& N, float x0, float x1, float x2, int lane,
                                               unsigned need = 0xffffffffu) {
  const unsigned FULLMASK = 0xffffffffu;
  const int g = lane >> 2;
  const int count = __popc(need);
  const int rank = __popc(need & ((1u << lane) - 1u));
  float out = 0.0f;
  const int src = 4 * (rank & 7);
  // The tiles are not unrolled: one copy of the network code.
#pragma unroll 1
  for (int mt = 0; mt < (count + 15) >> 4; ++mt) {
    // Rows past the last needing lane take lane 0's inputs (finite; ignored).
    const int q0 = mt * 16 + g, q1 = q0 + 8;
    const int r0 = q0 < count ? nth_set_lane(need, q0) : 0, r1 = q1 < count ? nth_set_lane(need, q1) : 0;
    const float u0 = __shfl_sync(FULLMASK, x0, r0), u1 = __shfl_sync(FULLMASK, x1, r0), u2 = __shfl_sync(FULLMASK, x2, r0);
    const float v0 = __shfl_sync(FULLMASK, x0, r1), v1 = __shfl_sync(FULLMASK, x1, r1), v2 = __shfl_sync(FULLMASK, x2, r1);
    float p0, p1;
    mlp_tile(N, u0, u1, u2, v0, v1, v2, count - mt * 16 > 8, lane, p0, p1);
    const float o0 = __shfl_sync(FULLMASK, p0, src), o1 = __shfl_sync(FULLMASK, p1, src);
    if ((rank >> 4) == mt) out = ((rank >> 3) & 1) ? o1 : o0;
  }
  return N.b4 + out;
}

// Host-side packing of the FP32 parameters into the block the kernels
// stage: small[kSurrSmall] then the four BF16 planes (hi/lo of W2, W3).
inline void surrogate_pack(const float* P, float* small, __nv_bfloat16* planes) {
  for (int i = 0; i < 192; ++i) small[i] = P[kW1 + i];
  for (int i = 0; i < 64; ++i) {
    small[192 + i] = P[kB1 + i];
    small[256 + i] = P[kB2 + i];
    small[320 + i] = P[kB3 + i];
    small[384 + i] = P[kW4 + i];
  }
  small[448] = P[kB4];
  for (int i = 0; i < 4 * kSurrPlane; ++i) planes[i] = __float2bfloat16_rn(0.0f);
  for (int layer = 0; layer < 2; ++layer) {
    const float* W = P + (layer == 0 ? kW2 : kW3);
    __nv_bfloat16* hi = planes + (2 * layer) * kSurrPlane;
    __nv_bfloat16* lo = planes + (2 * layer + 1) * kSurrPlane;
    for (int r = 0; r < 64; ++r)
      for (int k = 0; k < 64; ++k) {
        const float w = W[r * 64 + k];
        const __nv_bfloat16 h = __float2bfloat16_rn(w);
        hi[r * kMlpStride + k] = h;
        lo[r * kMlpStride + k] = __float2bfloat16_rn(w - __bfloat162float(h));
      }
  }
}

}  // namespace gal
