// galnode_fastmath.cuh -- FP64 elementary functions with few FP64-pipe
// instructions, for the integrator's critical path.
//
// On GB300 the FP64 pipe accepts about one warp instruction every 64-76
// cycles per SM sub-partition, whatever the number of active lanes.  A node
// that needs a thousand right-hand-side evaluations runs alone in its warp at
// the end of a batch, so its time is the number of FP64 instructions on its
// path times that interval.  The library log, exp, divide, sqrt and pow
// expand to 12-90 FP64 instructions each; the versions below use integer and
// single-precision instructions (other pipes) wherever they do not limit
// accuracy, and FP64 for the refinement:
//
//  * rcp/div/rsqrt/sqrt: the single-precision hardware approximation
//    (relative error ~1e-7) refined by two Newton-Raphson steps in FP64,
//    which square the error twice (~1e-28) before the final rounding.
//  * log: the table-driven reduction of Tang (1990, ACM TOMS 16, 378).  x = 2^e m, m in [1,2);
//    c = 1 + (j + 1/2)/128 from the top seven mantissa bits; then
//    ln x = e ln 2 + ln c + ln(1 + r), r = m/c - 1, |r| < 2^-8, with
//    ln(1 + r) from its Taylor series to r^6 (truncation < 2^-58).
//  * exp: the table-driven reduction of Tang (1989, ACM TOMS 15, 144):
//    x = (64 k + j) ln2/64 + r, |r| <= ln2/128, so
//    e^x = 2^k 2^(j/64) e^r with e^r from its Taylor series to r^6
//    (truncation < 2^-65) and 2^(j/64) from a table.
//  * inv_root: x^(-1/Q) from the single-precision seed and Newton steps
//    g <- g + g (1 - x g^Q)/Q (replaces pow in the step-size controller).
//
// The tables (ln c_j, 1/c_j and 2^(j/64)) are computed on the host in FP64
// from the C library and staged in shared memory.  Arguments outside the
// ranges the reductions cover fall back to the CUDA functions.  Every
// function is checked against the CUDA library by gal_selftest_fastmath.
#pragma once

#include <cmath>
#include <cstdint>

namespace gal {

struct FastTables {
  const double2* log;  // [128]: (ln c_j, 1/c_j)
  const double* exp2;  // [64]: 2^(j/64)
};

constexpr int kLogTableSize = 128;
constexpr int kExpTableSize = 64;
constexpr double kLn2Hi = 6.93147180369123816490e-01;  // ln 2 split into a head with trailing zero bits
constexpr double kLn2Lo = 1.90821492927058770002e-10;  // and the remainder

// Integer tests on the high word: x is positive with a binary exponent in
// [lo, hi]; |x| has a binary exponent in [lo, hi].
__device__ __forceinline__ bool positive_exponent_in(double x, int lo, int hi) {
  const int h = __double2hiint(x);
  return h >= ((lo + 1023) << 20) && h < ((hi + 1024) << 20);
}
__device__ __forceinline__ bool abs_exponent_in(double x, int lo, int hi) {
  const int h = __double2hiint(x) & 0x7fffffff;
  return h >= ((lo + 1023) << 20) && h < ((hi + 1024) << 20);
}

__device__ __forceinline__ double fast_rcp(double y) {
  if (!abs_exponent_in(y, -120, 120)) return 1.0 / y;
  double r = (double)__frcp_rn((float)y);
  double e = fma(-y, r, 1.0);
  r = fma(r, e, r);
  e = fma(-y, r, 1.0);
  return fma(r, e, r);
}

__device__ __forceinline__ double fast_div(double x, double y) { return x * fast_rcp(y); }

__device__ __forceinline__ double fast_rsqrt(double x) {
  if (!positive_exponent_in(x, -120, 120)) return 1.0 / sqrt(x);
  double r = (double)rsqrtf((float)x);
  const double hx = 0.5 * x;
  r = r * fma(-hx * r, r, 1.5);
  return r * fma(-hx * r, r, 1.5);
}

__device__ __forceinline__ double fast_sqrt(double x) {
  if (!positive_exponent_in(x, -120, 120)) return sqrt(x);
  const double r = fast_rsqrt(x);
  const double s = x * r;
  return fma(0.5 * r, fma(-s, s, x), s);
}

__device__ __forceinline__ double fast_log(const FastTables& T, double x) {
  if (!positive_exponent_in(x, -1000, 1000)) return log(x);
  const long long bits = __double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff) - 1023;
  const int j = (int)((bits >> 45) & 127);
  const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const double2 t = T.log[j];
  const double r = fma(m, t.y, -1.0);
  // ln(1+r) = r + r^2 (-1/2 + r/3 - r^2/4 + r^3/5 - r^4/6)
  double p = fma(r, -1.0 / 6.0, 1.0 / 5.0);
  p = fma(r, p, -0.25);
  p = fma(r, p, 1.0 / 3.0);
  p = fma(r, p, -0.5);
  p = fma(r * r, p, r);
  const double de = (double)e;
  return fma(de, kLn2Hi, t.x + fma(de, kLn2Lo, p));
}

__device__ __forceinline__ double fast_exp(const FastTables& T, double x) {
  if (!(x > -700.0 && x < 700.0)) return exp(x);
  const double shifter = 6755399441055744.0;  // 1.5 * 2^52: adding it rounds to an integer in the low bits
  const double kd = fma(x, 64.0 / 0.69314718055994530942, shifter);
  const int k = __double2loint(kd);
  const double n = kd - shifter;
  const double r = fma(-n, kLn2Lo / 64.0, fma(-n, kLn2Hi / 64.0, x));
  // e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720)
  double p = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  p = fma(r, p, 1.0 / 24.0);
  p = fma(r, p, 1.0 / 6.0);
  p = fma(r, p, 0.5);
  p = fma(r * r, p, r);
  const double s = T.exp2[k & 63];
  const double v = fma(s, p, s);
  // Multiply by 2^(k >> 6) through the exponent field (|k >> 6| < 1011 here).
  return __longlong_as_double(__double_as_longlong(v) + ((long long)(k >> 6) << 52));
}

template <int Q>
__device__ __forceinline__ double inv_root(double x) {
  double g = (double)exp2f(-(1.0f / Q) * __log2f((float)x));
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double g2 = g * g;
    const double gq = Q == 5 ? g2 * g2 * g : g2 * g2 * g2;
    g = fma(g * (1.0 / Q), fma(-x, gq, 1.0), g);
  }
  return g;
}

// FP64 min/max as compare-and-select (shorter than the min/max instruction).
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }

// ---------------------------------------------------------------------------
// Exact IEEE-754 comparisons of doubles on the integer pipe.  On GB300 every
// FP64 instruction of a warp -- compare and conversion included -- holds
// its SM sub-partition's FP64 pipe for ~64 cycles (an FP64 compare with its
// select ~110), while a 64-bit integer compare takes a few cycles; a lone
// node's step control is a chain of such compares.  Each function returns
// what the IEEE comparison returns, NaNs (false for every ordered
// comparison) and signed zeros (-0 == +0) included.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool d_isnan(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
// Order-preserving key of a non-NaN double: a < b <=> d_key(a) < d_key(b),
// with -0 mapped onto +0.
__device__ __forceinline__ long long d_key(double x) {
  long long b = __double_as_longlong(x);
  if (b == (long long)0x8000000000000000ULL) b = 0;
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool d_lt(double a, double b) { return !(d_isnan(a) || d_isnan(b)) && d_key(a) < d_key(b); }
__device__ __forceinline__ bool d_le(double a, double b) { return !(d_isnan(a) || d_isnan(b)) && d_key(a) <= d_key(b); }
__device__ __forceinline__ bool d_gt(double a, double b) { return d_lt(b, a); }
__device__ __forceinline__ bool d_ge(double a, double b) { return d_le(b, a); }
// x < 0.0: sign bit set, not -0, not NaN.
__device__ __forceinline__ bool d_neg(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && b != (long long)0x8000000000000000ULL && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL;
}
// Exact conversions between FP32 and FP64 on the integer pipe, for the
// values that are normal in both formats (a conversion instruction holds
// the FP64 pipe like an FP64 operation does).  float -> double: rebias the
// exponent and shift the significand; zero keeps its sign; subnormals,
// infinities and NaNs take the conversion instruction.
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned a = u & 0x7fffffffu;
  if (a - 0x00800000u >= 0x7f000000u) {  // zero, subnormal, infinity or NaN
    if (a == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)f;
  }
  return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + 0x38000000u)), (int)(u << 29));
}
// double -> float with round-to-nearest-even, for doubles whose float is
// normal (a carry out of the largest float gives infinity, as the
// conversion does); everything else takes the conversion instruction.
__device__ __forceinline__ float d2f_int(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned ahi = hi & 0x7fffffffu;
  if (ahi - 0x38100000u >= 0x0fe00000u) return (float)d;  // float exponent outside 1..254 (or inf/NaN)
  unsigned f = ((ahi - 0x38000000u) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1fffffffu;
  f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
  return __uint_as_float(f | (hi & 0x80000000u));
}
// Comparisons of a non-negative, non-NaN double with a positive constant:
// the bit patterns order as signed integers.
__device__ __forceinline__ bool dpos_gt(double x, double c) { return __double_as_longlong(x) > __double_as_longlong(c); }
__device__ __forceinline__ bool dpos_lt(double x, double c) { return __double_as_longlong(x) < __double_as_longlong(c); }

// 0.9 x^(-1/Q) (Q = 5 or 6) for the step-size controller, to full FP64
// precision, from the FP32 ratio xf ~ x that is at hand before x is.  The
// seed g0 = xf^(-1/Q) is formed in FP32 (its error, from xf's and the FP32
// functions', is ~1e-6); with e = 1 - x g0^Q, exactly
// x^(-1/Q) = g0 (1 - e)^(-1/Q) = g0 (1 + e/Q + (1+Q) e^2/(2Q^2) + c3 e^3 + ...),
// and for |e| < 2^-17 the terms from e^3 on are below 4e-17 relative, so the
// series to e^2 gives the root to rounding.  FP64 work: one conversion, Q's
// three products, four FMA/products -- against the two Newton steps of
// inv_root, 12 operations after a conversion round trip.  Returns a
// negative value when the seed is too far off (|e| >= 2^-17, or xf not a
// usable float); the caller then takes inv_root.
template <int Q>
__device__ __forceinline__ double ctrl_root09(double x, float xf) {
  if (!(xf > 1.0e-30f && xf < 1.0e30f)) return -1.0;
  const double g0 = f2d_int(exp2f(-(1.0f / Q) * __log2f(xf)));
  const double g2 = g0 * g0;  // exact: g0 has a 24-bit significand
  const double gq = Q == 5 ? (g2 * g2) * g0 : (g2 * g0) * (g2 * g0);
  const double e = fma(-x, gq, 1.0);
  if ((__double2hiint(e) & 0x7fffffff) >= ((1023 - 17) << 20)) return -1.0;  // |e| >= 2^-17 (or NaN)
  constexpr double c1 = 1.0 / Q, c2 = (1.0 + Q) / (2.0 * Q * Q);
  const double u = e * fma(c2, e, c1);
  return 0.9 * fma(g0, u, g0);
}

// 1/y to full FP64 precision from an FP32 approximation ys of y that is at
// hand before y is: two Newton steps from the FP32 reciprocal of ys, with
// no FP64<->FP32 conversion on the FP64 pipe.  Newton squares the relative
// error, so the second step lands at rounding when the residual after the
// first is below 2^-27; otherwise (a poor or unusable seed) fast_rcp.
__device__ __forceinline__ double rcp_seeded(double y, float ys) {
  if (!(ys > 1.0e-30f && ys < 1.0e30f) || !abs_exponent_in(y, -99, 99)) return fast_rcp(y);
  double r = f2d_int(__frcp_rn(ys));
  double e = fma(-y, r, 1.0);
  r = fma(r, e, r);
  e = fma(-y, r, 1.0);
  if ((__double2hiint(e) & 0x7fffffff) >= ((1023 - 27) << 20)) return fast_rcp(y);  // |e| >= 2^-27 (or NaN)
  return fma(r, e, r);
}

// Host-side construction of the tables.
inline void fast_tables_host(double2* logTable, double* exp2Table) {
  for (int j = 0; j < kLogTableSize; ++j) {
    const double c = 1.0 + (j + 0.5) / kLogTableSize;
    logTable[j] = make_double2(std::log(c), 1.0 / c);
  }
  for (int j = 0; j < kExpTableSize; ++j) exp2Table[j] = std::exp2((double)j / kExpTableSize);
}

}  // namespace gal
