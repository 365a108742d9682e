// galnode_krumholz.cuh -- Krumholz, McKee & Tumlinson (2009) star formation
// in disks on the GPU, for the FP64 and the FP32-rate forms.
//
// starFormationRateDisksIntgrtdSurfaceDensity (star_formation/rates/disks/
// integrated_surface_density.F90:131-190) integrates the surface density
// law of starFormationRateSurfaceDensityDisksKrumholz2009 (star_formation/
// rate_surface_density/disks/Krumholz2009.F90:312-620) over the exponential
// gas disk, 2 pi int r Sigma_SFR(r) dr on [0, 10 R_d], truncated where the
// molecular fraction falls below 1e-10 and split where X_H Sigma crosses
// the transition surface density, by GSL's adaptive QAG with the 15-point
// Gauss-Kronrod rule at relative tolerance 1e-3.  The same algorithm runs
// here per lane, with the reference's tables: the molecular fraction on
// 1000 points of s in [0, 10] and x^0.33 on [1, 1000] (math/
// exponentiation.F90), both linear.  The truncation and transition radii
// of the exponential disk are found in closed form (the reference's root
// finders converge to them at relative tolerance 1e-4).
#pragma once

#include <cmath>
#include "../../include/galnode.h"

namespace gal {

namespace kmt {
constexpr int kFractionCount = 1000;       // points of the molecular-fraction table on [0, 10]
constexpr double kFractionMaximum = 10.0;
constexpr int kPowerCount = 99901;         // points of the x^0.33 table on [1, 1000]
constexpr double kPowerMinimum = 1.0, kPowerMaximum = 1000.0;
constexpr double kFractionTiny = 1.0e-10;
constexpr double kSurfaceDensityTransition = 85.0e12;  // Msun/Mpc^2
constexpr double kDeltaInfinity = 0.214008;
constexpr int kMaxPieces = 24;             // QAG pieces per interval (the tolerance is met well before)
}  // namespace kmt

// Global-memory tables of one rate precision.
template <class Real>
struct KmtTables {
  const Real* fraction;  // [kFractionCount]
  const Real* power;     // [kPowerCount]
};

// krumholz2009MolecularFractionSlow (star_formation/rates/Krumholz2009/utilities.F90:36-63)
// and ...Fast (Krumholz2009.F90:462-476); host and device.
template <class Real>
__host__ __device__ inline Real kmt_fraction_formula(Real s, bool fast) {
  if (fast) return s < Real(2) ? Real(1) - Real(0.75) * s / (Real(1) + Real(0.25) * s) : Real(0);
  if (s < Real(1.0e-6)) return Real(1) - Real(0.75) * s;
  if (s >= Real(1.0e10)) return Real(0);
  if (s >= Real(10))
    return Real(1) / pow(Real(0.75) / (Real(1) + Real(kmt::kDeltaInfinity)), Real(5)) / Real(5) / pow(s, Real(5));
  const Real delta = Real(0.0712) / pow(Real(0.1) / s + Real(0.675), Real(2.8));
  return Real(1) - Real(1) / pow(Real(1) + pow((Real(1) + delta) / Real(0.75) / s, Real(5)), Real(0.2));
}

// The s at which the molecular fraction falls to 1e-10 (closed form of the
// reference's root; the fast function is zero beyond s = 2).
inline double kmt_s_truncation(bool fast) {
  if (fast) return (1.0 - kmt::kFractionTiny) / (0.5 + 0.25 * kmt::kFractionTiny);
  return std::pow(1.0 / (kmt::kFractionTiny * 5.0 * std::pow(0.75 / (1.0 + kmt::kDeltaInfinity), 5.0)), 0.2);
}

template <class Real>
__device__ __forceinline__ Real kmt_linear(const Real* t, int n, Real x0, Real x1, Real x) {
  const Real dx = (x1 - x0) / Real(n - 1);
  int i = (int)floor((x - x0) / dx);
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  const Real h = (x - (x0 + Real(i) * dx)) / dx;
  const Real a = t[i], b = t[i + 1];
  return a + h * (b - a);
}

// gsl_integration_qk15: 15-point Kronrod with 7-point Gauss, QUADPACK's
// error estimate (the power 1.5 as x sqrt(x)).
template <class Real, class F>
__device__ __noinline__ Real kmt_qk15(const F& f, Real a, Real b, Real& abserr) {
  const Real xgk[8] = {Real(0.991455371120812639206854697526329), Real(0.949107912342758524526189684047851),
                       Real(0.864864423359769072789712788640926), Real(0.741531185599394439863864773280788),
                       Real(0.586087235467691130294144845693013), Real(0.405845151377397166906606412076961),
                       Real(0.207784955007898467600689403773245), Real(0.0)};
  const Real wg[4] = {Real(0.129484966168869693270611432679082), Real(0.279705391489276667901467771423780),
                      Real(0.381830050505118944950369775488975), Real(0.417959183673469387755102040816327)};
  const Real wgk[8] = {Real(0.022935322010529224963732008058970), Real(0.063092092629978553290700663189204),
                       Real(0.104790010322250183839876322541518), Real(0.140653259715525918745189590510238),
                       Real(0.169004726639267902826583426598550), Real(0.190350578064785409913256402421014),
                       Real(0.204432940075298892414161999234649), Real(0.209482141084727828012999174891714)};
  const Real c = Real(0.5) * (a + b), h = Real(0.5) * (b - a);
  const Real fc = f(c);
  Real rg = fc * wg[3], rk = fc * wgk[7], rabs = fabs(rk);
  Real fv1[7], fv2[7];
  // The Gauss nodes (odd Kronrod indices) first, then the others, in
  // QUADPACK's order of summation.
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int jt = 2 * j + 1;
    const Real dx = h * xgk[jt];
    const Real f1 = f(c - dx), f2 = f(c + dx);
    fv1[jt] = f1;
    fv2[jt] = f2;
    rg += wg[j] * (f1 + f2);
    rk += wgk[jt] * (f1 + f2);
    rabs += wgk[jt] * (fabs(f1) + fabs(f2));
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int jt = 2 * j;
    const Real dx = h * xgk[jt];
    const Real f1 = f(c - dx), f2 = f(c + dx);
    fv1[jt] = f1;
    fv2[jt] = f2;
    rk += wgk[jt] * (f1 + f2);
    rabs += wgk[jt] * (fabs(f1) + fabs(f2));
  }
  const Real mean = Real(0.5) * rk;
  Real rasc = wgk[7] * fabs(fc - mean);
#pragma unroll
  for (int j = 0; j < 7; ++j) rasc += wgk[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  rabs *= fabs(h);
  rasc *= fabs(h);
  Real err = fabs((rk - rg) * h);
  if (rasc != Real(0) && err != Real(0)) {
    const Real x = Real(200) * err / rasc;
    const Real scale = x * sqrt(x);
    err = scale < Real(1) ? rasc * scale : rasc;
  }
  const Real tiny = sizeof(Real) == 8 ? Real(2.2250738585072014e-308 / (50.0 * 2.220446049250313e-16))
                                      : Real(1.17549435e-38f / (50.0f * 1.1920929e-7f));
  const Real eps50 = sizeof(Real) == 8 ? Real(50.0 * 2.220446049250313e-16) : Real(50.0f * 1.1920929e-7f);
  if (rabs > tiny) err = fmax(err, eps50 * rabs);
  abserr = err;
  return rk * h;
}

// gsl_integration_qag's global adaptive bisection (at most kMaxPieces pieces).
template <class Real, class F>
__device__ Real kmt_qag(const F& f, Real a, Real b, Real epsabs, Real epsrel) {
  Real pa[kmt::kMaxPieces], pb[kmt::kMaxPieces], pr[kmt::kMaxPieces], pe[kmt::kMaxPieces];
  int n = 1;
  pa[0] = a;
  pb[0] = b;
  pr[0] = kmt_qk15<Real>(f, a, b, pe[0]);
  for (;;) {
    Real total = Real(0), error = Real(0);
    int worst = 0;
    for (int k = 0; k < n; ++k) {
      total += pr[k];
      error += pe[k];
      if (pe[k] > pe[worst]) worst = k;
    }
    if (error <= fmax(epsabs, epsrel * fabs(total)) || n == kmt::kMaxPieces) return total;
    const Real m = Real(0.5) * (pa[worst] + pb[worst]);
    Real e1, e2;
    const Real r1 = kmt_qk15<Real>(f, pa[worst], m, e1), r2 = kmt_qk15<Real>(f, m, pb[worst], e2);
    pa[n] = m;
    pb[n] = pb[worst];
    pr[n] = r2;
    pe[n] = e2;
    pb[worst] = m;
    pr[worst] = r1;
    pe[worst] = e1;
    ++n;
  }
}

// r Sigma_SFR(r) of krumholz2009Rate (Krumholz2009.F90:360-414) for one disk.
template <class Real>
struct KmtIntegrand {
  KmtTables<Real> K;
  Real frequency, sNorm, sigmaNorm, sigma0, xH, radiusDisk;
  bool fast;
  __device__ Real operator()(Real r) const {
    const Real sg = sigma0 * exp(-r / radiusDisk);
    if (sg <= Real(sizeof(Real) == 8 ? 1.0e-100 : 1.0e-30)) return Real(0);
    const Real s = sNorm / (sigmaNorm * sg);
    const Real fraction = s > Real(kmt::kFractionMaximum) ? kmt_fraction_formula<Real>(s, fast)
                                                         : kmt_linear<Real>(K.fraction, kmt::kFractionCount, Real(0),
                                                                            Real(kmt::kFractionMaximum), s);
    const Real sd = xH * sg / Real(kmt::kSurfaceDensityTransition);
    const Real x = sd < Real(1) ? Real(1) / sd : sd;
    const Real factor = sd <= Real(0) ? Real(0)
                        : (x > Real(kmt::kPowerMaximum) ? pow(x, Real(0.33))
                                                        : kmt_linear<Real>(K.power, kmt::kPowerCount, Real(kmt::kPowerMinimum),
                                                                           Real(kmt::kPowerMaximum), x));
    return r * (frequency * sg * factor * fraction);
  }
};

// Star formation rate (Msun/Gyr) of a disk of gas mass massGas, metal mass
// metalsGas and exponential scale length radiusDisk.  frequency:
// frequencyStarFormation (1/Gyr); clumping: clumpingFactorMolecularComplex;
// sTruncation: kmt_s_truncation.
//
// Not inlined: the right-hand side is inlined at every stage, and one copy
// of this integrator per kernel keeps the code (and its compile time) small.
template <class Real>
__device__ __noinline__ Real krumholz2009_rate(const KmtTables<Real> K, Real frequency, Real clumping, Real sTruncation,
                                               bool fast, Real massGas, Real metalsGas, Real radiusDisk) {
  if (!(massGas > Real(0)) || !(radiusDisk > Real(0))) return Real(0);
  const Real Z = metalsGas > massGas ? Real(1) : (metalsGas <= Real(0) ? Real(0) : metalsGas / massGas);
  const Real zs = Z / Real(0.0188);
  if (!(zs > Real(0))) return Real(0);
  const Real xH = fmin(fmax(zs * Real(0.7070 - 0.7514) + Real(0.7514), Real(0.7)), Real(0.7514));
  // krumholz2009ComputeFactors (Krumholz2009.F90:312-358).
  const Real chi = Real(0.77) * (Real(1) + Real(3.1) * pow(zs, Real(0.365)));
  const Real sigmaNorm = xH * clumping / Real(1.0e12);
  if (!(sigmaNorm > Real(0))) return Real(0);
  const Real sNorm = log(Real(1) + Real(0.6) * chi + Real(0.01) * chi * chi) / (Real(0.04) * zs);
  const Real truncation = sNorm / sigmaNorm / sTruncation;
  const Real sigma0 = massGas / (Real(2.0 * 3.14159265358979323846) * radiusDisk * radiusDisk);
  // krumholz2009Rate (Krumholz2009.F90:360-414) times r.
  const KmtIntegrand<Real> integrand{K, frequency, sNorm, sigmaNorm, sigma0, xH, radiusDisk, fast};
  // krumholz2009Intervals (Krumholz2009.F90:478-587) for the monotonic disk.
  const Real rOut = Real(10) * radiusDisk;
  if (sigma0 <= truncation) return Real(0);
  const Real rMax = sigma0 * exp(-rOut / radiusDisk) <= truncation ? radiusDisk * log(sigma0 / truncation) : rOut;
  const Real sdIn = xH * sigma0 / Real(kmt::kSurfaceDensityTransition);
  const Real sdMax = xH * (sigma0 * exp(-rMax / radiusDisk)) / Real(kmt::kSurfaceDensityTransition);
  const Real epsabs = Real(1.0e-12), epsrel = Real(1.0e-3);
  Real integral;
  if (sdIn <= Real(1) || sdMax >= Real(1)) {
    integral = kmt_qag<Real>(integrand, Real(0), rMax, epsabs, epsrel);
  } else {
    const Real rCrit = radiusDisk * log(xH * sigma0 / Real(kmt::kSurfaceDensityTransition));
    integral = kmt_qag<Real>(integrand, Real(0), rCrit, epsabs, epsrel) + kmt_qag<Real>(integrand, rCrit, rMax, epsabs, epsrel);
  }
  return Real(2.0 * 3.14159265358979323846) * integral;
}

}  // namespace gal
