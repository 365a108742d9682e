// galnode_oracle.cpp -- CPU oracle for the node-evolution hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU kernels
// are compared against, and the timed CPU baseline of bench.py.  Nothing in
// the product (galacticus_gb300/, include/) links, loads or calls it.
//
// It restates, in plain scalar C++ and FP64, the reference's algorithm for
// one node evolution step (Galacticus mergerTreeNodeEvolverStandard%evolve)
// under the "P-std" physics profile.  Each function cites the reference
// source it follows (paths relative to the Galacticus repository root).
// The reference itself cannot be built here (Fortran 2008 + GSL + HDF5 +
// FoX, none installed), so this restatement is pinned instead against the
// reference's own known answers (closedBox / leakyBox reproducibility
// values, the ODE-solver unit-test values, baryon mass conservation and the
// CIE cooling-function normalisation); see tests/test_oracle_golden.py.
//
// The GSL Cash-Karp stepper, `gsl_odeiv2_evolve_apply` and the Brent root
// finder are third-party code that is not part of the reference tree.  They
// are restated from the published methods (Cash & Karp 1990, ACM TOMS 16,
// 201; Brent 1973, "Algorithms for Minimization without Derivatives") and
// the behaviour documented in the GSL manual (odeiv2 "Evolution" and
// "Adaptive Step-size Control"; root finding "brent" and
// gsl_root_test_interval).  The GSL version used by the reference is not
// pinned anywhere in its repository.
//
// Everything physical is templated on the scalar type so that the same code
// run with `Counted` (below) yields the algorithmic FP64 operation count per
// node-timestep used for the roofline.

#include <cmath>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

#include "../include/galnode.h"

namespace orc {

// ---------------------------------------------------------------------------
// Counting scalar.  Weights are declared in oracle/flop_weights.json and
// passed in by the caller of oracle_count_flops().
// ---------------------------------------------------------------------------
enum { OP_ADD, OP_MUL, OP_DIV, OP_SQRT, OP_LOG, OP_EXP, OP_POW, OP_ATAN, OP_CBRT, OP_N };
static thread_local uint64_t g_ops[OP_N];

struct Counted {
  double v;
  Counted() : v(0) {}
  Counted(double x) : v(x) {}
};
static inline Counted operator+(Counted a, Counted b) { g_ops[OP_ADD]++; return Counted(a.v + b.v); }
static inline Counted operator-(Counted a, Counted b) { g_ops[OP_ADD]++; return Counted(a.v - b.v); }
static inline Counted operator*(Counted a, Counted b) { g_ops[OP_MUL]++; return Counted(a.v * b.v); }
static inline Counted operator/(Counted a, Counted b) { g_ops[OP_DIV]++; return Counted(a.v / b.v); }
static inline Counted operator-(Counted a) { return Counted(-a.v); }
static inline Counted& operator+=(Counted& a, Counted b) { a = a + b; return a; }
static inline Counted& operator-=(Counted& a, Counted b) { a = a - b; return a; }
static inline Counted& operator*=(Counted& a, Counted b) { a = a * b; return a; }
static inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
static inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
static inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
static inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }
static inline bool operator==(Counted a, Counted b) { return a.v == b.v; }
static inline bool operator!=(Counted a, Counted b) { return a.v != b.v; }

static inline double val(double x) { return x; }
static inline double val(Counted x) { return x.v; }

static inline double xsqrt(double x) { return std::sqrt(x); }
static inline double xlog(double x) { return std::log(x); }
static inline double xexp(double x) { return std::exp(x); }
static inline double xpow(double x, double y) { return std::pow(x, y); }
static inline double xatan(double x) { return std::atan(x); }
static inline double xcbrt(double x) { return std::cbrt(x); }
static inline Counted xsqrt(Counted x) { g_ops[OP_SQRT]++; return Counted(std::sqrt(x.v)); }
static inline Counted xlog(Counted x) { g_ops[OP_LOG]++; return Counted(std::log(x.v)); }
static inline Counted xexp(Counted x) { g_ops[OP_EXP]++; return Counted(std::exp(x.v)); }
static inline Counted xpow(Counted x, Counted y) { g_ops[OP_POW]++; return Counted(std::pow(x.v, y.v)); }
static inline Counted xatan(Counted x) { g_ops[OP_ATAN]++; return Counted(std::atan(x.v)); }
static inline Counted xcbrt(Counted x) { g_ops[OP_CBRT]++; return Counted(std::cbrt(x.v)); }
template <class R> static inline R xabs(R x) { return x < R(0.0) ? -x : x; }
template <class R> static inline R xmax(R a, R b) { return a > b ? a : b; }
template <class R> static inline R xmin(R a, R b) { return a < b ? a : b; }

// ---------------------------------------------------------------------------
// Physical constants (source/numerical/constants/*.F90; values of the GSL
// MKSA constants they name).
// ---------------------------------------------------------------------------
namespace k {
const double Pi = 3.14159265358979323846;
const double gravitationalConstant = 6.673e-11;      // GSL_CONST_MKSA_GRAVITATIONAL_CONSTANT
const double massSolar = 1.98892e30;                  // GSL_CONST_MKSA_SOLAR_MASS
const double parsec = 3.08567758135e16;               // GSL_CONST_MKSA_PARSEC
const double megaParsec = 1.0e6 * parsec;
const double year = 3.15581497635456e7;               // astronomical.F90:66
const double gigaYear = 1.0e9 * year;
const double boltzmannsConstant = 1.3806504e-23;      // GSL_CONST_MKSA_BOLTZMANN
const double atomicMassUnit = 1.660538782e-27;        // GSL_CONST_MKSA_UNIFIED_ATOMIC_MASS
const double speedLight = 2.99792458e8;               // GSL_CONST_MKSA_SPEED_OF_LIGHT
const double thomsonCrossSection = 6.65245893699e-29; // GSL_CONST_MKSA_THOMSON_CROSS_SECTION
const double atomicMassHydrogen = 1.0078250322;       // atomic.F90
const double atomicMassHelium = 4.0026032545;
const double massHydrogenAtom = atomicMassHydrogen * atomicMassUnit;
const double hydrogenByMassPrimordial = 0.7514;       // astronomical.F90:53-54
const double heliumByMassPrimordial = 0.2486;
const double hydrogenByMassSolar = 0.7070;            // astronomical.F90:45-47
const double heliumByMassSolar = 0.2740;
const double metallicitySolar = 0.0188;
const double meanAtomicMassPrimordial =
    1.0 / (2.0 * hydrogenByMassPrimordial / atomicMassHydrogen + 3.0 * heliumByMassPrimordial / atomicMassHelium);
const double kilo = 1.0e3, hecto = 1.0e2, ergs = 1.0e-7;
const double gravitationalConstantInternal = gravitationalConstant * massSolar / (kilo * kilo) / megaParsec; // astronomical.F90:72
const double MpcPerKmPerSToGyr = megaParsec / kilo / gigaYear;                                             // astronomical.F90:77
const double feedbackEnergyInputAtInfinityCanonical = 4.517e5; // stellar_astrophysics/feedback/_class.F90:56
}  // namespace k

// Sound speed of a primordial ideal gas in km/s (thermodynamics/ideal_gases.F90:46-69).
static double sound_speed(double temperature) {
  return std::sqrt(5.0 * k::boltzmannsConstant * temperature / 3.0 / k::meanAtomicMassPrimordial / k::atomicMassUnit) / k::kilo;
}

// ---------------------------------------------------------------------------
// CIE tables (cooling_function/CIE_file.F90, chemical/state/CIE_file.F90).
// ---------------------------------------------------------------------------
struct Table {
  int nT = 0, nZ = 0;
  std::vector<double> lnT, lnZ, lnL, lnNe;  // logarithmic table (all entries > 0)
  double Tmin = 0, Tmax = 0, Zmin = 0, Zmax = 0;
  bool firstZero = false;
  double firstNonZero = 0;
};

// cieFileReadFile (CIE_file.F90:535-663): limits, Z=0 row handling, logs.
static int table_load(const gal_cie_table* t, Table& out) {
  if (!t || t->n_temperature < 2 || t->n_metallicity < 2) return GAL_ERR_TABLE;
  out.nT = t->n_temperature;
  out.nZ = t->n_metallicity;
  out.Tmin = t->temperature[0];
  out.Tmax = t->temperature[out.nT - 1];
  out.Zmin = t->metallicity[0];
  out.Zmax = t->metallicity[out.nZ - 1];
  for (int i = 0; i < out.nZ * out.nT; ++i)
    if (!(t->cooling_rate[i] > 0.0) || !(t->electron_density[i] > 0.0)) return GAL_ERR_TABLE;
  out.firstZero = (t->metallicity[0] == 0.0);
  if (out.firstZero) out.firstNonZero = t->metallicity[1];
  out.lnT.resize(out.nT);
  out.lnZ.resize(out.nZ);
  for (int i = 0; i < out.nT; ++i) out.lnT[i] = std::log(t->temperature[i]);
  for (int j = 0; j < out.nZ; ++j) out.lnZ[j] = t->metallicity[j] > 0.0 ? std::log(t->metallicity[j]) : -999.0;
  out.lnL.resize(out.nZ * out.nT);
  out.lnNe.resize(out.nZ * out.nT);
  for (int i = 0; i < out.nZ * out.nT; ++i) {
    out.lnL[i] = std::log(t->cooling_rate[i]);
    out.lnNe[i] = std::log(t->electron_density[i]);
  }
  return GAL_OK;
}

// Index of the grid cell holding x: the largest i with grid[i] <= x, kept in
// [0, n-2] (interpolator%locate followed by the clamp of CIE_file.F90:670-676).
static int locate(const std::vector<double>& g, double x) {
  int lo = 0, hi = (int)g.size() - 1;
  if (x < g[0]) return 0;
  if (x >= g[hi]) return hi - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (g[mid] <= x) lo = mid; else hi = mid;
  }
  return std::min(std::max(lo, 0), (int)g.size() - 2);
}

// Bilinear interpolation factors in (ln T, ln Z), with the Z=0 row treated
// linearly in Z (CIE_file.F90:665-715).  `metallicity` is Z/Zsun, already
// clamped to the table range ("fix" extrapolation) by the caller.
template <class R>
static void interp_factors(const Table& tb, R lnT, R metallicity, int& iT, R& hT, int& iZ, R& hZ) {
  iT = locate(tb.lnT, val(lnT));
  hT = (lnT - R(tb.lnT[iT])) / (R(tb.lnT[iT + 1]) - R(tb.lnT[iT]));
  R Zuse = xmax(metallicity, R(0.0));
  if (tb.firstZero && Zuse < R(tb.firstNonZero)) {
    iZ = 0;
    hZ = Zuse / R(tb.firstNonZero);
  } else {
    R lnZ = xlog(Zuse);
    iZ = locate(tb.lnZ, val(lnZ));
    hZ = (lnZ - R(tb.lnZ[iZ])) / (R(tb.lnZ[iZ + 1]) - R(tb.lnZ[iZ]));
  }
}

template <class R>
static R interp_table(const std::vector<double>& v, int nT, int iT, R hT, int iZ, R hZ) {
  // cieFileInterpolate (CIE_file.F90:717-735), in the log table, then exp.
  R f = R(v[iZ * nT + iT]) * (R(1.0) - hT) * (R(1.0) - hZ) + R(v[(iZ + 1) * nT + iT]) * (R(1.0) - hT) * hZ +
        R(v[iZ * nT + iT + 1]) * hT * (R(1.0) - hZ) + R(v[(iZ + 1) * nT + iT + 1]) * hT * hZ;
  return xexp(f);
}

// Temperature clamp: both files use "extrapolate" in T, which the reference
// implements by clamping the temperature to the table range before the
// interpolation (CIE_file.F90:257-274); metallicity uses "fix" (:276-292).
template <class R>
static void clamp_inputs(const Table& tb, R& T, R& Z) {
  if (T < R(tb.Tmin)) T = R(tb.Tmin);
  if (T > R(tb.Tmax)) T = R(tb.Tmax);
  if (Z < R(tb.Zmin)) Z = R(tb.Zmin);
  if (Z > R(tb.Zmax)) Z = R(tb.Zmax);
}

// Cooling function Lambda (erg cm^-3 s^-1) for hydrogen density nH (cm^-3):
// cieFileCoolingFunction (CIE_file.F90:238-317) = interpolated table * nH^2.
// `Zsolar` is Z/Zsun.
template <class R>
static R cooling_function(const Table& tb, R nH, R T, R Zsolar) {
  clamp_inputs(tb, T, Zsolar);
  int iT, iZ;
  R hT, hZ;
  interp_factors(tb, xlog(T), Zsolar, iT, hT, iZ, hZ);
  return interp_table(tb.lnL, tb.nT, iT, hT, iZ, hZ) * nH * nH;
}

// Electron density (cm^-3): chemicalStateCIEFile%electronDensity
// (chemical/state/CIE_file.F90:245-320) = interpolated n_e/n_H * nH.
template <class R>
static R electron_density(const Table& tb, R nH, R T, R Zsolar) {
  clamp_inputs(tb, T, Zsolar);
  int iT, iZ;
  R hT, hZ;
  interp_factors(tb, xlog(T), Zsolar, iT, hT, iZ, hZ);
  return interp_table(tb.lnNe, tb.nT, iT, hT, iZ, hZ) * nH;
}

// ---------------------------------------------------------------------------
// Abundances (objects/abundances.F90).
// ---------------------------------------------------------------------------
// Abundances_Mass_To_Mass_Fraction_Packed (:781-809).
template <class R>
static R mass_fraction(R metals, R mass) {
  if (metals > mass) return R(1.0);
  if (metals <= R(0.0)) return R(0.0);
  return metals / mass;
}
// Abundances_Hydrogen_Mass_Fraction (:830-850); Z is a mass fraction.
template <class R>
static R hydrogen_mass_fraction(R Z) {
  R x = Z / R(k::metallicitySolar) * R(k::hydrogenByMassSolar - k::hydrogenByMassPrimordial) + R(k::hydrogenByMassPrimordial);
  return xmin(xmax(x, R(0.7)), R(k::hydrogenByMassPrimordial));
}
// Abundances_Helium_Mass_Fraction (:852-868).
template <class R>
static R helium_mass_fraction(R Z) {
  R y = Z / R(k::metallicitySolar) * R(k::heliumByMassSolar - k::heliumByMassPrimordial) + R(k::heliumByMassPrimordial);
  return xmin(y, R(k::heliumByMassPrimordial));
}
// Abundances_Hydrogen_Number_Fraction (:870-883).
template <class R>
static R hydrogen_number_fraction(R Z) {
  R nH = hydrogen_mass_fraction(Z) / R(k::atomicMassHydrogen);
  R nHe = helium_mass_fraction(Z) / R(k::atomicMassHelium);
  return nH / (nH + nHe);
}

// ---------------------------------------------------------------------------
// Per-evolve-call node constants.  The halo scales (virial radius, velocity,
// temperature, dynamical time) and the galaxy sizes of the fixed structure
// solver are held at their start-of-call values; every state-dependent
// quantity is recomputed in each right-hand-side evaluation.
// ---------------------------------------------------------------------------
struct Node {
  double massHalo, massRate, radiusVirial, velocityVirial, spin;
  double temperatureVirial;   // virialDensityContrastDefinitionVirialTemperature (virial_density_contrast.F90:251-262)
  double timeDynamical;       // r_vir/V_vir in Gyr (:195-206)
  double radiusCore;          // virialFraction core radius
  double radiusOuter;         // hot-halo outer radius: min(max(.,0.1 r_vir), r_vir) = r_vir for these nodes
  double betaNormalization;   // 1/(x - atan x) of beta_profile.F90:243-250
  double radiusDisk, velocityDisk, radiusSpheroid, velocitySpheroid;
};

static void node_setup(const gal_params& p, const double* prm, Node& n) {
  n.massHalo = prm[GAL_P_MASS];
  n.massRate = prm[GAL_P_MASS_RATE];
  n.radiusVirial = prm[GAL_P_RADIUS_VIRIAL];
  n.velocityVirial = prm[GAL_P_VELOCITY_VIRIAL];
  n.spin = prm[GAL_P_SPIN];
  n.temperatureVirial = 0.5 * k::atomicMassUnit * k::meanAtomicMassPrimordial *
                        (k::kilo * n.velocityVirial) * (k::kilo * n.velocityVirial) / k::boltzmannsConstant;
  n.timeDynamical = n.radiusVirial / n.velocityVirial * (k::megaParsec / k::kilo / k::gigaYear);
  n.radiusCore = p.core_radius_fraction * n.radiusVirial;
  // Node_Component_Hot_Halo_Standard_Outer_Radius (hot_halo/standard/_class.F90:430-450)
  // with the stored outer radius initialised to the virial radius.
  n.radiusOuter = std::max(std::min(n.radiusVirial, n.radiusVirial), 0.1 * n.radiusVirial);
  double x = n.radiusOuter / n.radiusCore;
  n.betaNormalization = x < 1.0e-6 ? 3.0 / (x * x * x) + 9.0 / 5.0 / x - 36.0 * x / 175.0 : 1.0 / (x - std::atan(x));
  // galacticStructureSolverFixed, radiusFixed=virial (galactic_structure/radius_solver/fixed.F90):
  // r = factor * r_vir * J/J_scale = factor * lambda * r_vir, v = v_vir.
  n.radiusDisk = p.radius_factor_disk * n.spin * n.radiusVirial;
  n.velocityDisk = n.velocityVirial;
  n.radiusSpheroid = p.radius_factor_spheroid * n.spin * n.radiusVirial;
  n.velocitySpheroid = n.velocityVirial;
}

// Beta-profile (beta=2/3) density of the hot gas, truncated at the outer
// radius (mass_distributions/spherical/beta_profile.F90:303-320).
template <class R>
static R hot_density(const Node& n, R massHot, R r) {
  if (massHot <= R(0.0) || n.radiusOuter <= 0.0) return R(0.0);  // betaProfileGet returns no distribution
  if (r > R(n.radiusOuter)) return R(0.0);
  R rho0 = massHot / R(4.0 * k::Pi) / R(n.radiusCore * n.radiusCore * n.radiusCore) * R(n.betaNormalization);
  R x = r / R(n.radiusCore);
  return rho0 / (R(1.0) + x * x);
}

// Hernquist density of the spheroid gas (mass_distributions/spherical/Hernquist.F90:184,206-222).
template <class R>
static R spheroid_gas_density(const Node& n, R massGas, R r) {
  if (massGas <= R(0.0) || n.radiusSpheroid <= 0.0) return R(0.0);
  R a = R(n.radiusSpheroid);
  R rho0 = massGas / R(2.0 * k::Pi) / (a * a * a);
  R x = r / a;
  R opx = R(1.0) + x;
  return rho0 / x / (opx * opx * opx);
}

// Cooling time (Gyr) of hot gas at density rho (Msun/Mpc^3):
// coolingTimeSimple%time (cooling/cooling_time/simple.F90:128-179).
template <class R>
static R cooling_time(const gal_params& p, const Table& tb, R T, R rho, R Zfrac) {
  R xH = hydrogen_mass_fraction(Zfrac);
  R nH = rho * xH * R(k::massSolar / k::massHydrogenAtom / (k::hecto * k::hecto * k::hecto) /
                      (k::megaParsec * k::megaParsec * k::megaParsec));
  R Zsolar = Zfrac / R(k::metallicitySolar);
  R nAll = nH / hydrogen_number_fraction(Zfrac) + electron_density(tb, nH, T, Zsolar);
  R lambda = cooling_function(tb, nH, T, Zsolar);
  if (lambda > R(0.0)) {
    R energy = R(p.cooling_degrees_of_freedom) / R(2.0) * R(k::boltzmannsConstant) * T * nAll / R(k::ergs);
    return energy / lambda / R(k::gigaYear);
  }
  return R(1.0e10);
}

// Brent root finder on a bracketing interval with GSL's interval test
// (epsabs, epsrel).  Used by coolingRadiusSimple (cooling_radius/simple.F90:
// 147-151, 313-387); restated from Brent (1973) as implemented by GSL's
// `brent` fsolver.
template <class R, class F>
static R brent(F f, R a, R b, R fa, R fb, double epsabs, double epsrel) {
  // Solver state as initialised by GSL's brent fsolver: c = b, d = e = b - a.
  R c = b, fc = fb, d = b - a, e = b - a;
  for (int iter = 0; iter < 1000; ++iter) {
    bool acEqual = false;
    if ((fb < R(0.0) && fc < R(0.0)) || (fb > R(0.0) && fc > R(0.0))) {
      acEqual = true;
      c = a; fc = fa; d = b - a; e = b - a;
    }
    if (xabs(fc) < xabs(fb)) {
      acEqual = true;
      a = b; b = c; c = a; fa = fb; fb = fc; fc = fa;
    }
    R tol = R(0.5 * DBL_EPSILON) * xabs(b);
    R m = R(0.5) * (c - b);
    if (fb == R(0.0)) return b;
    if (xabs(m) <= tol) return b;
    if (xabs(e) < tol || xabs(fa) <= xabs(fb)) {
      d = m; e = m;  // bisection
    } else {
      R pp, q, r, s = fb / fa;
      if (acEqual) {
        pp = R(2.0) * m * s;
        q = R(1.0) - s;
      } else {
        q = fa / fc;
        r = fb / fc;
        pp = s * (R(2.0) * m * q * (q - r) - (b - a) * (r - R(1.0)));
        q = (q - R(1.0)) * (r - R(1.0)) * (s - R(1.0));
      }
      if (pp > R(0.0)) q = -q; else pp = -pp;
      R min1 = R(3.0) * m * q - xabs(tol * q), min2 = xabs(e * q);
      if (R(2.0) * pp < (min1 < min2 ? min1 : min2)) {
        e = d; d = pp / q;
      } else {
        d = m; e = m;
      }
    }
    a = b; fa = fb;
    if (xabs(d) > tol) b = b + d; else b = b + (m > R(0.0) ? tol : -tol);
    fb = f(b);
    // Bracket reported by the solver: [b, c], with c replaced by the previous
    // iterate when fb and fc share a sign; then gsl_root_test_interval.
    R cb = ((fb < R(0.0) && fc < R(0.0)) || (fb > R(0.0) && fc > R(0.0))) ? a : c;
    R lo = b < cb ? b : cb, hi = b < cb ? cb : b;
    R minAbs = (lo > R(0.0) && hi > R(0.0)) || (lo < R(0.0) && hi < R(0.0)) ? xmin(xabs(lo), xabs(hi)) : R(0.0);
    if (xabs(hi - lo) < R(epsabs) + R(epsrel) * minAbs) return b;
  }
  return b;
}

// ---------------------------------------------------------------------------
// Krumholz, McKee & Tumlinson (2009) star formation in disks: the surface
// density law of starFormationRateSurfaceDensityDisksKrumholz2009
// (star_formation/rate_surface_density/disks/Krumholz2009.F90:312-620)
// integrated over the exponential gas disk by
// starFormationRateDisksIntgrtdSurfaceDensity (star_formation/rates/disks/
// integrated_surface_density.F90:131-190) with GSL's adaptive QAG and the
// 15-point Gauss-Kronrod rule at relative tolerance 1e-3 (absolute 1e-12).
// The tables are the reference's: the molecular fraction on 1000 points of
// s in [0, 10] and x^0.33 on [1, 1000] at 100 points per unit
// (math/exponentiation.F90), both interpolated linearly.
// ---------------------------------------------------------------------------
namespace kmt {
const double sMaximum = 10.0;
const int sCount = 1000;
const double fractionTiny = 1.0e-10;
const double surfaceDensityTransition = 85.0e12;  // Msun/Mpc^2

// krumholz2009MolecularFractionSlow (star_formation/rates/Krumholz2009/utilities.F90:36-63).
double fraction_slow(double s) {
  const double deltaInfinity = 0.214008;
  if (s < 1.0e-6) return 1.0 - 0.75 * s;
  if (s >= 1.0e10) return 0.0;
  if (s >= 10.0) return 1.0 / std::pow(0.75 / (1.0 + deltaInfinity), 5.0) / 5.0 / std::pow(s, 5.0);
  const double delta = 0.0712 / std::pow(0.1 / s + 0.675, 2.8);
  return 1.0 - 1.0 / std::pow(1.0 + std::pow((1.0 + delta) / 0.75 / s, 5.0), 0.2);
}
// krumholz2009MolecularFractionFast (Krumholz2009.F90:462-476).
double fraction_fast(double s) { return s < 2.0 ? 1.0 - 0.75 * s / (1.0 + 0.25 * s) : 0.0; }

struct Tables {
  std::vector<double> fraction[2];  // slow, fast on [0, sMaximum]
  std::vector<double> power;        // x^0.33 on [1, 1000]
  double sTruncation[2];
  Tables() {
    for (int k = 0; k < 2; ++k) {
      fraction[k].resize(sCount);
      for (int i = 0; i < sCount; ++i) {
        const double s = sMaximum * i / (sCount - 1);
        fraction[k][i] = k ? fraction_fast(s) : fraction_slow(s);
      }
    }
    // The s at which the molecular fraction falls to fractionTiny (found by
    // a root finder at relative tolerance 1e-6 in the reference; both
    // fitting functions invert in closed form there).
    sTruncation[0] = std::pow(1.0 / (fractionTiny * 5.0 * std::pow(0.75 / (1.0 + 0.214008), 5.0)), 0.2);
    sTruncation[1] = (1.0 - fractionTiny) / (0.5 + 0.25 * fractionTiny);
    const int n = (int)((1000.0 - 1.0) * 100.0) + 1;
    power.resize(n);
    for (int i = 0; i < n; ++i) power[i] = std::pow(1.0 + (1000.0 - 1.0) * i / (n - 1), 0.33);
  }
  static double linear(const std::vector<double>& t, double x0, double x1, double x) {
    const int n = (int)t.size();
    const double dx = (x1 - x0) / (n - 1);
    int i = (int)std::floor((x - x0) / dx);
    i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
    const double h = (x - (x0 + i * dx)) / dx;
    return t[i] + h * (t[i + 1] - t[i]);
  }
  double fraction_of(double s, int fast) const {
    if (s > sMaximum) return fast ? fraction_fast(s) : fraction_slow(s);
    return linear(fraction[fast], 0.0, sMaximum, s);
  }
  // fastExponentiator%exponentiate (math/exponentiation.F90): table inside [1, 1000].
  double power033(double x) const { return (x < 1.0 || x > 1000.0) ? std::pow(x, 0.33) : linear(power, 1.0, 1000.0, x); }
};
const Tables& tables() {
  static const Tables t;
  return t;
}

// gsl_integration_qk15: the 15-point Kronrod rule with its 7-point Gauss
// rule and QUADPACK's error estimate (Piessens et al. 1983).
template <class F>
double qk15(F& f, double a, double b, double& abserr) {
  static const double xgk[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                                0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                                0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                                0.207784955007898467600689403773245, 0.0};
  static const double wg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                               0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
  static const double wgk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
  const double c = 0.5 * (a + b), h = 0.5 * (b - a);
  const double fc = f(c);
  double rg = fc * wg[3], rk = fc * wgk[7], rabs = std::fabs(rk);
  double fv1[7], fv2[7];
  for (int j = 0; j < 3; ++j) {
    const int jt = 2 * j + 1;
    const double dx = h * xgk[jt];
    const double f1 = f(c - dx), f2 = f(c + dx);
    fv1[jt] = f1;
    fv2[jt] = f2;
    rg += wg[j] * (f1 + f2);
    rk += wgk[jt] * (f1 + f2);
    rabs += wgk[jt] * (std::fabs(f1) + std::fabs(f2));
  }
  for (int j = 0; j < 4; ++j) {
    const int jt = 2 * j;
    const double dx = h * xgk[jt];
    const double f1 = f(c - dx), f2 = f(c + dx);
    fv1[jt] = f1;
    fv2[jt] = f2;
    rk += wgk[jt] * (f1 + f2);
    rabs += wgk[jt] * (std::fabs(f1) + std::fabs(f2));
  }
  const double mean = 0.5 * rk;
  double rasc = wgk[7] * std::fabs(fc - mean);
  for (int j = 0; j < 7; ++j) rasc += wgk[j] * (std::fabs(fv1[j] - mean) + std::fabs(fv2[j] - mean));
  const double result = rk * h;
  rabs *= std::fabs(h);
  rasc *= std::fabs(h);
  double err = std::fabs((rk - rg) * h);
  if (rasc != 0.0 && err != 0.0) {
    const double scale = std::pow(200.0 * err / rasc, 1.5);
    err = scale < 1.0 ? rasc * scale : rasc;
  }
  if (rabs > DBL_MIN / (50.0 * DBL_EPSILON)) err = std::max(err, 50.0 * DBL_EPSILON * rabs);
  abserr = err;
  return result;
}

// gsl_integration_qag's global adaptive bisection: split the interval with
// the largest error until the summed error meets max(epsabs, epsrel |I|).
template <class F>
double qag(F& f, double a, double b, double epsabs, double epsrel) {
  struct Piece { double a, b, r, e; };
  std::vector<Piece> pieces;
  double e0;
  const double r0 = qk15(f, a, b, e0);
  pieces.push_back({a, b, r0, e0});
  for (int it = 0; it < 1000; ++it) {
    double total = 0.0, error = 0.0;
    size_t worst = 0;
    for (size_t k = 0; k < pieces.size(); ++k) {
      total += pieces[k].r;
      error += pieces[k].e;
      if (pieces[k].e > pieces[worst].e) worst = k;
    }
    if (error <= std::max(epsabs, epsrel * std::fabs(total))) return total;
    const Piece p = pieces[worst];
    const double m = 0.5 * (p.a + p.b);
    double e1, e2;
    const double r1 = qk15(f, p.a, m, e1), r2 = qk15(f, m, p.b, e2);
    pieces[worst] = {p.a, m, r1, e1};
    pieces.push_back({m, p.b, r2, e2});
  }
  double total = 0.0;
  for (const Piece& p : pieces) total += p.r;
  return total;
}

// The disk's star formation rate (Msun/Gyr): 2 pi int r Sigma_SFR(r) dr over
// [0, 10 R_d], truncated where the molecular fraction falls below 1e-10 and
// split at the radius where X_H Sigma equals the transition surface density.
double star_formation_rate(const gal_params& p, double massGas, double metalsGas, double radiusDisk) {
  if (!(massGas > 0.0) || !(radiusDisk > 0.0)) return 0.0;
  const Tables& T = tables();
  // Abundances of the fuel (objects/abundances.F90:781-868).
  const double Z = metalsGas > massGas ? 1.0 : (metalsGas <= 0.0 ? 0.0 : metalsGas / massGas);
  const double zs = Z / k::metallicitySolar;
  const double xH = std::min(std::max(zs * (k::hydrogenByMassSolar - k::hydrogenByMassPrimordial) + k::hydrogenByMassPrimordial, 0.7),
                             k::hydrogenByMassPrimordial);
  if (!(zs > 0.0)) return 0.0;
  // krumholz2009ComputeFactors (Krumholz2009.F90:312-358).
  const double chi = 0.77 * (1.0 + 3.1 * std::pow(zs, 0.365));
  const double sigmaNorm = xH * p.krumholz_clumping / 1.0e12;
  if (!(sigmaNorm > 0.0)) return 0.0;
  const double sNorm = std::log(1.0 + 0.6 * chi + 0.01 * chi * chi) / (0.04 * zs);
  const int fast = p.krumholz_fast ? 1 : 0;
  const double truncation = sNorm / sigmaNorm / T.sTruncation[fast];
  // The exponential gas disk (mass_distributions/cylindrical/exponential_disk.F90).
  const double sigma0 = massGas / (2.0 * k::Pi * radiusDisk * radiusDisk);
  auto sigma_at = [&](double r) { return sigma0 * std::exp(-r / radiusDisk); };
  // krumholz2009Rate (Krumholz2009.F90:360-414).
  auto rate = [&](double r) {
    const double sg = sigma_at(r);
    if (sg <= 1.0e-100) return 0.0;
    const double s = sNorm / (sigmaNorm * sg);
    const double fraction = T.fraction_of(s, fast);
    const double sd = xH * sg / surfaceDensityTransition;
    const double factor = sd <= 0.0 ? 0.0 : (sd < 1.0 ? T.power033(1.0 / sd) : T.power033(sd));
    return p.krumholz_frequency * sg * factor * fraction;
  };
  auto integrand = [&](double r) { return r * rate(r); };
  // krumholz2009Intervals (Krumholz2009.F90:478-587) for the monotonic disk.
  const double rIn = 0.0, rOut = 10.0 * radiusDisk;
  if (sigma_at(rIn) <= truncation) return 0.0;
  const double rMax = sigma_at(rOut) <= truncation ? radiusDisk * std::log(sigma0 / truncation) : rOut;
  const double sdIn = xH * sigma_at(rIn) / surfaceDensityTransition, sdMax = xH * sigma_at(rMax) / surfaceDensityTransition;
  double integral;
  if (sdIn <= 1.0 || sdMax >= 1.0) {
    integral = qag(integrand, rIn, rMax, 1.0e-12, 1.0e-3);
  } else {
    const double rCrit = radiusDisk * std::log(xH * sigma0 / surfaceDensityTransition);
    integral = qag(integrand, rIn, rCrit, 1.0e-12, 1.0e-3) + qag(integrand, rCrit, rMax, 1.0e-12, 1.0e-3);
  }
  return 2.0 * k::Pi * integral;
}
}  // namespace kmt

// Right-hand side of the node ODE system for the P-std profile: the sum of
// the node operators of nodeOperatorMulti (nodes/operators/multi.F90:313-332)
// in the order of parameters/quickTest.xml.  `dydt` is overwritten.
template <class R>
struct Rhs {
  const gal_params& p;
  const Table& tb;
  const Node& n;
  bool cooling_radius_brent;  // true: Brent root (reference); false: closed form
  uint64_t evaluations = 0;

  // Star-formation timescale (star_formation/timescales/dynamical_time.F90:121-189 or fixed).
  R sf_timescale(const gal_star_formation& sf, double radius, double velocity) const {
    if (sf.timescale_type == GAL_SF_TIMESCALE_FIXED) return R(sf.timescale_fixed);
    if (velocity <= 0.0 || sf.efficiency == 0.0) return R(0.0);
    R tdyn = R(k::MpcPerKmPerSToGyr) * R(radius) / R(velocity);
    return xmax(tdyn * xpow(R(velocity) / R(200.0), R(sf.exponent_velocity)) / R(sf.efficiency), R(sf.timescale_minimum));
  }
  // Outflow rate (power_law/_class.F90:118-164 or fixed.F90) limited by
  // rate_limit.F90; returns the (ejective) total, expulsive being zero.
  R outflow_rate(const gal_outflow& o, double radius, double velocity, R massGas, R rateStarFormation) const {
    R energy = R(k::feedbackEnergyInputAtInfinityCanonical) * rateStarFormation;
    R ejective;
    if (o.type == GAL_OUTFLOW_FIXED) {
      ejective = R(o.fraction) * energy / R(k::feedbackEnergyInputAtInfinityCanonical);
    } else if (velocity <= 0.0) {
      ejective = R(0.0);
    } else {
      ejective = xpow(R(o.velocity_characteristic) / R(velocity), R(o.exponent)) * energy /
                 R(k::feedbackEnergyInputAtInfinityCanonical);
    }
    if (o.timescale_fractional_minimum > 0.0) {
      R tdyn = (velocity <= 0.0 || radius <= 0.0) ? R(1.0) : R(k::MpcPerKmPerSToGyr) * R(radius) / R(velocity);
      R maximum = xmax(massGas / tdyn / R(o.timescale_fractional_minimum), R(0.0));
      if (ejective > maximum) ejective = ejective * maximum / ejective;
    }
    return ejective;
  }

  // Cooling radius (cooling_radius/simple.F90:313-427) for hot mass M and metal fraction Z.
  R cooling_radius(R massHot, R Zfrac) const {
    R T = R(n.temperatureVirial);
    R tAvail = R(n.timeDynamical);  // coolingTimeAvailableWhiteFrenk1991 with ageFactor=0
    auto root = [&](R r) { return cooling_time(p, tb, T, hot_density(n, massHot, r), Zfrac) - tAvail; };
    R rOuter = R(n.radiusOuter);
    R fOuter = root(rOuter);
    if (fOuter < R(0.0)) return rOuter;
    R fZero = root(R(0.0));
    if (fZero > R(0.0)) return R(0.0);
    if (cooling_radius_brent) return brent(root, R(0.0), rOuter, fZero, fOuter, 0.0, 1.0e-6);
    // Closed form: t_cool is proportional to 1/rho at fixed T and Z, so the
    // root solves rho(r) = rho(0) t_cool(0)/t_avail.
    R rhoCool = hot_density(n, massHot, R(0.0)) * (fZero + tAvail) / tAvail;
    return R(n.radiusCore) * xsqrt(hot_density(n, massHot, R(0.0)) / rhoCool - R(1.0));
  }

  void operator()(R /*t*/, const R* y, R* dydt) {
    ++evaluations;
    for (int i = 0; i < GAL_NY; ++i) dydt[i] = R(0.0);
    const uint32_t ph = p.physics;
    const R massHot = y[GAL_Y_HOT_MASS], metalsHot = y[GAL_Y_HOT_METALS];
    // Cooling radius is shared by the cooling rate and the BH hot-mode fraction.
    bool coolingRadiusKnown = false;
    R radiusCooling = R(0.0);
    auto get_cooling_radius = [&]() {
      if (!coolingRadiusKnown) {
        radiusCooling = cooling_radius(massHot, mass_fraction(metalsHot, massHot));
        coolingRadiusKnown = true;
      }
      return radiusCooling;
    };

    // --- starFormationDisks (nodes/operators/physics/star_formation/disks.F90:200-324)
    R sfrDisk = R(0.0);
    const R gasDisk = y[GAL_Y_DISK_GAS];
    const bool diskOk = !(n.radiusDisk < 0.0 || gasDisk < R(0.0));
    if (diskOk) {
      if (p.sf_disk_rate == GAL_SF_RATE_KRUMHOLZ2009) {
        // intgrtdSurfaceDensityRate with krumholz2009 (evaluated in FP64; not counted by the counting scalar).
        sfrDisk = R(kmt::star_formation_rate(p, val(gasDisk), val(y[GAL_Y_DISK_GAS_METALS]), n.radiusDisk));
      } else {
        R ts = sf_timescale(p.sf_disk, n.radiusDisk, n.velocityDisk);
        sfrDisk = ts > R(0.0) ? gasDisk / ts : R(0.0);  // timescaleRate (rates/disks/timescale.F90:109-130)
      }
    }
    if ((ph & GAL_PHYS_STAR_FORMATION_DISK) && diskOk) {
      // stellarPopulationPropertiesInstantaneous%rates (stellar_populations/properties/instantaneous.F90:133-219)
      R Z = mass_fraction(y[GAL_Y_DISK_GAS_METALS], gasDisk);
      R rateStars = R(1.0 - p.recycled_fraction) * sfrDisk;
      R rateMetalsStars = Z * rateStars;
      dydt[GAL_Y_DISK_STARS] += rateStars;
      dydt[GAL_Y_DISK_GAS] += -rateStars;
      dydt[GAL_Y_DISK_STARS_METALS] += rateMetalsStars;
      dydt[GAL_Y_DISK_GAS_METALS] += -rateMetalsStars + R(p.metal_yield) * sfrDisk;
    }
    // --- starFormationSpheroids (star_formation/spheroids.F90:152-); plausibility minima of :156-158.
    R sfrSph = R(0.0);
    const R gasSph = y[GAL_Y_SPHEROID_GAS];
    const bool sphOk = !(n.radiusSpheroid < 1.0e-12 || gasSph < R(1.0e-6));
    if (sphOk) {
      R ts = sf_timescale(p.sf_spheroid, n.radiusSpheroid, n.velocitySpheroid);
      sfrSph = ts > R(0.0) ? gasSph / ts : R(0.0);
    }
    if ((ph & GAL_PHYS_STAR_FORMATION_SPHEROID) && sphOk) {
      R Z = mass_fraction(y[GAL_Y_SPHEROID_GAS_METALS], gasSph);
      R rateStars = R(1.0 - p.recycled_fraction) * sfrSph;
      dydt[GAL_Y_SPHEROID_STARS] += rateStars;
      dydt[GAL_Y_SPHEROID_GAS] += -rateStars;
      dydt[GAL_Y_SPHEROID_GAS_METALS] += -(Z * rateStars) + R(p.metal_yield) * sfrSph;
    }
    // --- stellarFeedbackDisks (stellar_feedback/disks.F90:116-205)
    if ((ph & GAL_PHYS_FEEDBACK_DISK) && diskOk) {
      R Z = mass_fraction(y[GAL_Y_DISK_GAS_METALS], gasDisk);
      R total = outflow_rate(p.outflow_disk, n.radiusDisk, n.velocityDisk, gasDisk, sfrDisk);
      if (total > R(0.0)) {
        R metals = gasDisk > R(0.0) ? Z * total : R(0.0);
        dydt[GAL_Y_OUTFLOWED_MASS] += total;  // outflowing pipe, fractionStripped=0 (hot_halo/standard/_class.F90:598-668)
        dydt[GAL_Y_DISK_GAS] += -total;
        dydt[GAL_Y_OUTFLOWED_METALS] += metals;
        dydt[GAL_Y_DISK_GAS_METALS] += -metals;
      }
    }
    // --- stellarFeedbackSpheroids (stellar_feedback/spheroids.F90:116-208)
    if ((ph & GAL_PHYS_FEEDBACK_SPHEROID) && sphOk) {
      R Z = mass_fraction(y[GAL_Y_SPHEROID_GAS_METALS], gasSph);
      R total = outflow_rate(p.outflow_spheroid, n.radiusSpheroid, n.velocitySpheroid, gasSph, sfrSph);
      if (total > R(0.0)) {
        R metals = gasSph > R(0.0) ? Z * total : R(0.0);
        dydt[GAL_Y_OUTFLOWED_MASS] += total;
        dydt[GAL_Y_SPHEROID_GAS] += -total;
        dydt[GAL_Y_OUTFLOWED_METALS] += metals;
        dydt[GAL_Y_SPHEROID_GAS_METALS] += -metals;
      }
    }
    // --- blackHolesAccretion (nodes/operators/physics/black_holes/accretion.F90:113-174)
    //     with blackHoleAccretionRateStandard (black_holes/accretion_rates/standard.F90:221-440).
    const R massBH = y[GAL_Y_BLACK_HOLE];
    if ((ph & GAL_PHYS_BLACK_HOLE_ACCRETION) && massBH > R(0.0)) {
      const double G = k::gravitationalConstantInternal;
      const R eddington = R(4.0 * k::Pi * k::gravitationalConstant * k::massHydrogenAtom * k::gigaYear /
                            k::thomsonCrossSection / k::speedLight) * massBH;  // black_holes/fundamentals.F90:123-138
      const double eps = p.bh_efficiency_radiative;
      const double bhl = k::kilo * k::gigaYear / k::megaParsec * 4.0 * k::Pi;  // Bondi_Hoyle_Lyttleton.F90:34-59
      // Spheroid gas.
      R rateSph = R(0.0);
      {
        double cs = sound_speed(p.bh_temperature_spheroid);
        R rAcc = xmax(R(G) * massBH / R(cs * cs), R(0.0));  // radialPosition = 0
        R rho = spheroid_gas_density(n, gasSph, rAcc);
        if (rho > R(1.0)) {
          R jeans = R(cs / std::sqrt(G)) / xsqrt(rho);  // Ideal_Gas_Jeans_Length (thermodynamics/ideal_gases.F90:34-44)
          jeans = xmin(jeans, R(n.radiusSpheroid));
          if (jeans > rAcc) rho = spheroid_gas_density(n, gasSph, jeans);
          // velocity relative = 0: (G M)^2 rho / cs^3
          rateSph = xmax(R(p.bh_enhancement_spheroid) * R(bhl * G * G) * massBH * massBH * rho / R(cs * cs * cs), R(0.0));
          if (eps > 0.0) rateSph = xmin(rateSph, eddington / R(eps));
        }
      }
      // Hot halo gas.
      R rateHot = R(0.0);
      {
        double T = n.temperatureVirial;
        double cs = sound_speed(T);
        R rAcc = T > 0.0 ? R(G) * massBH / R(cs * cs) : R(HUGE_VAL);
        rAcc = xmin(rAcc, R(n.radiusOuter));
        R fractionHot = R(1.0);
        if (p.bh_hot_mode_only) {
          // standardHotModeFraction (accretion_rates/standard.F90:442-468)
          R x = get_cooling_radius() / R(n.radiusVirial);
          if (x < R(0.9)) fractionHot = R(1.0);
          else if (x > R(1.0)) fractionHot = R(0.0);
          else {
            R u = (x - R(0.9)) / R(0.1);
            fractionHot = u * u * (R(2.0) * u - R(3.0)) + R(1.0);
          }
        }
        R rho = fractionHot * hot_density(n, massHot, rAcc);
        if (rho > R(1.0)) {
          rateHot = xmax(R(p.bh_enhancement_hot_halo) * R(bhl) * rAcc * rAcc * rho * R(cs), R(0.0));
          R maximum = xmax(massHot / (R(n.radiusOuter) / R(cs) * R(k::MpcPerKmPerSToGyr)), R(0.0));
          rateHot = xmin(rateHot, maximum);
          if (eps > 0.0) rateHot = xmin(rateHot, eddington / R(eps));
        }
      }
      R total = rateSph + rateHot;
      if (total > R(0.0)) {
        R reduced = total * R(1.0 - p.bh_efficiency_radiative - p.bh_efficiency_jet);
        if (!(massBH <= R(0.0) && reduced < R(0.0))) {
          dydt[GAL_Y_BLACK_HOLE] += reduced;
          // Node_Component_Spheroid_Standard_Mass_Gas_Sink_Rate (spheroid/standard/_class.F90:638-671)
          if (rateSph != R(0.0) && gasSph > R(0.0) && gasSph + y[GAL_Y_SPHEROID_STARS] > R(0.0)) {
            dydt[GAL_Y_SPHEROID_GAS] += -rateSph;
            dydt[GAL_Y_SPHEROID_GAS_METALS] += (-rateSph / gasSph) * y[GAL_Y_SPHEROID_GAS_METALS];
          }
          // Node_Component_Hot_Halo_Standard_Hot_Gas_All_Rate (hot_halo/standard/_class.F90:771-799)
          if (rateHot != R(0.0) && massHot > R(0.0)) {
            dydt[GAL_Y_HOT_MASS] += -rateHot;
            dydt[GAL_Y_HOT_METALS] += metalsHot * (-rateHot / massHot);
          }
        }
      }
    }
    // --- CGMAccretion (circumgalactic_medium/accretion.F90:517-593) with
    //     accretionHaloSimple (accretion/halo/simple.F90:281-319): failed fraction 0,
    //     primordial (metal-free) accretion, negative accretion not allowed.
    if (ph & GAL_PHYS_CGM_ACCRETION) {
      R rate = n.massRate > 0.0 ? R(p.omega_baryon / p.omega_matter) * R(n.massRate) : R(0.0);
      dydt[GAL_Y_HOT_MASS] += rate;
    }
    // --- CGMOutflowReincorporation (circumgalactic_medium/outflow_reincorporation.F90:272-349)
    //     with haloDynamicalTime (hot_halo/outflow_reincorporation/halo_dynamical_time.F90:113-128).
    if (ph & GAL_PHYS_REINCORPORATION) {
      R massOut = y[GAL_Y_OUTFLOWED_MASS];
      if (massOut > R(0.0)) {
        R rate = massOut * R(p.reincorporation_multiplier) / R(n.timeDynamical);
        R metals = rate * y[GAL_Y_OUTFLOWED_METALS] / massOut;
        dydt[GAL_Y_OUTFLOWED_MASS] += -rate;
        dydt[GAL_Y_OUTFLOWED_METALS] += -metals;
        dydt[GAL_Y_HOT_MASS] += rate;
        dydt[GAL_Y_HOT_METALS] += metals;
      }
    }
    // --- CGMCoolingHeating (circumgalactic_medium/cooling_heating.F90:216-381), heating zero,
    //     cooling onto the disk, coolingRateWhiteFrenk1991 (cooling/cooling_rate/White-Frenk.F90:132-185).
    if ((ph & GAL_PHYS_COOLING) && massHot > R(0.0) && n.radiusOuter > 0.0) {
      R rate = R(0.0);
      if (!(n.velocityVirial > p.cooling_velocity_cutoff)) {
        R rCool = get_cooling_radius();
        if (rCool >= R(n.radiusOuter)) {
          rate = massHot / R(n.timeDynamical);
        } else {
          // simpleRadiusGrowthRate (cooling_radius/simple.F90:229-311): isothermal profile,
          // dln t_cool/dln rho = 1 - 2, temperature slope zero, dt_avail/dt = 1.
          R growth = R(0.0);
          if (rCool > R(0.0)) {
            R x = rCool / R(n.radiusCore);
            R densityLogSlope = R(-3.0 * (2.0 / 3.0)) * x * x / (x * x + R(1.0));
            R slope = densityLogSlope * R(-1.0);
            if (slope != R(0.0)) growth = rCool / R(n.timeDynamical) * R(1.0) / slope;
          }
          rate = R(4.0 * k::Pi) * rCool * rCool * hot_density(n, massHot, rCool) * growth;
        }
      }
      if (rate > R(0.0)) {
        R metals = rate * metalsHot / massHot;
        dydt[GAL_Y_HOT_MASS] += -rate;
        dydt[GAL_Y_HOT_METALS] += -metals;
        dydt[GAL_Y_DISK_GAS] += rate;
        dydt[GAL_Y_DISK_GAS_METALS] += metals;
      }
    }
  }
};

// Post-step clamps of the standard components (return value: status after
// the clamps; GSL_Continue is mapped to success as in
// standardPostStepProcessing, node_evolver/standard.F90:1160-1185).
template <class R>
static void post_step(R* y) {
  // Node_Component_Hot_Halo_Standard_Post_Step (hot_halo/standard/_class.F90:455-530)
  if (y[GAL_Y_HOT_MASS] < R(0.0)) y[GAL_Y_HOT_MASS] = R(0.0);
  // Node_Component_Disk_Standard_Post_Step (disk/standard/_class.F90:473-677)
  if (y[GAL_Y_DISK_GAS] < R(0.0)) {
    if (y[GAL_Y_DISK_GAS] + y[GAL_Y_DISK_STARS] == R(0.0)) {
      y[GAL_Y_DISK_STARS] = R(0.0);
      y[GAL_Y_DISK_STARS_METALS] = R(0.0);
    }
    y[GAL_Y_DISK_GAS] = R(0.0);
    y[GAL_Y_DISK_GAS_METALS] = R(0.0);
  }
  if (y[GAL_Y_DISK_STARS] < R(0.0)) {
    if (y[GAL_Y_DISK_GAS] + y[GAL_Y_DISK_STARS] == R(0.0)) {
      y[GAL_Y_DISK_GAS] = R(0.0);
      y[GAL_Y_DISK_GAS_METALS] = R(0.0);
    }
    y[GAL_Y_DISK_STARS] = R(0.0);
    y[GAL_Y_DISK_STARS_METALS] = R(0.0);
  }
  // Node_Component_Spheroid_Standard_Post_Step (spheroid/standard/_class.F90:464-636)
  if (y[GAL_Y_SPHEROID_GAS] < R(0.0)) {
    if (y[GAL_Y_SPHEROID_GAS] + y[GAL_Y_SPHEROID_STARS] == R(0.0)) y[GAL_Y_SPHEROID_STARS] = R(0.0);
    y[GAL_Y_SPHEROID_GAS] = R(0.0);
    y[GAL_Y_SPHEROID_GAS_METALS] = R(0.0);
  }
  if (y[GAL_Y_SPHEROID_STARS] < R(0.0)) {
    if (y[GAL_Y_SPHEROID_GAS] + y[GAL_Y_SPHEROID_STARS] == R(0.0)) {
      y[GAL_Y_SPHEROID_GAS] = R(0.0);
      y[GAL_Y_SPHEROID_GAS_METALS] = R(0.0);
    }
    y[GAL_Y_SPHEROID_STARS] = R(0.0);
  }
}

// Absolute-tolerance scales, set once per evolve call from the initial
// state (scaleSetTask hooks): hot halo (hot_halo/standard/_class.F90:804-850),
// disk (disk/standard/_class.F90:735-824), spheroid
// (spheroid/standard/_class.F90:804-897), black hole
// (black_hole/standard/_class.F90:195-257).
static void scales(const double* y, double massHalo, double* s) {
  double hot = massHalo * 1.0e-3;
  s[GAL_Y_HOT_MASS] = s[GAL_Y_HOT_METALS] = s[GAL_Y_OUTFLOWED_MASS] = s[GAL_Y_OUTFLOWED_METALS] = hot;
  double mass = std::max(std::fabs(y[GAL_Y_DISK_GAS]) + std::fabs(y[GAL_Y_SPHEROID_GAS]) + std::fabs(y[GAL_Y_DISK_STARS]) +
                             std::fabs(y[GAL_Y_SPHEROID_STARS]),
                         1.0);
  double metals = std::max(std::fabs(y[GAL_Y_DISK_GAS_METALS]) + std::fabs(y[GAL_Y_DISK_STARS_METALS]) +
                               std::fabs(y[GAL_Y_SPHEROID_GAS_METALS]),
                           std::max(mass * 1.0e-4, 1.0));
  s[GAL_Y_DISK_GAS] = s[GAL_Y_DISK_STARS] = s[GAL_Y_SPHEROID_GAS] = s[GAL_Y_SPHEROID_STARS] = mass;
  s[GAL_Y_DISK_GAS_METALS] = s[GAL_Y_DISK_STARS_METALS] = s[GAL_Y_SPHEROID_GAS_METALS] = metals;
  double stars = y[GAL_Y_SPHEROID_STARS] > 0.0 ? y[GAL_Y_SPHEROID_STARS] : 0.0;
  s[GAL_Y_BLACK_HOLE] = std::max(std::max(1.0, 1.0e-4 * stars), y[GAL_Y_BLACK_HOLE]);
}

// ---------------------------------------------------------------------------
// Generic ODE machinery (dimension up to 16).
// ---------------------------------------------------------------------------
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_BUDGET = -2 };  // GSL_BUDGET: step budget used up
enum { HADJ_DEC = -1, HADJ_NIL = 0, HADJ_INC = 1 };
const int MAXDIM = 16;

// Cash-Karp 4(5) tableau (Cash & Karp 1990).
namespace ck {
const double a2 = 1.0 / 5.0, a3 = 3.0 / 10.0, a4 = 3.0 / 5.0, a5 = 1.0, a6 = 7.0 / 8.0;
const double b21 = 1.0 / 5.0;
const double b31 = 3.0 / 40.0, b32 = 9.0 / 40.0;
const double b41 = 3.0 / 10.0, b42 = -9.0 / 10.0, b43 = 6.0 / 5.0;
const double b51 = -11.0 / 54.0, b52 = 5.0 / 2.0, b53 = -70.0 / 27.0, b54 = 35.0 / 27.0;
const double b61 = 1631.0 / 55296.0, b62 = 175.0 / 512.0, b63 = 575.0 / 13824.0, b64 = 44275.0 / 110592.0, b65 = 253.0 / 4096.0;
const double c1 = 37.0 / 378.0, c3 = 250.0 / 621.0, c4 = 125.0 / 594.0, c6 = 512.0 / 1771.0;
const double e1 = 37.0 / 378.0 - 2825.0 / 27648.0, e3 = 250.0 / 621.0 - 18575.0 / 48384.0,
             e4 = 125.0 / 594.0 - 13525.0 / 55296.0, e5 = -277.0 / 14336.0, e6 = 512.0 / 1771.0 - 0.25;
const unsigned order = 5;  // order reported by GSL's rkck stepper to the controller
}  // namespace ck

// sc2_control_hadjust (external/gslODEInitVal2/cscal2.c:93-169) with
// a_y=1, a_dydt=0 (numerical/ODE_solver/solver.F90:365-366) and no
// non-negativity constraints (enforceNonNegativity=false by default).
template <class R>
static int control_hadjust(int dim, const R* y, const R* yerr, double epsAbs, double epsRel, const double* scale, R& h) {
  const R hOld = h;
  R rmax = R(DBL_MIN);
  for (int i = 0; i < dim; ++i) {
    R D0 = R(epsRel) * xabs(y[i]) + R(epsAbs) * R(scale[i]);
    R r = xabs(yerr[i]) / xabs(D0);
    rmax = xmax(r, rmax);
  }
  if (rmax > R(1.1)) {
    R r = R(0.9) / xpow(rmax, R(1.0 / (double)ck::order));
    if (r < R(0.2)) r = R(0.2);
    h = r * hOld;
    return HADJ_DEC;
  } else if (rmax < R(0.5)) {
    R r = R(0.9) / xpow(rmax, R(1.0 / ((double)ck::order + 1.0)));
    if (r > R(4.9)) r = R(4.9);
    if (r < R(1.0)) r = R(1.0);
    h = r * hOld;
    return HADJ_INC;
  }
  return HADJ_NIL;
}

template <class R, class F>
struct Solver {
  int dim;
  F& f;
  double epsAbs, epsRel;
  const double* scale;
  bool hasPostStep;
  uint64_t budget = 0;  // attempted-step budget per solve (0: unlimited)
  // evolve state
  uint64_t count = 0, failed = 0, accepted = 0;
  R dydtIn[MAXDIM], dydtOut[MAXDIM], yerr[MAXDIM], y0[MAXDIM];
  R k2[MAXDIM], k3[MAXDIM], k4[MAXDIM], k5[MAXDIM], k6[MAXDIM], tmp[MAXDIM];

  // One Cash-Karp step of size h from (t, y) with k1 = dydtIn; y is
  // replaced by the 5th-order solution and yerr by the embedded error.
  void step(R t, R h, R* y) {
    const R* k1 = dydtIn;
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + R(ck::b21) * h * k1[i];
    f(t + R(ck::a2) * h, tmp, k2);
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + h * (R(ck::b31) * k1[i] + R(ck::b32) * k2[i]);
    f(t + R(ck::a3) * h, tmp, k3);
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + h * (R(ck::b41) * k1[i] + R(ck::b42) * k2[i] + R(ck::b43) * k3[i]);
    f(t + R(ck::a4) * h, tmp, k4);
    for (int i = 0; i < dim; ++i)
      tmp[i] = y[i] + h * (R(ck::b51) * k1[i] + R(ck::b52) * k2[i] + R(ck::b53) * k3[i] + R(ck::b54) * k4[i]);
    f(t + R(ck::a5) * h, tmp, k5);
    for (int i = 0; i < dim; ++i)
      tmp[i] = y[i] + h * (R(ck::b61) * k1[i] + R(ck::b62) * k2[i] + R(ck::b63) * k3[i] + R(ck::b64) * k4[i] + R(ck::b65) * k5[i]);
    f(t + R(ck::a6) * h, tmp, k6);
    for (int i = 0; i < dim; ++i) {
      R d = R(ck::c1) * k1[i] + R(ck::c3) * k3[i] + R(ck::c4) * k4[i] + R(ck::c6) * k6[i];
      y[i] = y[i] + h * d;
    }
    // dydt_out = f(t+h, y) is evaluated by evolve_apply once the step is
    // accepted (it does not enter the error control, a_dydt = 0).
    for (int i = 0; i < dim; ++i)
      yerr[i] = h * (R(ck::e1) * k1[i] + R(ck::e3) * k3[i] + R(ck::e4) * k4[i] + R(ck::e5) * k5[i] + R(ck::e6) * k6[i]);
  }

  // The step-size controller (control_hadjust).
  int hadjust(const R* y, R& h) { return control_hadjust(dim, y, yerr, epsAbs, epsRel, scale, h); }

  // gsl_odeiv2_evolve_apply for a stepper that can use dydt_in (GSL manual,
  // "Evolution"): take one accepted step from *t toward t1, retrying with the
  // controller's smaller step after a rejection.
  int evolve_apply(R& t, R t1, R& h, R* y) {
    const R t0 = t;
    R h0 = h;
    R dt = t1 - t0;
    for (int i = 0; i < dim; ++i) y0[i] = y[i];
    if (count == 0) f(t0, y, dydtIn);
    else for (int i = 0; i < dim; ++i) dydtIn[i] = dydtOut[i];
    for (;;) {
      bool finalStep;
      if ((dt >= R(0.0) && h0 > dt) || (dt < R(0.0) && h0 < dt)) {
        h0 = dt;
        finalStep = true;
      } else {
        finalStep = false;
      }
      step(t0, h0, y);
      ++count;
      t = finalStep ? t1 : t0 + h0;
      R hOld = h0;
      int status = hadjust(y, h0);
      if (status == HADJ_DEC) {
        volatile double tCurr = val(t), tNext = val(t + h0);
        if (xabs(h0) < xabs(hOld) && tNext != tCurr) {
          for (int i = 0; i < dim; ++i) y[i] = y0[i];
          ++failed;
          if (budget && count >= budget) return GSL_BUDGET;
          continue;
        }
        h = hOld;
        return GSL_FAILURE;
      }
      ++accepted;
      h = h0;
      // dydt_out at the accepted point, the next step's dydt_in.  Not needed
      // after the final step of the interval, which ends the solve.
      if (!finalStep && t != t1) f(t, y, dydtOut);
      return GSL_SUCCESS;
    }
  }

  // gsl_odeiv2_driver2_apply (external/gslODEInitVal2/driver2.c:148-250)
  // with the post-step hook; no latent integrator, hmax unlimited.
  template <class P>
  int driver_apply(R& t, R t1, R& h, R* y, P postStep, uint64_t stepBudget, bool& budgetExhausted) {
    int sign = h > R(0.0) ? 1 : -1;
    budget = stepBudget;
    while (R((double)sign) * (t1 - t) > R(0.0)) {
      int s = evolve_apply(t, t1, h, y);
      if (s == GSL_BUDGET) {
        budgetExhausted = true;
        return GSL_FAILURE;
      }
      if (s != GSL_SUCCESS) return s;
      if (hasPostStep) postStep(y);  // clamps return GSL_Continue -> no evolver reset
      if (stepBudget && count >= stepBudget && R((double)sign) * (t1 - t) > R(0.0)) {
        budgetExhausted = true;
        return GSL_FAILURE;
      }
    }
    return GSL_SUCCESS;
  }
};

// One node: mergerTreeNodeEvolverStandard%evolve (node_evolver/standard.F90:
// 385-755) restricted to the non-interrupted, non-Jacobian path, with the
// trial loop of :587-706 and odeSolver%solve (numerical/ODE_solver/
// solver.F90:492-691).
template <class R>
static int evolve_node(const gal_params& p, const Table& tb, const double* prm, double* yio, double t0, double t1,
                       double& stepInOut, uint32_t counters[3], bool brent, uint64_t* rhsOut = nullptr) {
  Node n;
  node_setup(p, prm, n);
  double s[GAL_NY];
  scales(yio, n.massHalo, s);
  Rhs<R> rhs{p, tb, n, brent};
  int status = GAL_STATUS_SUCCESS;
  uint32_t nAcc = 0, nRej = 0;
  double stepSize = -1.0;
  if (t0 != t1) {
    int trial = 0;
    int ode = GSL_FAILURE;
    double ysave[GAL_NY];
    for (int i = 0; i < GAL_NY; ++i) ysave[i] = yio[i];
    while (trial < p.trial_count_maximum && ode != GSL_SUCCESS) {
      stepSize = p.reuse_step_size ? stepInOut / std::ldexp(1.0, trial) : -1.0;
      // odeSolverSolve: initial step min(xStep, x1-x0) when xStep > 0.
      double hStart = t1 - t0;
      if (stepSize > 0.0) hStart = std::min(stepSize, hStart);
      Solver<R, Rhs<R>> sv{GAL_NY, rhs, p.ode_tolerance_absolute, p.ode_tolerance_relative, s, true};
      R y[GAL_NY];
      for (int i = 0; i < GAL_NY; ++i) y[i] = R(yio[i]);
      R t = R(t0), h = R(hStart);
      bool exhausted = false;
      ode = sv.driver_apply(t, R(t1), h, y, [](R* yy) { post_step(yy); }, (uint64_t)p.step_budget, exhausted);
      nAcc += (uint32_t)sv.accepted;
      nRej += (uint32_t)sv.failed;
      if (exhausted) {
        for (int i = 0; i < GAL_NY; ++i) yio[i] = ysave[i];
        status = GAL_STATUS_XCPU;
        break;
      }
      if (ode == GSL_SUCCESS) {
        for (int i = 0; i < GAL_NY; ++i) yio[i] = val(y[i]);
        stepSize = val(h);
      } else {
        ++trial;
        for (int i = 0; i < GAL_NY; ++i) yio[i] = ysave[i];
      }
    }
    if (status == GAL_STATUS_SUCCESS && ode != GSL_SUCCESS) status = GAL_STATUS_UNDERFLOW;
  }
  if (status == GAL_STATUS_SUCCESS) {
    for (int i = 0; i < GAL_NY; ++i)
      if (!std::isfinite(yio[i])) status = GAL_STATUS_NOT_FINITE;
    stepInOut = stepSize;  // node%timeStepSet(stepSize)
  }
  if (counters) {
    counters[0] = nAcc;
    counters[1] = nRej;
    counters[2] = (uint32_t)rhs.evaluations;
  }
  if (rhsOut) *rhsOut = rhs.evaluations;
  return status;
}

// ---------------------------------------------------------------------------
// Interrupts: a node operator may interrupt the integration (the null
// component's rate functions do so to create a component that receives a
// rate, e.g. cooling into a disk that does not exist yet).  standardODEs
// (node_evolver/standard.F90:895-945) returns zero derivatives from an
// evaluation that requests one and, when it is the earliest so far, records
// its time and task and returns odeSolverInterrupt (= GSL_EBADFUNC,
// numerical/ODE_solver/error_codes.F90:33); GSL's rkck and evolve_apply
// abandon the step (the state stays at its start); odeSolver%solve
// (solver.F90:608-620) then re-targets the integration to the interrupt time
// and carries on, every evaluation at or after that time returning zero
// derivatives; evolve (standard.F90:575-578, 729-737) reports the node as
// interrupted at that time with node%timeStep = -1.  The stepper evaluates
// dydt_out = f(t+h, y_new) on every attempt, as GSL's rkck does, since that
// evaluation can interrupt too.  After an abandoned attempt the next one
// starts from the same (t, y) and its derivative.  The interrupt time and
// task persist over the trials of one evolve call; a trial restarted after
// an interrupt integrates to the interrupt time (the reference integrates
// on to the end with zero derivatives beyond it, which leaves the state at
// the interrupt time up to the steps that straddle it).
// ---------------------------------------------------------------------------
enum { GSL_INTERRUPT = -3 };

struct Interrupts {
  uint32_t components;  // GAL_COMPONENT_* of the components that exist
  bool found = false;
  double time = 0.0;
  int32_t task = 0;     // GAL_INTERRUPT_* of the earliest interrupt
};

// The components to create for one evaluation: those that do not exist and
// receive a non-zero rate in one of their properties.
static int32_t interrupt_request(uint32_t components, const double* d) {
  int32_t task = 0;
  if (!(components & GAL_COMPONENT_DISK) && (d[GAL_Y_DISK_GAS] != 0.0 || d[GAL_Y_DISK_GAS_METALS] != 0.0 ||
                                             d[GAL_Y_DISK_STARS] != 0.0 || d[GAL_Y_DISK_STARS_METALS] != 0.0))
    task |= GAL_INTERRUPT_CREATE_DISK;
  if (!(components & GAL_COMPONENT_SPHEROID) &&
      (d[GAL_Y_SPHEROID_GAS] != 0.0 || d[GAL_Y_SPHEROID_GAS_METALS] != 0.0 || d[GAL_Y_SPHEROID_STARS] != 0.0))
    task |= GAL_INTERRUPT_CREATE_SPHEROID;
  if (!(components & GAL_COMPONENT_BLACK_HOLE) && d[GAL_Y_BLACK_HOLE] != 0.0) task |= GAL_INTERRUPT_CREATE_BLACK_HOLE;
  return task;
}

template <class F>
struct SolverI {
  int dim;
  F& f;
  Interrupts& in;
  double epsAbs, epsRel;
  const double* scale;
  uint64_t budget = 0;
  uint64_t count = 0, failed = 0, accepted = 0;
  bool haveDydtIn = false;  // dydtIn holds f at the current (t, y)
  double dydtIn[MAXDIM], dydtOut[MAXDIM], yerr[MAXDIM];
  double k2[MAXDIM], k3[MAXDIM], k4[MAXDIM], k5[MAXDIM], k6[MAXDIM], tmp[MAXDIM];

  // One evaluation at time ts (standardODEs): zero beyond the first
  // interrupt; true when it requests the earliest interrupt so far.
  bool eval(double ts, const double* y, double* d) {
    if (in.found && ts >= in.time) {
      for (int i = 0; i < dim; ++i) d[i] = 0.0;
      return false;
    }
    f(ts, y, d);
    const int32_t req = interrupt_request(in.components, d);
    if (req) {
      for (int i = 0; i < dim; ++i) d[i] = 0.0;
      if (!in.found || ts < in.time) {
        in.found = true;
        in.time = ts;
        in.task = req;
        return true;
      }
    }
    return false;
  }

  // rkck_apply with dydt_out: true when an evaluation interrupts (y untouched).
  bool step(double t, double h, const double* y, double* yn) {
    const double* k1 = dydtIn;
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + ck::b21 * h * k1[i];
    if (eval(t + ck::a2 * h, tmp, k2)) return true;
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + h * (ck::b31 * k1[i] + ck::b32 * k2[i]);
    if (eval(t + ck::a3 * h, tmp, k3)) return true;
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + h * (ck::b41 * k1[i] + ck::b42 * k2[i] + ck::b43 * k3[i]);
    if (eval(t + ck::a4 * h, tmp, k4)) return true;
    for (int i = 0; i < dim; ++i) tmp[i] = y[i] + h * (ck::b51 * k1[i] + ck::b52 * k2[i] + ck::b53 * k3[i] + ck::b54 * k4[i]);
    if (eval(t + ck::a5 * h, tmp, k5)) return true;
    for (int i = 0; i < dim; ++i)
      tmp[i] = y[i] + h * (ck::b61 * k1[i] + ck::b62 * k2[i] + ck::b63 * k3[i] + ck::b64 * k4[i] + ck::b65 * k5[i]);
    if (eval(t + ck::a6 * h, tmp, k6)) return true;
    for (int i = 0; i < dim; ++i) yn[i] = y[i] + h * (ck::c1 * k1[i] + ck::c3 * k3[i] + ck::c4 * k4[i] + ck::c6 * k6[i]);
    if (eval(t + h, yn, dydtOut)) return true;
    for (int i = 0; i < dim; ++i)
      yerr[i] = h * (ck::e1 * k1[i] + ck::e3 * k3[i] + ck::e4 * k4[i] + ck::e5 * k5[i] + ck::e6 * k6[i]);
    return false;
  }

  int hadjust(const double* y, double& h) { return control_hadjust(dim, y, yerr, epsAbs, epsRel, scale, h); }

  int evolve_apply(double& t, double t1, double& h, double* y) {
    const double t0 = t;
    double h0 = h;
    const double dt = t1 - t0;
    if (!haveDydtIn) {
      if (eval(t0, y, dydtIn)) return GSL_INTERRUPT;
      haveDydtIn = true;
    }
    for (;;) {
      const bool finalStep = (dt >= 0.0 && h0 > dt) || (dt < 0.0 && h0 < dt);
      if (finalStep) h0 = dt;
      double yn[MAXDIM];
      if (step(t0, h0, y, yn)) return GSL_INTERRUPT;  // t, y and h as they were
      ++count;
      const double tNew = finalStep ? t1 : t0 + h0;
      const double hOld = h0;
      if (hadjust(yn, h0) == HADJ_DEC) {
        volatile double tCurr = tNew, tNext = tNew + h0;
        if (std::fabs(h0) < std::fabs(hOld) && tNext != tCurr) {
          ++failed;
          if (budget && count >= budget) return GSL_BUDGET;
          continue;
        }
        h = hOld;
        return GSL_FAILURE;
      }
      ++accepted;
      t = tNew;
      h = h0;
      for (int i = 0; i < dim; ++i) {
        y[i] = yn[i];
        dydtIn[i] = dydtOut[i];
      }
      return GSL_SUCCESS;
    }
  }

  // driver2_apply, then odeSolver%solve's re-targeting at each interrupt.
  int solve(double& t, double t1, double& h, double* y, uint64_t stepBudget, bool& budgetExhausted) {
    budget = stepBudget;
    double target = t1;
    while (target - t > 0.0) {
      const int s = evolve_apply(t, target, h, y);
      if (s == GSL_INTERRUPT) {
        target = in.time;
        continue;
      }
      if (s == GSL_BUDGET) {
        budgetExhausted = true;
        return GSL_FAILURE;
      }
      if (s != GSL_SUCCESS) return s;
      post_step(y);
      if (stepBudget && count >= stepBudget && target - t > 0.0) {
        budgetExhausted = true;
        return GSL_FAILURE;
      }
    }
    return GSL_SUCCESS;
  }
};

// evolve with interrupts (node_evolver/standard.F90:385-755 with the
// interrupted/functionInterrupt outputs): as evolve_node, plus the time
// reached and the interrupt task (0: not interrupted).
static int evolve_node_interruptible(const gal_params& p, const Table& tb, const double* prm, double* yio, double t0,
                                     double t1, double& stepInOut, uint32_t components, double& tReached,
                                     int32_t& task, uint32_t counters[3], bool brent) {
  Node n;
  node_setup(p, prm, n);
  double s[GAL_NY];
  scales(yio, n.massHalo, s);
  Rhs<double> rhs{p, tb, n, brent};
  Interrupts in{components};
  int status = GAL_STATUS_SUCCESS;
  uint32_t nAcc = 0, nRej = 0;
  double stepSize = -1.0;
  if (t0 != t1) {
    int trial = 0;
    int ode = GSL_FAILURE;
    double ysave[GAL_NY];
    for (int i = 0; i < GAL_NY; ++i) ysave[i] = yio[i];
    while (trial < p.trial_count_maximum && ode != GSL_SUCCESS) {
      stepSize = p.reuse_step_size ? stepInOut / std::ldexp(1.0, trial) : -1.0;
      const double target = in.found ? std::min(in.time, t1) : t1;
      double hStart = target - t0;
      if (stepSize > 0.0) hStart = std::min(stepSize, hStart);
      SolverI<Rhs<double>> sv{GAL_NY, rhs, in, p.ode_tolerance_absolute, p.ode_tolerance_relative, s};
      double y[GAL_NY];
      for (int i = 0; i < GAL_NY; ++i) y[i] = yio[i];
      double t = t0, h = hStart;
      bool exhausted = false;
      ode = target > t0 ? sv.solve(t, target, h, y, (uint64_t)p.step_budget, exhausted) : GSL_SUCCESS;
      nAcc += (uint32_t)sv.accepted;
      nRej += (uint32_t)sv.failed;
      if (exhausted) {
        for (int i = 0; i < GAL_NY; ++i) yio[i] = ysave[i];
        status = GAL_STATUS_XCPU;
        break;
      }
      if (ode == GSL_SUCCESS) {
        for (int i = 0; i < GAL_NY; ++i) yio[i] = y[i];
        stepSize = h;
      } else {
        ++trial;
        for (int i = 0; i < GAL_NY; ++i) yio[i] = ysave[i];
      }
    }
    if (status == GAL_STATUS_SUCCESS && ode != GSL_SUCCESS) status = GAL_STATUS_UNDERFLOW;
  }
  tReached = t1;
  task = 0;
  if (status == GAL_STATUS_SUCCESS) {
    for (int i = 0; i < GAL_NY; ++i)
      if (!std::isfinite(yio[i])) status = GAL_STATUS_NOT_FINITE;
    stepInOut = stepSize;  // node%timeStepSet(stepSize)
    if (status == GAL_STATUS_SUCCESS && in.found) {
      status = GAL_STATUS_INTERRUPTED;
      tReached = in.time;  // basic%timeSet(timeInterruptFirst)
      task = in.task;
      stepInOut = -1.0;    // node%timeStepSet(-1)
    }
  }
  if (counters) {
    counters[0] = nAcc;
    counters[1] = nRej;
    counters[2] = (uint32_t)rhs.evaluations;
  }
  return status;
}

// ---------------------------------------------------------------------------
// Forests: the tree evolver's node loop (merger_trees/evolver/standard.F90:
// 762-1035) over a whole forest.  A node evolves from its own time to its
// parent's, in pieces cut at the output times and at the timestep limit of
// mergerTreeEvolveTimestepSimple (each piece one evolve call,
// the step size carried over as node%timeStep), and on reaching the parent
// the primary progenitor's state is promoted and the other progenitors
// merge into it in index order (merge_satellite).
// ---------------------------------------------------------------------------
struct Cosmology {
  double om, ol, h0;
  double hubbleGyr() const { return h0 / (1.0e6 * 3.08567758135e16 / 1.0e3 / (1.0e9 * 3.15581497635456e7)); }
  // cosmologyFunctionsMatterLambda for a flat model: a(t) from the analytic solution.
  double redshift(double t) const {
    const double x = std::sinh(1.5 * hubbleGyr() * std::sqrt(ol) * t);
    return 1.0 / std::pow(x / std::sqrt(ol / om), 2.0 / 3.0) - 1.0;
  }
  // mergerTreeEvolveTimestepSimple%timeEvolveTo (merger_trees/evolve/
  // timesteps/simple.F90:124-161): a node at time t may be evolved to at most
  // t + min(relative / H(t), absolute), H = expansionRate(a(t)) (1/Gyr).
  double step_limit(double t, double relative, double absolute) const {
    if (!(relative > 0.0)) return absolute;
    const double zp = 1.0 + redshift(t);
    const double rate = hubbleGyr() * std::sqrt(om * zp * zp * zp + ol);
    return std::min(relative / rate, absolute);
  }
  // Bryan & Norman (1998) contrast relative to the mean density
  // (virial_density_contrast/Bryan_Norman.F90:172-196); r_vir and V_vir.
  void virial(double M, double z, double& r, double& v) const {
    const double G = 6.673e-11 * 1.98892e30 / 1.0e6 / (1.0e6 * 3.08567758135e16);
    const double zp = (1.0 + z) * (1.0 + z) * (1.0 + z);
    const double omz = om * zp / (om * zp + ol);
    const double x = omz - 1.0;
    const double contrast = (18.0 * M_PI * M_PI + 82.0 * x - 39.0 * x * x) / (x + 1.0);
    const double rhoMean = om * 3.0 * h0 * h0 / (8.0 * M_PI * G) * zp;
    r = std::cbrt(3.0 * M / (4.0 * M_PI * contrast * rhoMean));
    v = std::sqrt(G * M / r);
  }
};

struct ForestIn {
  int64_t n;
  const int32_t *parent, *childFirst, *childCount;
  const double *time, *mass, *spin, *state0;
  int32_t nOut;
  const double* tOut;
  const int32_t* satHost;      // host at infall of a satellite phase, else -1 (NULL: no satellites)
  std::vector<double> massIn;  // mass of the satellites falling into each node at its time
  bool satellite(int64_t i) const { return satHost && satHost[i] >= 0; }
};

// A secondary progenitor merging into the primary at their parent's time:
// mergerMassMovementsSimple%get (satellites/merging/mass_movements/simple.F90,
// defaults massRatioMajorMerger = 0.25, destinationGasMinorMerger =
// destinationStarsMinorMerger = spheroid): in a major merger (the smaller
// galaxy, disk plus spheroid, at least the ratio times the larger) both
// galaxies go to the remnant's spheroid, in a minor one the satellite's
// gas and stars go to the host's spheroid and the host is unmoved.  The
// satellite's hot halo and outflowed gas join the host's, and the black
// holes merge (masses add).  The state holds no spheroid stellar metals, so
// a disk's stellar metals leave it when its stars move to the spheroid.
// `sat` is the satellite's column of an [NY][n] array.
static void merge_satellite(const gal_params& p, double* y, const double* sat, int64_t n) {
  double s[GAL_NY];
  for (int v = 0; v < GAL_NY; ++v) s[v] = sat[v * n];
  const double massHost = y[GAL_Y_DISK_GAS] + y[GAL_Y_DISK_STARS] + y[GAL_Y_SPHEROID_GAS] + y[GAL_Y_SPHEROID_STARS];
  const double massSat = s[GAL_Y_DISK_GAS] + s[GAL_Y_DISK_STARS] + s[GAL_Y_SPHEROID_GAS] + s[GAL_Y_SPHEROID_STARS];
  const bool major = massSat > 0.0 && massHost > 0.0 &&
                     std::min(massSat, massHost) >= p.merger_mass_ratio_major * std::max(massSat, massHost);
  for (int v : {GAL_Y_HOT_MASS, GAL_Y_HOT_METALS, GAL_Y_OUTFLOWED_MASS, GAL_Y_OUTFLOWED_METALS, GAL_Y_BLACK_HOLE}) y[v] += s[v];
  y[GAL_Y_SPHEROID_GAS] += s[GAL_Y_DISK_GAS] + s[GAL_Y_SPHEROID_GAS];
  y[GAL_Y_SPHEROID_GAS_METALS] += s[GAL_Y_DISK_GAS_METALS] + s[GAL_Y_SPHEROID_GAS_METALS];
  y[GAL_Y_SPHEROID_STARS] += s[GAL_Y_DISK_STARS] + s[GAL_Y_SPHEROID_STARS];
  if (major) {
    y[GAL_Y_SPHEROID_GAS] += y[GAL_Y_DISK_GAS];
    y[GAL_Y_SPHEROID_GAS_METALS] += y[GAL_Y_DISK_GAS_METALS];
    y[GAL_Y_SPHEROID_STARS] += y[GAL_Y_DISK_STARS];
    y[GAL_Y_DISK_GAS] = y[GAL_Y_DISK_GAS_METALS] = y[GAL_Y_DISK_STARS] = y[GAL_Y_DISK_STARS_METALS] = 0.0;
  }
}

// Evolve one node of a forest whose progenitors are done; y holds its
// initial state, stepIo the carried step size.
static int evolve_forest_node(const gal_params& p, const Table& tb, const Cosmology& cos, const ForestIn& F, int64_t i,
                              double* y, double& stepIo, uint32_t counters[3], bool brent,
                              const std::vector<int64_t>& snapFirst, double* snapshot, int64_t snapTotal) {
  const int32_t par = F.parent[i];
  const double t0 = F.time[i], t1 = par >= 0 ? F.time[par] : F.time[i];
  const bool primary = par >= 0 && F.childFirst[par] == i;
  // dmoInterpolateNodeInitialize (nodes/operators/physics/dark_matter_only_
  // mass/interpolate.F90:118-168): the primary progenitor's mass grows by
  // its parent's unresolved mass (beyond its progenitors' and the
  // satellites falling in) at a constant rate; other progenitors and
  // satellites (isSatellite: accretion zero) keep their mass.
  double massEnd = F.mass[i], accretion = 0.0;
  if (primary && t1 > t0 && !F.satellite(i)) {
    double brought = F.massIn[(size_t)par];
    for (int32_t c = 0; c < F.childCount[par]; ++c)
      if (!F.satellite(F.childFirst[par] + c)) brought += F.mass[F.childFirst[par] + c];
    accretion = std::max(F.mass[par] - brought, 0.0) / (t1 - t0);
    massEnd = F.mass[i] + accretion * (t1 - t0);
  }
  // A satellite's dark-matter halo scales are those at its infall (its time
  // of last isolation).
  const double zFrozen = F.satellite(i) ? cos.redshift(t0) : 0.0;
  int64_t slot = snapFirst[i];
  auto snap = [&](const double* v) {
    for (int k = 0; k < GAL_NY; ++k) snapshot[k * snapTotal + slot] = v[k];
    ++slot;
  };
  for (int32_t k = 0; k < F.nOut; ++k)
    if (F.tOut[k] == t0 && (par < 0 || t0 < t1)) snap(y);
  counters[0] = counters[1] = counters[2] = 0;
  int status = GAL_STATUS_SUCCESS;
  double a = t0;
  int32_t k = 0;
  while (k < F.nOut && !(F.tOut[k] > t0)) ++k;
  while (a < t1 && status == GAL_STATUS_SUCCESS) {
    // timeEvolveTo (merger_trees/evolver/standard.F90:762-1035): the earliest
    // of the parent's time, the next output and the timestep criterion.
    const double limit = a + cos.step_limit(a, p.timestep_relative, p.timestep_absolute);
    const bool atOutput = k < F.nOut && F.tOut[k] < t1 && !(limit < F.tOut[k]);
    const double b = atOutput ? F.tOut[k] : std::min(limit, t1);
    const double M = F.mass[i] + (massEnd - F.mass[i]) * (a - t0) / (t1 - t0);
    double prm[GAL_NP];
    double r, v;
    cos.virial(M, F.satellite(i) ? zFrozen : cos.redshift(a), r, v);
    prm[GAL_P_MASS] = M;
    prm[GAL_P_MASS_RATE] = accretion;
    prm[GAL_P_RADIUS_VIRIAL] = r;
    prm[GAL_P_VELOCITY_VIRIAL] = v;
    prm[GAL_P_SPIN] = F.spin[i];
    uint32_t c[3];
    status = evolve_node<double>(p, tb, prm, y, a, b, stepIo, c, brent);
    for (int j = 0; j < 3; ++j) counters[j] += c[j];
    if (status == GAL_STATUS_SUCCESS && atOutput) snap(y);
    a = b;
    if (atOutput) ++k;
  }
  return status;
}

}  // namespace orc

// ===========================================================================
// C interface used by the tests and by bench.py's CPU baseline.
// ===========================================================================
extern "C" {

// Evolve a batch of nodes on the host with `threads` OpenMP threads
// (<= 0: all).  Same arrays and semantics as gal_gpu_evolve_batch.  With
// cooling_brent != 0 the cooling radius is found by Brent's method as in the
// reference; otherwise by its closed form.
int oracle_evolve_batch(const gal_params* p, const gal_cie_table* table, int64_t n, double* state, const double* param,
                        const double* t_start, const double* t_end, double* step, int32_t* status, uint32_t* counters,
                        int threads, int cooling_brent) {
  if (!p || !table || n < 0) return GAL_ERR_ARGUMENT;
  orc::Table tb;
  int rc = orc::table_load(table, tb);
  if (rc) return rc;
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (int64_t i = 0; i < n; ++i) {
    double y[GAL_NY], prm[GAL_NP];
    for (int v = 0; v < GAL_NY; ++v) y[v] = state[v * n + i];
    for (int v = 0; v < GAL_NP; ++v) prm[v] = param[v * n + i];
    double h = step[i];
    uint32_t c[3];
    int s = orc::evolve_node<double>(*p, tb, prm, y, t_start[i], t_end[i], h, c, cooling_brent != 0);
    for (int v = 0; v < GAL_NY; ++v) state[v * n + i] = y[v];
    step[i] = h;
    status[i] = s;
    if (counters)
      for (int v = 0; v < 3; ++v) counters[v * n + i] = c[v];
  }
  return GAL_OK;
}

// Evolve a batch with interrupts (gal_gpu_evolve_batch_interrupt's arrays).
int oracle_evolve_batch_interrupt(const gal_params* p, const gal_cie_table* table, int64_t n, double* state,
                                  const double* param, const double* t_start, const double* t_end, double* step,
                                  const int32_t* components, int32_t* status, uint32_t* counters, double* t_reached,
                                  int32_t* task, int threads, int cooling_brent) {
  if (!p || !table || n < 0 || !components || !t_reached || !task) return GAL_ERR_ARGUMENT;
  orc::Table tb;
  int rc = orc::table_load(table, tb);
  if (rc) return rc;
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (int64_t i = 0; i < n; ++i) {
    double y[GAL_NY], prm[GAL_NP];
    for (int v = 0; v < GAL_NY; ++v) y[v] = state[v * n + i];
    for (int v = 0; v < GAL_NP; ++v) prm[v] = param[v * n + i];
    double h = step[i];
    uint32_t c[3];
    double tr = 0.0;
    int32_t tk = 0;
    int s = orc::evolve_node_interruptible(*p, tb, prm, y, t_start[i], t_end[i], h, (uint32_t)components[i], tr, tk, c,
                                           cooling_brent != 0);
    for (int v = 0; v < GAL_NY; ++v) state[v * n + i] = y[v];
    step[i] = h;
    status[i] = s;
    t_reached[i] = tr;
    task[i] = tk;
    if (counters)
      for (int v = 0; v < 3; ++v) counters[v * n + i] = c[v];
  }
  return GAL_OK;
}

// Cooling function, electron density and cooling radius of the oracle, for
// unit tests of the table interpolation.
double oracle_cooling_function(const gal_cie_table* table, double nH, double T, double Zsolar) {
  orc::Table tb;
  if (orc::table_load(table, tb)) return -1.0;
  return orc::cooling_function<double>(tb, nH, T, Zsolar);
}
double oracle_electron_density(const gal_cie_table* table, double nH, double T, double Zsolar) {
  orc::Table tb;
  if (orc::table_load(table, tb)) return -1.0;
  return orc::electron_density<double>(tb, nH, T, Zsolar);
}
double oracle_cooling_radius(const gal_params* p, const gal_cie_table* table, const double* param, double massHot,
                             double metalsHot, int brent) {
  orc::Table tb;
  if (orc::table_load(table, tb)) return -1.0;
  orc::Node n;
  orc::node_setup(*p, param, n);
  orc::Rhs<double> rhs{*p, tb, n, brent != 0};
  return rhs.cooling_radius(massHot, orc::mass_fraction(metalsHot, massHot));
}

// Right-hand side at one state (for derivative-level tests).
int oracle_rhs(const gal_params* p, const gal_cie_table* table, const double* param, const double* y, double* dydt) {
  orc::Table tb;
  int rc = orc::table_load(table, tb);
  if (rc) return rc;
  orc::Node n;
  orc::node_setup(*p, param, n);
  orc::Rhs<double> rhs{*p, tb, n, true};
  rhs(0.0, y, dydt);
  return GAL_OK;
}

// Known-answer ODE problems of the reference's unit test
// (source/tests/ODE_solver.F90:59-110, functions in tests/ODE_solver/functions.F90):
//   problem 1: y' = sin(x)                               (dim 1)
//   problem 2: y1' = y2, y2' = -y1, z1' = 1/sqrt(1+y1^2),
//              z2' = 1/sqrt(1+y2^2)                      (dim 4: y and the latent integrals)
// integrated from x0 to x1 with the same Cash-Karp driver and controller.
int oracle_ode_test(int problem, double x0, double x1, double* y, double tolAbs, double tolRel) {
  int dim = problem == 1 ? 1 : 4;
  struct F {
    int problem;
    void operator()(double x, const double* yy, double* d) const {
      if (problem == 1) {
        d[0] = std::sin(x);
      } else {
        d[0] = yy[1];
        d[1] = -yy[0];
        d[2] = 1.0 / std::sqrt(1.0 + yy[0] * yy[0]);
        d[3] = 1.0 / std::sqrt(1.0 + yy[1] * yy[1]);
      }
    }
  } f{problem};
  double s[4] = {1.0, 1.0, 1.0, 1.0};
  orc::Solver<double, F> sv{dim, f, tolAbs, tolRel, s, false};
  double t = x0, h = x1 - x0;
  bool exhausted = false;
  return sv.driver_apply(t, x1, h, y, [](double*) {}, 0, exhausted);
}

// Algorithmic FP64 operation counts of one node evolution, with the cooling
// radius in closed form (as the GPU kernel computes it).  ops[0..8] receive
// the counts of add/sub, mul, div, sqrt, log, exp, pow, atan, cbrt;
// counters[3] the accepted/rejected/RHS counts.
int oracle_count_flops(const gal_params* p, const gal_cie_table* table, const double* param, double* y, double t0,
                       double t1, double step, uint64_t* ops, uint32_t* counters) {
  orc::Table tb;
  int rc = orc::table_load(table, tb);
  if (rc) return rc;
  for (int i = 0; i < orc::OP_N; ++i) orc::g_ops[i] = 0;
  double h = step;
  int s = orc::evolve_node<orc::Counted>(*p, tb, param, y, t0, t1, h, counters, false);
  for (int i = 0; i < orc::OP_N; ++i) ops[i] = orc::g_ops[i];
  return s;
}


// Snapshot slots of a forest: for each node in index order, one slot per
// output time equal to its own time (a non-root only if it has an interval
// to evolve) and one per output time strictly inside its interval.
int64_t oracle_forest_snapshots(int64_t n, const int32_t* parent, const double* time, int32_t nOut, const double* tOut,
                                int64_t* snapFirst) {
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double t0 = time[i], t1 = parent[i] >= 0 ? time[parent[i]] : time[i];
    if (snapFirst) snapFirst[i] = total;
    for (int32_t k = 0; k < nOut; ++k) {
      if (tOut[k] == t0 && (parent[i] < 0 || t0 < t1)) ++total;
      else if (tOut[k] > t0 && tOut[k] < t1) ++total;
    }
  }
  return total;
}

// Evolve a forest on the host: every tree (from each root) in post-order,
// OpenMP-parallel over trees.  state[GAL_NY][n] receives each node's state
// on reaching its parent's time; snapshot[GAL_NY][m] the states at the
// output times (slots of oracle_forest_snapshots).
int oracle_evolve_forest(const gal_params* p, const gal_cie_table* table, int64_t n, const int32_t* parent,
                         const int32_t* childFirst, const int32_t* childCount, const double* time, const double* mass,
                         const double* spin, const int32_t* satHost, const double* state0, int32_t nOut,
                         const double* tOut, double* state, int32_t* status, uint32_t* counters, double* snapshot,
                         int threads, int cooling_brent) {
  if (!p || !table || n < 0 || !parent || !childFirst || !childCount || !time || !mass || !spin || !state0 || !state ||
      !status || (nOut > 0 && !tOut))
    return GAL_ERR_ARGUMENT;
  orc::Table tb;
  int rc = orc::table_load(table, tb);
  if (rc) return rc;
  if (threads <= 0) threads = omp_get_max_threads();
  const orc::Cosmology cos{p->omega_matter, p->omega_dark_energy, p->hubble_constant};
  orc::ForestIn F{n, parent, childFirst, childCount, time, mass, spin, state0, nOut, tOut, satHost, {}};
  F.massIn.assign((size_t)n, 0.0);
  if (satHost)
    for (int64_t i = 0; i < n; ++i)
      if (satHost[i] >= 0) F.massIn[(size_t)satHost[i]] += mass[i];
  std::vector<int64_t> snapFirst((size_t)n);
  const int64_t snapTotal = oracle_forest_snapshots(n, parent, time, nOut, tOut, snapFirst.data());
  std::vector<double> stepOf((size_t)n, -1.0);
  std::vector<int64_t> roots;
  for (int64_t i = 0; i < n; ++i)
    if (parent[i] < 0) roots.push_back(i);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int64_t r = 0; r < (int64_t)roots.size(); ++r) {
    // Post-order walk of this tree with an explicit stack.
    std::vector<std::pair<int64_t, int32_t>> stack{{roots[(size_t)r], 0}};
    while (!stack.empty()) {
      auto& top = stack.back();
      const int64_t i = top.first;
      if (top.second < childCount[i]) {
        const int64_t c = childFirst[i] + top.second;
        ++top.second;
        stack.push_back({c, 0});
        continue;
      }
      stack.pop_back();
      double y[GAL_NY];
      double h = -1.0;
      if (childCount[i] == 0) {
        for (int v = 0; v < GAL_NY; ++v) y[v] = state0[v * n + i];
      } else {
        const int64_t c0 = childFirst[i];
        for (int v = 0; v < GAL_NY; ++v) y[v] = state[v * n + c0];
        for (int32_t c = 1; c < childCount[i]; ++c) orc::merge_satellite(*p, y, &state[c0 + c], n);
        h = stepOf[(size_t)c0];
      }
      uint32_t cnt[3];
      status[i] = orc::evolve_forest_node(*p, tb, cos, F, i, y, h, cnt, cooling_brent != 0, snapFirst, snapshot,
                                          snapTotal);
      for (int v = 0; v < GAL_NY; ++v) state[v * n + i] = y[v];
      stepOf[(size_t)i] = h;
      if (counters)
        for (int v = 0; v < 3; ++v) counters[v * n + i] = cnt[v];
    }
  }
  return GAL_OK;
}


}  // extern "C"

// ------------------------------------------------------------ tree branching
//
// One tree of the Cole et al. (2000) builder with the Parkinson, Cole &
// Helly (2008) rates (merger_trees/construct/builder/Cole2000/
// _class.F90:360-913, merger_trees/branching_probability/
// Parkinson_Cole_Helly.F90:265-634), grown as the builder's GPU branching
// grows it, sequentially: from the root back in w = delta_c0/D(z), each
// step limited so that the split probability R dw, the sub-resolution mass
// fraction F dw (both times (w/sigma)^gamma2) and dw/sqrt(2 (S(M/2) - S(M)))
// stay below the accuracy parameters; a split draws q from the tabulated
// distribution in ln q and makes two progenitors (the larger first) at
// w + dw; a branch that falls below the resolution or reaches w_max ends in
// a leaf.  The tables (sigma(M), R, F, the ln q distribution; inputs of the
// walk, like the cooling table of the node evolution) come from the
// builder.
//
// This is the GPU walk's specification: the rates in FP32 from FP32 copies
// of the tables, its table-driven logarithm and exponential (Tang 1990,
// 1989; Cody & Waite 1980 argument reduction; short series evaluated with
// fmaf), the step limit with one division, the split test on a 24-bit draw
// and the kept mass fraction in FP32, the split's q from FP32 copies of its
// distribution, the mass and w accumulated in FP64,
// and each node's branch drawing
// from its own SplitMix64 stream (Steele, Lea & Flood 2014) keyed by its
// tree and its path from the root.  Every operation is IEEE-defined, so
// the GPU's trees must equal these bit for bit.

namespace orc {
namespace branch {

uint64_t mix64(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
constexpr uint64_t kGamma = 0x9e3779b97f4a7c15ull;
uint64_t root_key(uint64_t seed, int64_t tree) {
  return mix64(seed + kGamma) ^ mix64((uint64_t)tree * 0xd1b54a32d192ed03ull + 0x5851f42d4c957f2dull);
}
uint64_t child_key(uint64_t k, int c) { return mix64(k ^ (0xa0761d6478bd642full * (uint64_t)(c + 1))); }
double draw(uint64_t key, uint32_t k) { return (double)(mix64(key + (uint64_t)(k + 1) * kGamma) >> 11) * 0x1.0p-53; }

constexpr float kLn2Hi = 0.693359375f;          // 355/512
constexpr float kLn2Lo = -2.12194440e-4f;       // ln 2 - 355/512
constexpr float kLn2By32Hi = 0.0216674805f;     // 355/16384
constexpr float kLn2By32Lo = -6.63107626e-6f;   // (ln 2 - 355/512)/32
constexpr float k32ByLn2 = 46.1662445f;

// Function tables: ln c_j and 1/c_j at c_j = 1 + (j + 1/2)/128 (Tang 1990,
// ACM TOMS 16, 378), 2^(j/32) (Tang 1989, ACM TOMS 15, 144), as floats.
struct FnTables {
  float lnc[128], invc[128], pow2[32];
  FnTables() {
    for (int j = 0; j < 128; ++j) {
      const double c = 1.0 + (j + 0.5) / 128.0;
      lnc[j] = (float)std::log(c);
      invc[j] = (float)(1.0 / c);
    }
    for (int j = 0; j < 32; ++j) pow2[j] = (float)std::exp2(j / 32.0);
  }
};
const FnTables& fn_tables() {
  static const FnTables t;
  return t;
}

// ln x for a positive normal double: x = 2^e f, f in [1, 2) from its top 23
// mantissa bits (truncated), r = f/c_j - 1 with c_j the centre of f's 1/128
// interval, ln x = e ln 2 + ln c_j + r - r^2/2 + r^3/3.
float ln_pos(double x) {
  const FnTables& t = fn_tables();
  int64_t b;
  std::memcpy(&b, &x, sizeof b);
  const int e = (int)(b >> 52) - 1023;
  const int j = (int)((b >> 45) & 127);
  const uint32_t fb = 0x3f800000u | (uint32_t)((b >> 29) & 0x7fffff);
  float f;
  std::memcpy(&f, &fb, sizeof f);
  const float r = std::fmaf(f, t.invc[j], -1.0f);
  const float p = std::fmaf(std::fmaf(r, 1.0f / 3.0f, -0.5f), r * r, r);
  const float ef = (float)e;
  return std::fmaf(ef, kLn2Hi, std::fmaf(ef, kLn2Lo, t.lnc[j] + p));
}

// e^x for |x| < 80: x = (32 k + j) ln 2/32 + r, e^x = 2^k 2^(j/32) e^r with
// e^r = 1 + r + r^2/2 + r^3/6.
float exp_f(float x) {
  const FnTables& t = fn_tables();
  x = std::fmin(std::fmax(x, -80.0f), 80.0f);
  const float n = std::rint(x * k32ByLn2);
  const int ni = (int)n;
  const int j = ni & 31;
  const int k = ni >> 5;
  const float r = std::fmaf(-n, kLn2By32Lo, std::fmaf(-n, kLn2By32Hi, x));
  const float p = std::fmaf(std::fmaf(std::fmaf(r, 1.0f / 6.0f, 0.5f), r, 1.0f), r, 1.0f);
  const uint32_t sb = (uint32_t)(k + 127) << 23;
  float scale;
  std::memcpy(&scale, &sb, sizeof scale);
  return (t.pow2[j] * p) * scale;
}

float draw24(uint64_t key, uint32_t k) {
  return (float)(uint32_t)(mix64(key + (uint64_t)(k + 1) * kGamma) >> 40) * 0x1.0p-24f;
}

struct Tables {
  std::vector<float> lnSigma, R, F;  // FP32 copies
  std::vector<float> lnqA, lnqD;     // per row: ln q of the first point, spacing in ln q
  std::vector<float> cdf;            // [rows][kNq], FP32
  float sigLnMin, sigInv, halfShift, rtLnMin, rtInv, gamma2, acc1, acc2;
  double mRes, wMax;
  static constexpr int kNq = 96;
};

float interp(const std::vector<float>& t, float x) {
  const int n = (int)t.size();
  x = std::fmin(std::fmax(x, 0.0f), (float)(n - 1));
  const int i = std::min((int)x, n - 2);
  const float f = x - (float)i;
  return t[(size_t)i] + f * (t[(size_t)i + 1] - t[(size_t)i]);
}

struct Node {
  double mass, w;
  int32_t parent, childFirst, childCount;
  uint64_t key;
};

void grow(const Tables& t, double rootMass, double rootW, uint64_t rootKey, std::vector<Node>& nodes) {
  constexpr int nq = Tables::kNq;
  const int rows = (int)t.R.size();
  nodes.assign(1, Node{rootMass, rootW, -1, 0, 0, rootKey});
  std::vector<int32_t> stack{0};
  while (!stack.empty()) {
    const int32_t i = stack.back();
    stack.pop_back();
    const uint64_t key = nodes[(size_t)i].key;
    double m = nodes[(size_t)i].mass, w = nodes[(size_t)i].w;
    double mPrev = m, wPrev = w;
    uint32_t k = 0;
    bool split = false;
    int guard = 0;
    while (w < t.wMax && m >= t.mRes && ++guard < 100000) {
      const float lm = ln_pos(m);
      const float x = (lm - t.rtLnMin) * t.rtInv;
      const float xs = (lm - t.sigLnMin) * t.sigInv;
      const float lns2 = interp(t.lnSigma, xs);
      const float S2 = exp_f(2.0f * lns2);
      const float Sh = exp_f(2.0f * interp(t.lnSigma, xs - t.halfShift));
      const float wf = exp_f(t.gamma2 * (ln_pos(w) - lns2));
      const float xc = std::fmin(std::fmax(x, 0.0f), (float)(rows - 1));
      const int j = std::min((int)xc, rows - 2);
      const float fx = xc - (float)j;
      const float R = m <= 2.0 * t.mRes ? 0.0f : wf * (t.R[(size_t)j] + fx * (t.R[(size_t)j + 1] - t.R[(size_t)j]));
      const float F = wf * (t.F[(size_t)j] + fx * (t.F[(size_t)j + 1] - t.F[(size_t)j]));
      float dwf = t.acc2 * std::sqrt(2.0f * std::fmax(Sh - S2, 0.0f));
      const float RF = std::fmax(R, F);
      if (RF > 0.0f) dwf = std::fmin(dwf, t.acc1 / RF);
      if (!(dwf > 0.0f)) dwf = 1.0e-3f;
      double dw = (double)dwf;
      const double wStep = w + dw;
      const bool last = wStep >= t.wMax;
      if (last) {
        dw = t.wMax - w;
        dwf = (float)dw;
      }
      const double wNext = last ? t.wMax : wStep;
      const double keep = (double)(1.0f - F * dwf);
      mPrev = m;
      wPrev = w;
      if (R > 0.0f && draw24(key, k++) < R * dwf) {
        int row = fx < 0.5f ? j : j + 1;
        if (!(t.R[(size_t)row] > 0.0f)) row = j + 1;
        const float* cdf = t.cdf.data() + (size_t)row * nq;
        const float target = draw24(key, k++);
        const int kk = (int)(std::upper_bound(cdf, cdf + nq, target) - cdf);
        const int k1 = std::min(std::max(kk, 1), nq - 1);
        const float c0 = cdf[k1 - 1];
        const float f = (target - c0) / std::fmax(cdf[k1] - c0, 1e-30f);
        const double q = (double)exp_f(std::fmaf((float)(k1 - 1) + f, t.lnqD[(size_t)row], t.lnqA[(size_t)row]));
        const double m1 = q * m;
        const double m2 = m * keep - m1;
        const double big = std::max(m1, m2), small = std::min(m1, m2);
        const int32_t first = (int32_t)nodes.size();
        int32_t count = 0;
        if (big >= t.mRes) nodes.push_back(Node{big, wNext, i, 0, 0, child_key(key, count++)});
        if (small >= t.mRes) nodes.push_back(Node{small, wNext, i, 0, 0, child_key(key, count++)});
        nodes[(size_t)i].childFirst = first;
        nodes[(size_t)i].childCount = count;
        for (int32_t c = count - 1; c >= 0; --c) stack.push_back(first + c);
        split = true;
        break;
      }
      m *= keep;
      w = wNext;
      if (last) break;
    }
    if (!split) {
      double lm = m, lw = w;
      if (m < t.mRes) {
        lm = mPrev;
        lw = wPrev;
      }
      if (lw > nodes[(size_t)i].w && lm >= t.mRes) {
        nodes[(size_t)i].childFirst = (int32_t)nodes.size();
        nodes[(size_t)i].childCount = 1;
        nodes.push_back(Node{lm, lw, i, 0, 0, child_key(key, 0)});
      }
    }
  }
}

}  // namespace branch
}  // namespace orc

extern "C" {

// The walk's FP32 logarithm (of doubles) and exponential, for n arguments.
void oracle_branch_math(int64_t n, const double* x, float* ln_x, const float* y, float* exp_y) {
  for (int64_t i = 0; i < n; ++i) {
    ln_x[i] = orc::branch::ln_pos(x[i]);
    exp_y[i] = orc::branch::exp_f(y[i]);
  }
}

// Grow trees tree0..tree0+n-1 of seed from their root masses (at w =
// meta[9]); meta[10], sizes[2] and the arrays as gal_pch_branch_tables
// returns them.  Node arrays of capacity cap receive the trees one after
// another, each in the builder's order (depth first, the larger progenitor
// first); treeFirst[n] the first node of each.  Returns the node count, or
// -(the count needed) when cap is too small.
int64_t oracle_grow_trees(const double* meta, const int32_t* sizes, const double* lnSigma, const double* rate,
                          const double* accretion, const double* lnq, const double* cdf, uint64_t seed, int64_t tree0,
                          int64_t n, const double* rootMass, int64_t cap, double* mass, double* w, int32_t* parent,
                          int32_t* childFirst, int32_t* childCount, int64_t* treeFirst) {
  orc::branch::Tables t;
  t.lnSigma.assign(lnSigma, lnSigma + sizes[0]);
  t.R.assign(rate, rate + sizes[1]);
  t.F.assign(accretion, accretion + sizes[1]);
  if (sizes[0] < 2 || sizes[1] < 2) return 0;
  t.lnqA.resize((size_t)sizes[1]);
  t.lnqD.resize((size_t)sizes[1]);
  t.cdf.assign(cdf, cdf + (size_t)sizes[1] * orc::branch::Tables::kNq);
  for (int32_t r = 0; r < sizes[1]; ++r) {
    const double* q = lnq + (size_t)r * orc::branch::Tables::kNq;
    t.lnqA[(size_t)r] = (float)q[0];
    t.lnqD[(size_t)r] = (float)((q[orc::branch::Tables::kNq - 1] - q[0]) / (orc::branch::Tables::kNq - 1));
  }
  t.sigLnMin = (float)meta[0];
  t.sigInv = (float)(1.0 / meta[1]);
  t.halfShift = (float)(0.6931471805599453 / meta[1]);
  t.rtLnMin = (float)meta[2];
  t.rtInv = (float)(1.0 / meta[3]);
  t.mRes = meta[4];
  t.wMax = meta[5];
  t.gamma2 = (float)meta[6];
  t.acc1 = (float)meta[7];
  t.acc2 = (float)meta[8];
  std::vector<std::vector<orc::branch::Node>> trees((size_t)n);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t j = 0; j < n; ++j)
    orc::branch::grow(t, rootMass[j], meta[9], orc::branch::root_key(seed, tree0 + j), trees[(size_t)j]);
  int64_t total = 0;
  for (const auto& tr : trees) total += (int64_t)tr.size();
  if (total > cap) return -total;
  int64_t off = 0;
  for (int64_t j = 0; j < n; ++j) {
    treeFirst[j] = off;
    for (const auto& nd : trees[(size_t)j]) {
      mass[off] = nd.mass;
      w[off] = nd.w;
      parent[off] = nd.parent;
      childFirst[off] = nd.childFirst;
      childCount[off] = nd.childCount;
      ++off;
    }
  }
  return total;
}

}  // extern "C"
