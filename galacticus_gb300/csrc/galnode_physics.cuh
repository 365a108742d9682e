// galnode_physics.cuh -- device physics of the P-std node ODE system.
//
// One thread evaluates the full right-hand side of one node.  Quantities
// that do not change during an evolve call (halo scales, galaxy sizes,
// star-formation timescales, outflow loading factors, the temperature
// coordinate of the CIE tables) are computed once per node in
// node_setup(); the right-hand side only does the state-dependent work.
// Reference sources are cited per function (paths relative to the
// Galacticus repository root).
#pragma once

#include <cmath>
#include <cstdint>
#include "../../include/galnode.h"
#include "galnode_fastmath.cuh"
#include "galnode_krumholz.cuh"

namespace gal {

// ---- physical constants (source/numerical/constants/*.F90; GSL MKSA values)
namespace k {
constexpr double Pi = 3.14159265358979323846;
constexpr double gravitationalConstant = 6.673e-11;
constexpr double massSolar = 1.98892e30;
constexpr double megaParsec = 1.0e6 * 3.08567758135e16;
constexpr double gigaYear = 1.0e9 * 3.15581497635456e7;
constexpr double boltzmannsConstant = 1.3806504e-23;
constexpr double atomicMassUnit = 1.660538782e-27;
constexpr double speedLight = 2.99792458e8;
constexpr double thomsonCrossSection = 6.65245893699e-29;
constexpr double atomicMassHydrogen = 1.0078250322;
constexpr double atomicMassHelium = 4.0026032545;
constexpr double massHydrogenAtom = atomicMassHydrogen * atomicMassUnit;
constexpr double hydrogenByMassPrimordial = 0.7514;
constexpr double heliumByMassPrimordial = 0.2486;
constexpr double hydrogenByMassSolar = 0.7070;
constexpr double heliumByMassSolar = 0.2740;
constexpr double metallicitySolar = 0.0188;
constexpr double meanAtomicMassPrimordial =
    1.0 / (2.0 * hydrogenByMassPrimordial / atomicMassHydrogen + 3.0 * heliumByMassPrimordial / atomicMassHelium);
constexpr double kilo = 1.0e3, hecto = 1.0e2, ergs = 1.0e-7;
constexpr double gravitationalConstantInternal = gravitationalConstant * massSolar / (kilo * kilo) / megaParsec;
constexpr double MpcPerKmPerSToGyr = megaParsec / kilo / gigaYear;
constexpr double feedbackEnergyInputAtInfinityCanonical = 4.517e5;
// n_H per (rho X_H) with rho in Msun/Mpc^3 and n_H in cm^-3 (cooling_time/simple.F90:150-155).
constexpr double densityToHydrogenNumber =
    massSolar / massHydrogenAtom / (hecto * hecto * hecto) / (megaParsec * megaParsec * megaParsec);
// Eddington rate per unit black-hole mass (black_holes/fundamentals.F90:123-138).
constexpr double eddingtonPerMass = 4.0 * Pi * gravitationalConstant * massHydrogenAtom * gigaYear / thomsonCrossSection / speedLight;
// Bondi-Hoyle-Lyttleton prefactor (accretion/Bondi_Hoyle_Lyttleton.F90:34-59).
constexpr double bhlPrefactor = kilo * gigaYear / megaParsec * 4.0 * Pi;
}  // namespace k

// Constants shared by every node, derived on the host from gal_params.
struct Globals {
  gal_params p;
  int nT, nZ;                 // table shape
  int firstZero;              // first metallicity row is Z = 0
  double firstNonZero;        // Z/Zsun of the first non-zero row
  double invFirstNonZero;
  int zUniform;               // non-zero rows evenly spaced in ln Z: cell by arithmetic
  int zFirstLog;              // index of the first non-zero row
  double lnZFirst, invDlnZ;   // its ln Z and the reciprocal spacing
  double Tmin, Tmax, Zmin, Zmax;
  double soundSpeedSpheroid;  // km/s at bh_temperature_spheroid
  double jeansPrefactor;      // c_s/sqrt(G) for the spheroid gas
  double bhSpheroidCoef;      // enhancement * bhl * G^2 / c_s^3
  double bhRadiusSpheroidCoef;  // G / c_s^2
  double coolingCoef;         // (dof/2) k_B / ergs / Gyr / densityToHydrogenNumber
  double accretionFraction;   // Omega_b / Omega_m
  double kmtSTruncation;      // Krumholz (2009) disks: s where the molecular fraction falls to 1e-10
  // FP32 copies for the FP32-rate forms, derived once on the host
  // (fill_fast_constants) so that no rate evaluation converts or divides in FP64.
  struct Fast {
    float oneMinusR, metalYield;
    float eddingtonOverEps;   // eddingtonPerMass / epsilon_radiative (0: no Eddington cap)
    float bhRetained;         // 1 - epsilon_radiative - epsilon_jet
    float bhRadiusSpheroidCoef, jeansPrefactor, bhSpheroidCoef;
    float Zmin, Zmax, firstNonZero, invFirstNonZero, lnZFirst, invDlnZ;
    int capped;               // epsilon_radiative > 0
    // Coefficients of node_setup_fast(): every per-node constant is one of
    // these times powers of r_vir, V_vir and the spin.
    float tempPerV2;          // T_vir / V_vir^2 (K s^2 km^-2)
    float tdynCoef;           // MpcPerKmPerSToGyr
    float coreFraction;       // r_core / r_vir
    float rho0Norm;           // 1/(4 pi (x - atan x)), x = r_vir/r_core
    float twoPiRho0Norm;      // 2 pi rho0Norm
    float onePlusXOuter2;     // 1 + x^2
    float Tmin, Tmax;         // table temperature range ("extrapolate" = clamp)
    float lnTFirst, invDlnT;  // ln T of the first row, reciprocal spacing (tUniform)
    float coolingCoef;        // Globals::coolingCoef
    float radiusFactorDisk, radiusFactorSpheroid;
    float csSquaredPerT;      // c_s^2 / T of the primordial gas (km^2 s^-2 K^-1)
    float gravitationalConstant;  // G in Mpc (km/s)^2 / Msun
    float bhHotPrefactor;     // enhancement (hot halo) * Bondi-Hoyle-Lyttleton prefactor
    float accretionFraction;  // Omega_b / Omega_m
    float reincorporationMultiplier;
    float invTwoPi;
    struct Sf { float fixed, efficiency, exponent, minimum; } sfDisk, sfSph;
    struct Out { float fraction, velocity, exponent, fractionalMinimum; } outDisk, outSph;
    float kmtFrequency, kmtClumping, kmtSTruncation;  // Krumholz (2009) disks
  } f;
  int tUniform;               // temperature rows evenly spaced in ln T: cell by arithmetic
};

// Fill Globals::f from the FP64 constants (host).
inline void fill_fast_constants(Globals& g) {
  g.f.oneMinusR = (float)(1.0 - g.p.recycled_fraction);
  g.f.metalYield = (float)g.p.metal_yield;
  g.f.capped = g.p.bh_efficiency_radiative > 0.0;
  g.f.eddingtonOverEps = g.f.capped ? (float)(k::eddingtonPerMass / g.p.bh_efficiency_radiative) : 0.0f;
  g.f.bhRetained = (float)(1.0 - g.p.bh_efficiency_radiative - g.p.bh_efficiency_jet);
  g.f.bhRadiusSpheroidCoef = (float)g.bhRadiusSpheroidCoef;
  g.f.jeansPrefactor = (float)g.jeansPrefactor;
  g.f.bhSpheroidCoef = (float)g.bhSpheroidCoef;
  g.f.Zmin = (float)g.Zmin;
  g.f.Zmax = (float)g.Zmax;
  g.f.firstNonZero = (float)g.firstNonZero;
  g.f.invFirstNonZero = (float)g.invFirstNonZero;
  g.f.lnZFirst = (float)g.lnZFirst;
  g.f.invDlnZ = (float)g.invDlnZ;
  // node_setup() with r_vir, V_vir and the spin factored out.
  g.f.tempPerV2 = (float)(0.5 * k::atomicMassUnit * k::meanAtomicMassPrimordial * k::kilo * k::kilo / k::boltzmannsConstant);
  g.f.tdynCoef = (float)k::MpcPerKmPerSToGyr;
  g.f.coreFraction = (float)g.p.core_radius_fraction;
  const double x = 1.0 / g.p.core_radius_fraction;
  const double norm = x < 1.0e-6 ? 3.0 / (x * x * x) + 9.0 / 5.0 / x - 36.0 * x / 175.0 : 1.0 / (x - std::atan(x));
  g.f.rho0Norm = (float)(norm / (4.0 * k::Pi));
  g.f.twoPiRho0Norm = (float)(2.0 * k::Pi * norm / (4.0 * k::Pi));
  g.f.onePlusXOuter2 = (float)(1.0 + x * x);
  g.f.Tmin = (float)g.Tmin;
  g.f.Tmax = (float)g.Tmax;
  g.f.coolingCoef = (float)g.coolingCoef;
  g.f.radiusFactorDisk = (float)g.p.radius_factor_disk;
  g.f.radiusFactorSpheroid = (float)g.p.radius_factor_spheroid;
  g.f.csSquaredPerT = (float)(5.0 * k::boltzmannsConstant / 3.0 / k::meanAtomicMassPrimordial / k::atomicMassUnit / (k::kilo * k::kilo));
  g.f.gravitationalConstant = (float)k::gravitationalConstantInternal;
  g.f.bhHotPrefactor = (float)(g.p.bh_enhancement_hot_halo * k::bhlPrefactor);
  g.f.accretionFraction = (float)g.accretionFraction;
  g.f.reincorporationMultiplier = (float)g.p.reincorporation_multiplier;
  g.f.invTwoPi = (float)(1.0 / (2.0 * k::Pi));
  auto sf = [](const gal_star_formation& s) {
    return Globals::Fast::Sf{(float)s.timescale_fixed, (float)s.efficiency, (float)s.exponent_velocity, (float)s.timescale_minimum};
  };
  auto out = [](const gal_outflow& o) {
    return Globals::Fast::Out{(float)o.fraction, (float)o.velocity_characteristic, (float)o.exponent,
                              (float)o.timescale_fractional_minimum};
  };
  g.kmtSTruncation = kmt_s_truncation(g.p.krumholz_fast != 0);
  g.f.kmtFrequency = (float)g.p.krumholz_frequency;
  g.f.kmtClumping = (float)g.p.krumholz_clumping;
  g.f.kmtSTruncation = (float)g.kmtSTruncation;
  g.f.sfDisk = sf(g.p.sf_disk);
  g.f.sfSph = sf(g.p.sf_spheroid);
  g.f.outDisk = out(g.p.outflow_disk);
  g.f.outSph = out(g.p.outflow_spheroid);
}

// Per-node constants of one evolve call.  Reciprocals of the per-node
// lengths and times are taken here once, so that the right-hand side
// multiplies instead of dividing (an FP64 divide is ~10 slow-pipe
// instructions on GB300).
struct NodeC {
  double massHalo;            // basic mass at the start (tolerance scale)
  double tdyn;                // halo dynamical time r_vir/V_vir (Gyr)
  double invTdyn;
  double rcore;               // beta-profile core radius (Mpc)
  double invRcore;
  double rho0PerMass;         // central beta-profile density per unit hot mass
  double rOuter;              // hot-halo outer radius = virial radius (Mpc)
  double invRvir;
  double onePlusXOuter2;      // 1 + (r_outer/r_core)^2
  double coolingTimeCoef;     // coolingCoef * T_vir
  double coolingRateCoef;     // 2 pi rho0PerMass r_core^2 / t_dyn
  double hT;                  // temperature interpolation weight
  int iT;                     // temperature cell of T_vir
  int coolingAllowed;         // V_vir <= velocity cut-off
  float log10T;               // log10 T_vir (input of the cooling surrogate)
  int netRow;                 // with the surrogate: first error-map cell of the node's T row, or -1
                              // when no cell of that row is served by the network
  double sfrDisk, sfrSph;     // 1/tau_* of the disk and spheroid (0: none)
  double outDisk, outSph;     // outflow rate per unit SFR
  double outDiskMax, outSphMax; // 1/(t_dyn f_min) of the rate limit (<0: no limit)
  double aSph;                // spheroid scale radius (Mpc)
  double invASph;
  double rhoSphPerMass;       // 1/(2 pi a^3)
  double radiusDisk;          // disk radius (Mpc)
  double bhRadiusHotCoef;     // G / c_s(T_vir)^2
  double bhHotCoef;           // enhancement * bhl * c_s(T_vir)
  double bhHotMaxCoef;        // c_s/(r_outer MpcPerKmPerSToGyr)
  double accretionRate;       // hot-gas accretion rate (Msun/Gyr)
  double reincorporationRate; // multiplier / t_dyn
};

// Shared-memory tables used by the right-hand side.
struct Smem {
  const double2* tab;      // (ln Lambda, ln n_e/n_H) [nZ][nT]
  const double* lnZ;       // ln Z/Zsun of the rows
  const double* invDlnZ;   // 1/(ln Z[i+1] - ln Z[i])
  FastTables fast;         // tables of the short FP64 log/exp
  KmtTables<double> kmt;   // Krumholz (2009) tables (global memory)
};

// Abundances_Mass_To_Mass_Fraction_Packed (objects/abundances.F90:781-809)
// given the reciprocal of the mass.
__device__ __forceinline__ double mass_fraction(double metals, double mass, double invMass) {
  return metals > mass ? 1.0 : (metals <= 0.0 ? 0.0 : metals * invMass);
}

// Largest i with g[i] <= x, kept in [0, n-2]; g in shared memory.
__device__ __forceinline__ int locate(const double* g, int n, double x) {
  if (!(x >= g[0])) return 0;
  if (x >= g[n - 1]) return n - 2;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (g[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// Set up the per-node constants (node_setup in the oracle; each line
// restates the cited reference function for a node whose scales are fixed
// over the call).
__device__ __forceinline__ void node_setup(const Globals& G, const double* sLnT, const double* prm, NodeC& c) {
  const gal_params& p = G.p;
  const double M = prm[GAL_P_MASS], Mdot = prm[GAL_P_MASS_RATE];
  const double rvir = prm[GAL_P_RADIUS_VIRIAL], vvir = prm[GAL_P_VELOCITY_VIRIAL], spin = prm[GAL_P_SPIN];
  c.massHalo = M;
  // virialDensityContrastDefinition{VirialTemperature,DynamicalTimescale} (virial_density_contrast.F90:195-262)
  const double T = 0.5 * k::atomicMassUnit * k::meanAtomicMassPrimordial * (k::kilo * vvir) * (k::kilo * vvir) / k::boltzmannsConstant;
  c.tdyn = rvir / vvir * k::MpcPerKmPerSToGyr;
  c.invTdyn = 1.0 / c.tdyn;
  c.rcore = p.core_radius_fraction * rvir;
  c.invRcore = 1.0 / c.rcore;
  c.rOuter = rvir;  // outer radius clamp of hot_halo/standard/_class.F90:430-450
  c.invRvir = 1.0 / rvir;
  const double x = c.rOuter / c.rcore;
  const double norm = x < 1.0e-6 ? 3.0 / (x * x * x) + 9.0 / 5.0 / x - 36.0 * x / 175.0 : 1.0 / (x - atan(x));
  c.rho0PerMass = norm / (4.0 * k::Pi) / (c.rcore * c.rcore * c.rcore);
  c.onePlusXOuter2 = 1.0 + x * x;
  c.coolingRateCoef = 2.0 * k::Pi * c.rho0PerMass * c.rcore * c.rcore * c.invTdyn;
  // Temperature coordinate of the CIE tables ("extrapolate" in T = clamp).
  const double Tc = fmin(fmax(T, G.Tmin), G.Tmax);
  const double lnT = log(Tc);
  c.iT = locate(sLnT, G.nT, lnT);
  c.hT = (lnT - sLnT[c.iT]) / (sLnT[c.iT + 1] - sLnT[c.iT]);
  c.coolingTimeCoef = G.coolingCoef * T;
  c.log10T = T > 0.0 ? (float)log10(T) : -1.0e30f;
  c.coolingAllowed = !(vvir > p.cooling_velocity_cutoff);
  // galacticStructureSolverFixed: r = f lambda r_vir, V = V_vir.
  const double Rd = p.radius_factor_disk * spin * rvir, Rs = p.radius_factor_spheroid * spin * rvir;
  c.radiusDisk = Rd;
  c.aSph = Rs;
  c.invASph = Rs > 0.0 ? 1.0 / Rs : 0.0;
  c.rhoSphPerMass = Rs > 0.0 ? 1.0 / (2.0 * k::Pi) / (Rs * Rs * Rs) : 0.0;
  // Star-formation timescales (star_formation/timescales/dynamical_time.F90:121-189).
  auto timescale = [&](const gal_star_formation& sf, double R) -> double {
    if (sf.timescale_type == GAL_SF_TIMESCALE_FIXED) return sf.timescale_fixed;
    if (vvir <= 0.0 || sf.efficiency == 0.0) return 0.0;
    const double t = k::MpcPerKmPerSToGyr * R / vvir;
    return fmax(t * pow(vvir / 200.0, sf.exponent_velocity) / sf.efficiency, sf.timescale_minimum);
  };
  const double tsD = timescale(p.sf_disk, Rd), tsS = timescale(p.sf_spheroid, Rs);
  c.sfrDisk = tsD > 0.0 ? 1.0 / tsD : 0.0;
  c.sfrSph = tsS > 0.0 ? 1.0 / tsS : 0.0;
  // Outflow loading (power_law/_class.F90:118-164, fixed.F90) and rateLimit (rate_limit.F90).
  auto loading = [&](const gal_outflow& o) -> double {
    if (o.type == GAL_OUTFLOW_FIXED) return o.fraction;
    if (vvir <= 0.0) return 0.0;
    return pow(o.velocity_characteristic / vvir, o.exponent);
  };
  auto limit = [&](const gal_outflow& o, double R) -> double {
    if (!(o.timescale_fractional_minimum > 0.0)) return -1.0;
    const double t = (vvir <= 0.0 || R <= 0.0) ? 1.0 : k::MpcPerKmPerSToGyr * R / vvir;
    return 1.0 / t / o.timescale_fractional_minimum;
  };
  c.outDisk = loading(p.outflow_disk);
  c.outSph = loading(p.outflow_spheroid);
  c.outDiskMax = limit(p.outflow_disk, Rd);
  c.outSphMax = limit(p.outflow_spheroid, Rs);
  // Hot-halo Bondi accretion constants at the virial temperature.
  const double cs = sqrt(5.0 * k::boltzmannsConstant * T / 3.0 / k::meanAtomicMassPrimordial / k::atomicMassUnit) / k::kilo;
  c.bhRadiusHotCoef = T > 0.0 ? k::gravitationalConstantInternal / (cs * cs) : 0.0;
  c.bhHotCoef = p.bh_enhancement_hot_halo * k::bhlPrefactor * cs;
  c.bhHotMaxCoef = cs / (c.rOuter * k::MpcPerKmPerSToGyr);
  c.accretionRate = Mdot > 0.0 ? G.accretionFraction * Mdot : 0.0;
  c.reincorporationRate = p.reincorporation_multiplier * c.invTdyn;
}

// Interpolated cooling function (erg cm^3 s^-1, without the n_H^2 factor)
// and n_e/n_H at the node temperature and metallicity Z/Zsun
// (cooling_function/CIE_file.F90:238-317, 665-735; chemical/state/
// CIE_file.F90:245-320).  `tab` interleaves (ln Lambda, ln n_e/n_H);
// sInvDlnZ[i] = 1/(ln Z[i+1] - ln Z[i]).
__device__ __forceinline__ void cie_lookup(const Globals& G, const Smem& S, const NodeC& c, double zSolar, double& lambda,
                                          double& electrons) {
  const double* sLnZ = S.lnZ;
  zSolar = dmin(dmax(zSolar, G.Zmin), G.Zmax);  // "fix" extrapolation in metallicity
  const double zUse = dmax(zSolar, 0.0);
  int iZ;
  double hZ;
  if (G.firstZero && zUse < G.firstNonZero) {
    iZ = 0;
    hZ = zUse * G.invFirstNonZero;
  } else {
    const double lnZ = fast_log(S.fast, zUse);
    if (G.zUniform) {
      // Evenly spaced rows: estimate the cell, then settle it against the
      // grid values so that it is exactly locate()'s answer.
      const int last = G.nZ - 2;
      int j = G.zFirstLog + (int)floor((lnZ - G.lnZFirst) * G.invDlnZ);
      j = j < G.zFirstLog ? G.zFirstLog : (j > last ? last : j);
      if (j > G.zFirstLog && lnZ < sLnZ[j]) --j;
      if (j < last && lnZ >= sLnZ[j + 1]) ++j;
      if (lnZ < sLnZ[j]) j = 0 > j - 1 ? 0 : j - 1;  // below the first non-zero row
      iZ = j;
    } else {
      iZ = locate(sLnZ, G.nZ, lnZ);
    }
    hZ = (lnZ - sLnZ[iZ]) * S.invDlnZ[iZ];
  }
  const double2* tab = S.tab;
  const int nT = G.nT;
  const double2 a = tab[iZ * nT + c.iT], b = tab[(iZ + 1) * nT + c.iT];
  const double2 d = tab[iZ * nT + c.iT + 1], e = tab[(iZ + 1) * nT + c.iT + 1];
  const double hT = c.hT;
  const double w00 = (1.0 - hT) * (1.0 - hZ), w01 = (1.0 - hT) * hZ, w10 = hT * (1.0 - hZ), w11 = hT * hZ;
  lambda = fast_exp(S.fast, a.x * w00 + b.x * w01 + d.x * w10 + e.x * w11);
  electrons = fast_exp(S.fast, a.y * w00 + b.y * w01 + d.y * w10 + e.y * w11);
}

// Cooling radius (cooling_radius/simple.F90:313-427) in closed form.  At
// fixed temperature and metallicity the cooling time is proportional to
// 1/rho (Lambda scales as n_H^2, n_e as n_H), so t_cool(r) = t_avail solves
// as r = r_core sqrt(t_avail/t_cool(0) - 1) inside the bracket [0, r_outer]
// that the reference's root finder searches; t_avail = t_dyn
// (coolingTimeAvailableWhiteFrenk1991 with ageFactor = 0).  The cooling time
// of coolingTimeSimple (cooling_time/simple.F90:128-179) is
//   t_cool(0) = (dof/2) k T (n_H/x_num + n_e) / ergs / (Lambda n_H^2) / Gyr
// with n_H = rho(0) X_H and 1/x_num = 1 + (Y m_H)/(X_H m_He); the ratio
// q = t_avail/t_cool(0) below is that expression with one division.
// Cooling function and electron fraction supplied by the surrogate for this
// evaluation (use = false: interpolate the table).
struct CoolingValues {
  bool use;
  double lambda, electrons;
};

__device__ __forceinline__ double cooling_radius(const Globals& G, const Smem& S, const NodeC& c, double massHot, double zHot,
                                                const CoolingValues& cv) {
  // Abundances_Hydrogen/Helium_Mass_Fraction (objects/abundances.F90:830-868).
  const double zs = zHot * (1.0 / k::metallicitySolar);
  const double xH = dmin(dmax(zs * (k::hydrogenByMassSolar - k::hydrogenByMassPrimordial) + k::hydrogenByMassPrimordial, 0.7),
                         k::hydrogenByMassPrimordial);
  const double yHe = dmin(zs * (k::heliumByMassSolar - k::heliumByMassPrimordial) + k::heliumByMassPrimordial, k::heliumByMassPrimordial);
  double lambda, electrons;
  if (cv.use) {
    lambda = cv.lambda;
    electrons = cv.electrons;
  } else {
    cie_lookup(G, S, c, zs, lambda, electrons);
  }
  const double num = c.tdyn * lambda * massHot * c.rho0PerMass * xH * xH;
  const double den = c.coolingTimeCoef * (xH * (1.0 + electrons) + yHe * (k::atomicMassHydrogen / k::atomicMassHelium));
  const double q = massHot > 0.0 ? fast_div(num, den) : 0.0;
  if (q > c.onePlusXOuter2) return c.rOuter;  // t_cool(r_outer) < t_avail
  if (q < 1.0) return 0.0;                    // t_cool(0) > t_avail
  return c.rcore * fast_sqrt(q - 1.0);
}

// Right-hand side of the node ODE system: the node operators of
// nodeOperatorMulti (nodes/operators/multi.F90:313-332) in the order of
// parameters/quickTest.xml.  Same logic, branch by branch, as the oracle.
// KMT: the disk star-formation rate is krumholz2009 (gal_params.sf_disk_rate;
// a separate kernel instantiation, so that the timescale form carries no
// call to the integrator).
template <bool KMT = false>
__device__ __forceinline__ void rhs(const Globals& G, const Smem& S, const NodeC& c, const double* y, double* dydt,
                                   const CoolingValues& cv = CoolingValues{false, 0.0, 0.0}) {
  const gal_params& p = G.p;
  const uint32_t ph = p.physics;
#pragma unroll
  for (int i = 0; i < GAL_NY; ++i) dydt[i] = 0.0;
  const double massHot = y[GAL_Y_HOT_MASS], metalsHot = y[GAL_Y_HOT_METALS];
  const double gasDisk = y[GAL_Y_DISK_GAS], gasSph = y[GAL_Y_SPHEROID_GAS];
  const double invHot = massHot > 0.0 ? fast_rcp(massHot) : 0.0;
  const double zHot = mass_fraction(metalsHot, massHot, invHot);
  bool coolingRadiusKnown = false;
  double rCool = 0.0;

  // starFormationDisks (star_formation/disks.F90:200-324) + instantaneous populations
  // (stellar_populations/properties/instantaneous.F90:133-219).
  const bool diskOk = !(c.radiusDisk < 0.0 || gasDisk < 0.0);
  double sfrDisk = 0.0;
  if (diskOk) {
    if constexpr (KMT)
      // starFormationRateDisksIntgrtdSurfaceDensity with krumholz2009.
      sfrDisk = krumholz2009_rate<double>(S.kmt, p.krumholz_frequency, p.krumholz_clumping, G.kmtSTruncation,
                                          p.krumholz_fast != 0, gasDisk, y[GAL_Y_DISK_GAS_METALS], c.radiusDisk);
    else
      sfrDisk = gasDisk * c.sfrDisk;
  }
  const double zDisk = mass_fraction(y[GAL_Y_DISK_GAS_METALS], gasDisk, gasDisk > 0.0 ? fast_rcp(gasDisk) : 0.0);
  if ((ph & GAL_PHYS_STAR_FORMATION_DISK) && diskOk) {
    const double rateStars = (1.0 - p.recycled_fraction) * sfrDisk;
    const double rateMetals = zDisk * rateStars;
    dydt[GAL_Y_DISK_STARS] += rateStars;
    dydt[GAL_Y_DISK_GAS] += -rateStars;
    dydt[GAL_Y_DISK_STARS_METALS] += rateMetals;
    dydt[GAL_Y_DISK_GAS_METALS] += -rateMetals + p.metal_yield * sfrDisk;
  }
  // starFormationSpheroids (star_formation/spheroids.F90:152-)
  const bool sphOk = !(c.aSph < 1.0e-12 || gasSph < 1.0e-6);
  const double sfrSph = sphOk ? gasSph * c.sfrSph : 0.0;
  const double invSph = gasSph > 0.0 ? fast_rcp(gasSph) : 0.0;
  const double zSph = mass_fraction(y[GAL_Y_SPHEROID_GAS_METALS], gasSph, invSph);
  if ((ph & GAL_PHYS_STAR_FORMATION_SPHEROID) && sphOk) {
    const double rateStars = (1.0 - p.recycled_fraction) * sfrSph;
    dydt[GAL_Y_SPHEROID_STARS] += rateStars;
    dydt[GAL_Y_SPHEROID_GAS] += -rateStars;
    dydt[GAL_Y_SPHEROID_GAS_METALS] += -(zSph * rateStars) + p.metal_yield * sfrSph;
  }
  // stellarFeedbackDisks (stellar_feedback/disks.F90:116-205); rateLimit caps at the maximum.
  if ((ph & GAL_PHYS_FEEDBACK_DISK) && diskOk) {
    double total = c.outDisk * sfrDisk;
    if (c.outDiskMax >= 0.0) total = dmin(total, dmax(gasDisk * c.outDiskMax, 0.0));
    if (total > 0.0) {
      const double metals = gasDisk > 0.0 ? zDisk * total : 0.0;
      dydt[GAL_Y_OUTFLOWED_MASS] += total;
      dydt[GAL_Y_DISK_GAS] += -total;
      dydt[GAL_Y_OUTFLOWED_METALS] += metals;
      dydt[GAL_Y_DISK_GAS_METALS] += -metals;
    }
  }
  // stellarFeedbackSpheroids (stellar_feedback/spheroids.F90:116-208)
  if ((ph & GAL_PHYS_FEEDBACK_SPHEROID) && sphOk) {
    double total = c.outSph * sfrSph;
    if (c.outSphMax >= 0.0) total = dmin(total, dmax(gasSph * c.outSphMax, 0.0));
    if (total > 0.0) {
      const double metals = gasSph > 0.0 ? zSph * total : 0.0;
      dydt[GAL_Y_OUTFLOWED_MASS] += total;
      dydt[GAL_Y_SPHEROID_GAS] += -total;
      dydt[GAL_Y_OUTFLOWED_METALS] += metals;
      dydt[GAL_Y_SPHEROID_GAS_METALS] += -metals;
    }
  }
  // blackHolesAccretion (black_holes/accretion.F90:113-174) with
  // blackHoleAccretionRateStandard (black_holes/accretion_rates/standard.F90:221-440).
  const double massBH = y[GAL_Y_BLACK_HOLE];
  if ((ph & GAL_PHYS_BLACK_HOLE_ACCRETION) && massBH > 0.0) {
    const double eps = p.bh_efficiency_radiative;
    const double eddingtonCap = eps > 0.0 ? k::eddingtonPerMass * massBH / eps : 0.0;
    double rateSph = 0.0;
    if (gasSph > 0.0 && c.aSph > 0.0) {
      // Bondi-Hoyle from the spheroid gas (Hernquist density at max(r_BHL, Jeans length)).
      const double rAcc = dmax(G.bhRadiusSpheroidCoef * massBH, 0.0);
      double xx = rAcc * c.invASph, opx = 1.0 + xx;
      double rho = fast_div(gasSph * c.rhoSphPerMass, xx * opx * opx * opx);
      if (rho > 1.0) {
        const double jeans = dmin(G.jeansPrefactor * fast_rsqrt(rho), c.aSph);
        if (jeans > rAcc) {
          xx = jeans * c.invASph;
          opx = 1.0 + xx;
          rho = fast_div(gasSph * c.rhoSphPerMass, xx * opx * opx * opx);
        }
        rateSph = dmax(G.bhSpheroidCoef * massBH * massBH * rho, 0.0);
        if (eps > 0.0) rateSph = dmin(rateSph, eddingtonCap);
      }
    }
    double rateHot = 0.0;
    {
      const double rAcc = dmin(c.bhRadiusHotCoef > 0.0 ? c.bhRadiusHotCoef * massBH : HUGE_VAL, c.rOuter);
      double fractionHot = 1.0;
      if (p.bh_hot_mode_only) {
        // standardHotModeFraction (accretion_rates/standard.F90:442-468)
        rCool = cooling_radius(G, S, c, massHot, zHot, cv);
        coolingRadiusKnown = true;
        const double xx = rCool * c.invRvir;
        if (xx < 0.9) fractionHot = 1.0;
        else if (xx > 1.0) fractionHot = 0.0;
        else {
          const double u = (xx - 0.9) * 10.0;
          fractionHot = u * u * (2.0 * u - 3.0) + 1.0;
        }
      }
      if (massHot > 0.0 && fractionHot > 0.0) {
        const double xx = rAcc * c.invRcore;
        const double rho = fast_div(fractionHot * massHot * c.rho0PerMass, 1.0 + xx * xx);
        if (rho > 1.0) {
          rateHot = dmax(c.bhHotCoef * rAcc * rAcc * rho, 0.0);
          rateHot = dmin(rateHot, dmax(massHot * c.bhHotMaxCoef, 0.0));
          if (eps > 0.0) rateHot = dmin(rateHot, eddingtonCap);
        }
      }
    }
    const double total = rateSph + rateHot;
    if (total > 0.0) {
      dydt[GAL_Y_BLACK_HOLE] += total * (1.0 - p.bh_efficiency_radiative - p.bh_efficiency_jet);
      // spheroid gas sink (spheroid/standard/_class.F90:638-671)
      if (rateSph != 0.0 && gasSph > 0.0 && gasSph + y[GAL_Y_SPHEROID_STARS] > 0.0) {
        dydt[GAL_Y_SPHEROID_GAS] += -rateSph;
        dydt[GAL_Y_SPHEROID_GAS_METALS] += (-rateSph * invSph) * y[GAL_Y_SPHEROID_GAS_METALS];
      }
      // hot-halo mass sink (hot_halo/standard/_class.F90:771-799)
      if (rateHot != 0.0 && massHot > 0.0) {
        dydt[GAL_Y_HOT_MASS] += -rateHot;
        dydt[GAL_Y_HOT_METALS] += metalsHot * (-rateHot * invHot);
      }
    }
  }
  // CGMAccretion (circumgalactic_medium/accretion.F90:517-593; accretion/halo/simple.F90:281-319)
  if (ph & GAL_PHYS_CGM_ACCRETION) dydt[GAL_Y_HOT_MASS] += c.accretionRate;
  // CGMOutflowReincorporation (circumgalactic_medium/outflow_reincorporation.F90:272-349;
  // hot_halo/outflow_reincorporation/halo_dynamical_time.F90:113-128):
  // rate = M_out k, metals = rate MZ_out/M_out = MZ_out k.
  if (ph & GAL_PHYS_REINCORPORATION) {
    const double massOut = y[GAL_Y_OUTFLOWED_MASS];
    if (massOut > 0.0) {
      const double rate = massOut * c.reincorporationRate;
      const double metals = y[GAL_Y_OUTFLOWED_METALS] * c.reincorporationRate;
      dydt[GAL_Y_OUTFLOWED_MASS] += -rate;
      dydt[GAL_Y_OUTFLOWED_METALS] += -metals;
      dydt[GAL_Y_HOT_MASS] += rate;
      dydt[GAL_Y_HOT_METALS] += metals;
    }
  }
  // CGMCoolingHeating (circumgalactic_medium/cooling_heating.F90:216-381) with
  // coolingRateWhiteFrenk1991 (cooling/cooling_rate/White-Frenk.F90:132-185).
  if ((ph & GAL_PHYS_COOLING) && massHot > 0.0 && c.rOuter > 0.0) {
    double rate = 0.0;
    if (c.coolingAllowed) {
      if (!coolingRadiusKnown) rCool = cooling_radius(G, S, c, massHot, zHot, cv);
      if (rCool >= c.rOuter) {
        rate = massHot * c.invTdyn;
      } else if (rCool > 0.0) {
        // 4 pi r^2 rho(r) dr_cool/dt with dr/dt = r/t_avail/(2x^2/(1+x^2))
        // (cooling_radius/simple.F90:229-311, isothermal gas)
        //   = 2 pi rho(0) r_core^2 r_cool / t_dyn.
        rate = massHot * c.coolingRateCoef * rCool;
      }
    }
    if (rate > 0.0) {
      const double metals = rate * metalsHot * invHot;
      dydt[GAL_Y_HOT_MASS] += -rate;
      dydt[GAL_Y_HOT_METALS] += -metals;
      dydt[GAL_Y_DISK_GAS] += rate;
      dydt[GAL_Y_DISK_GAS_METALS] += metals;
    }
  }
}

// A secondary progenitor (the satellite) merging into the primary (the host)
// at their parent's time, with the mass movements of
// mergerMassMovementsSimple (satellites/merging/mass_movements/simple.F90,
// defaults: gas and stars of a minor merger's satellite to the host's
// spheroid, the host unmoved; a major merger -- the smaller galaxy at least
// ratioMajor of the larger in disk plus spheroid mass -- puts both galaxies
// into the spheroid).  The hot halo, its outflowed reservoir and the black
// hole add to the host's.  Stellar metals of a disk moving to the spheroid
// leave the state, which holds no spheroid stellar metals.
__host__ __device__ inline void merge_satellite(double* host, const double* sat, double ratioMajor) {
  const double massHost = host[GAL_Y_DISK_GAS] + host[GAL_Y_DISK_STARS] + host[GAL_Y_SPHEROID_GAS] + host[GAL_Y_SPHEROID_STARS];
  const double massSat = sat[GAL_Y_DISK_GAS] + sat[GAL_Y_DISK_STARS] + sat[GAL_Y_SPHEROID_GAS] + sat[GAL_Y_SPHEROID_STARS];
  const double smaller = massSat < massHost ? massSat : massHost, larger = massSat < massHost ? massHost : massSat;
  const bool major = massSat > 0.0 && massHost > 0.0 && smaller >= ratioMajor * larger;
  host[GAL_Y_HOT_MASS] += sat[GAL_Y_HOT_MASS];
  host[GAL_Y_HOT_METALS] += sat[GAL_Y_HOT_METALS];
  host[GAL_Y_OUTFLOWED_MASS] += sat[GAL_Y_OUTFLOWED_MASS];
  host[GAL_Y_OUTFLOWED_METALS] += sat[GAL_Y_OUTFLOWED_METALS];
  host[GAL_Y_BLACK_HOLE] += sat[GAL_Y_BLACK_HOLE];
  host[GAL_Y_SPHEROID_GAS] += sat[GAL_Y_DISK_GAS] + sat[GAL_Y_SPHEROID_GAS];
  host[GAL_Y_SPHEROID_GAS_METALS] += sat[GAL_Y_DISK_GAS_METALS] + sat[GAL_Y_SPHEROID_GAS_METALS];
  host[GAL_Y_SPHEROID_STARS] += sat[GAL_Y_DISK_STARS] + sat[GAL_Y_SPHEROID_STARS];
  if (major) {
    host[GAL_Y_SPHEROID_GAS] += host[GAL_Y_DISK_GAS];
    host[GAL_Y_SPHEROID_GAS_METALS] += host[GAL_Y_DISK_GAS_METALS];
    host[GAL_Y_SPHEROID_STARS] += host[GAL_Y_DISK_STARS];
    host[GAL_Y_DISK_GAS] = host[GAL_Y_DISK_GAS_METALS] = host[GAL_Y_DISK_STARS] = host[GAL_Y_DISK_STARS_METALS] = 0.0;
  }
}

// The components to create for one evaluation of an interrupt-form
// integration: those missing from `components` (GAL_COMPONENT_*) that
// receive a non-zero rate in one of their properties (a null component's
// rate function interrupts to create the component).
__device__ __forceinline__ int32_t interrupt_request(uint32_t components, const double* d) {
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

// Post-step clamps of the standard components (hot_halo/standard/_class.F90:
// 455-530, disk/standard/_class.F90:473-677, spheroid/standard/_class.F90:
// 464-636); all return GSL_Continue, so the evolver is not reset.  Returns
// whether any value was changed.
__device__ __forceinline__ bool post_step(double* y) {
  const bool any = y[GAL_Y_HOT_MASS] < 0.0 || y[GAL_Y_DISK_GAS] < 0.0 || y[GAL_Y_DISK_STARS] < 0.0 ||
                   y[GAL_Y_SPHEROID_GAS] < 0.0 || y[GAL_Y_SPHEROID_STARS] < 0.0;
  if (!any) return false;
  if (y[GAL_Y_HOT_MASS] < 0.0) y[GAL_Y_HOT_MASS] = 0.0;
  if (y[GAL_Y_DISK_GAS] < 0.0) {
    if (y[GAL_Y_DISK_GAS] + y[GAL_Y_DISK_STARS] == 0.0) {
      y[GAL_Y_DISK_STARS] = 0.0;
      y[GAL_Y_DISK_STARS_METALS] = 0.0;
    }
    y[GAL_Y_DISK_GAS] = 0.0;
    y[GAL_Y_DISK_GAS_METALS] = 0.0;
  }
  if (y[GAL_Y_DISK_STARS] < 0.0) {
    if (y[GAL_Y_DISK_GAS] + y[GAL_Y_DISK_STARS] == 0.0) {
      y[GAL_Y_DISK_GAS] = 0.0;
      y[GAL_Y_DISK_GAS_METALS] = 0.0;
    }
    y[GAL_Y_DISK_STARS] = 0.0;
    y[GAL_Y_DISK_STARS_METALS] = 0.0;
  }
  if (y[GAL_Y_SPHEROID_GAS] < 0.0) {
    if (y[GAL_Y_SPHEROID_GAS] + y[GAL_Y_SPHEROID_STARS] == 0.0) y[GAL_Y_SPHEROID_STARS] = 0.0;
    y[GAL_Y_SPHEROID_GAS] = 0.0;
    y[GAL_Y_SPHEROID_GAS_METALS] = 0.0;
  }
  if (y[GAL_Y_SPHEROID_STARS] < 0.0) {
    if (y[GAL_Y_SPHEROID_GAS] + y[GAL_Y_SPHEROID_STARS] == 0.0) {
      y[GAL_Y_SPHEROID_GAS] = 0.0;
      y[GAL_Y_SPHEROID_GAS_METALS] = 0.0;
    }
    y[GAL_Y_SPHEROID_STARS] = 0.0;
  }
  return true;
}

// post_step() with its test for a negative mass done on the integer pipe
// (exact, d_neg), so that the usual case -- nothing to clamp -- issues no
// FP64 compare.
__device__ __forceinline__ bool post_step_int(double* y) {
  if (!(d_neg(y[GAL_Y_HOT_MASS]) || d_neg(y[GAL_Y_DISK_GAS]) || d_neg(y[GAL_Y_DISK_STARS]) ||
        d_neg(y[GAL_Y_SPHEROID_GAS]) || d_neg(y[GAL_Y_SPHEROID_STARS])))
    return false;
  return post_step(y);
}

// Absolute-tolerance scales from the initial state (scaleSetTask hooks of
// hot_halo :804-850, disk :735-824, spheroid :804-897, black hole :195-257).
__device__ __forceinline__ void scales(const double* y, double massHalo, double* s) {
  const double hot = massHalo * 1.0e-3;
  s[GAL_Y_HOT_MASS] = s[GAL_Y_HOT_METALS] = s[GAL_Y_OUTFLOWED_MASS] = s[GAL_Y_OUTFLOWED_METALS] = hot;
  const double mass = fmax(fabs(y[GAL_Y_DISK_GAS]) + fabs(y[GAL_Y_SPHEROID_GAS]) + fabs(y[GAL_Y_DISK_STARS]) +
                               fabs(y[GAL_Y_SPHEROID_STARS]), 1.0);
  const double metals = fmax(fabs(y[GAL_Y_DISK_GAS_METALS]) + fabs(y[GAL_Y_DISK_STARS_METALS]) + fabs(y[GAL_Y_SPHEROID_GAS_METALS]),
                             fmax(mass * 1.0e-4, 1.0));
  s[GAL_Y_DISK_GAS] = s[GAL_Y_DISK_STARS] = s[GAL_Y_SPHEROID_GAS] = s[GAL_Y_SPHEROID_STARS] = mass;
  s[GAL_Y_DISK_GAS_METALS] = s[GAL_Y_DISK_STARS_METALS] = s[GAL_Y_SPHEROID_GAS_METALS] = metals;
  const double stars = y[GAL_Y_SPHEROID_STARS] > 0.0 ? y[GAL_Y_SPHEROID_STARS] : 0.0;
  s[GAL_Y_BLACK_HOLE] = fmax(fmax(1.0, 1.0e-4 * stars), y[GAL_Y_BLACK_HOLE]);
}

}  // namespace gal
