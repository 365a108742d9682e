// galnode_physics_fast.cuh -- the P-std right-hand side with FP32 rate
// arithmetic, for the fast form of the evolver.
//
// GB300 issues FP64 at one warp instruction per ~64 cycles on each SM
// sub-partition (about 1/64 of its FP32 rate), and the FP64 right-hand side
// is ~300 such instructions, so in the plain form a node's integration time
// is set by the FP64 pipe however few lanes are busy.  The fast form keeps
// what the masses need in FP64 -- the state vector, the accepted-step
// update, the error norm and the step-size control -- and evaluates the
// rates (star formation, feedback, black-hole accretion, cooling) in FP32:
// a rate is only ever used as an increment h*k_i to a state held in FP64,
// and its FP32 rounding (~6e-8 relative) is four orders of magnitude below
// the relative tolerance of the step controller.
//
// Every branch restates the same reference function as the FP64 rhs() in
// galnode_physics.cuh (same operators, same order, same clamps); the
// constants are the per-node constants of node_setup(), formed in FP32 by
// node_setup_fast() and grouped so that no intermediate leaves the FP32
// range for halo masses of 1e6-1e16 Msun.
#pragma once

#include "galnode_physics.cuh"

namespace gal {

// The per-node constants of NodeC in FP32 (node_setup_fast()).
struct NodeF {
  float tdyn, invTdyn;
  float rcore, invRcore;
  float rho0PerMass;
  float rOuter, invRvir;
  float onePlusXOuter2;
  float coolingQCoef;        // t_dyn rho0PerMass / coolingTimeCoef: q = coef Lambda M_hot X_H^2 / (...)
  float coolingRateCoef;
  float hT;
  int iT;
  int coolingAllowed;
  float log10T;
  int netRow;                // as NodeC::netRow
  float sfrDisk, sfrSph;
  float outDisk, outSph, outDiskMax, outSphMax;
  float aSph, invASph, rhoSphPerMass, radiusDisk;
  float bhRadiusHotCoef, bhHotCoef, bhHotMaxCoef;
  float accretionRate, reincorporationRate;
};

// node_setup() for the FP32-rate forms: the same constants (same reference
// functions, same guards), formed in FP32 from r_vir, V_vir, the spin and
// the host-folded coefficients of Globals::Fast, so that setting up a node
// issues no FP64 division, logarithm or power.  Its values agree with the
// FP64 node_setup() rounded to FP32 to a few FP32 ulps (the powers to ~1e-6
// relative), far inside the rates' own FP32 rounding against the tolerance.
// The T cell is found by arithmetic when the table rows are evenly spaced
// in ln T.
__device__ __forceinline__ void node_setup_fast(const Globals& G, const double* sLnT, const double* prm, NodeF& f) {
  const Globals::Fast& g = G.f;
  const gal_params& p = G.p;
  const double vvirD = prm[GAL_P_VELOCITY_VIRIAL];
  const float rvir = (float)prm[GAL_P_RADIUS_VIRIAL], vvir = (float)vvirD, spin = (float)prm[GAL_P_SPIN];
  const double mdot = prm[GAL_P_MASS_RATE];
  // virialDensityContrastDefinition{VirialTemperature,DynamicalTimescale} (virial_density_contrast.F90:195-262)
  const float T = g.tempPerV2 * vvir * vvir;
  f.tdyn = g.tdynCoef * rvir / vvir;
  f.invTdyn = 1.0f / f.tdyn;
  const float rcore = g.coreFraction * rvir;
  f.rcore = rcore;
  f.invRcore = 1.0f / rcore;
  f.rOuter = rvir;  // hot_halo/standard/_class.F90:430-450
  f.invRvir = 1.0f / rvir;
  // beta-profile normalisation (beta_profile.F90:190-320): r_outer/r_core is the same for every node.
  f.rho0PerMass = g.rho0Norm / (rcore * rcore * rcore);
  f.onePlusXOuter2 = g.onePlusXOuter2;
  f.coolingRateCoef = g.twoPiRho0Norm / rcore * f.invTdyn;
  f.coolingQCoef = f.tdyn * f.rho0PerMass / (g.coolingCoef * T);
  // Temperature coordinate of the CIE tables ("extrapolate" in T = clamp).
  const float lnT = logf(fminf(fmaxf(T, g.Tmin), g.Tmax));
  const int last = G.nT - 2;
  if (G.tUniform) {
    const float u = (lnT - g.lnTFirst) * g.invDlnT;
    int j = (int)floorf(u);
    j = j < 0 ? 0 : (j > last ? last : j);
    f.iT = j;
    f.hT = u - (float)j;
  } else {
    int lo = 0, hi = G.nT - 1;
    if (lnT >= (float)sLnT[hi]) lo = last;
    else
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((float)sLnT[mid] <= lnT) lo = mid; else hi = mid;
      }
    f.iT = lo;
    f.hT = (lnT - (float)sLnT[lo]) / ((float)sLnT[lo + 1] - (float)sLnT[lo]);
  }
  f.log10T = T > 0.0f ? log10f(T) : -1.0e30f;
  f.coolingAllowed = !(vvirD > p.cooling_velocity_cutoff);
  // galacticStructureSolverFixed: r = f lambda r_vir.
  const float Rd = g.radiusFactorDisk * spin * rvir, Rs = g.radiusFactorSpheroid * spin * rvir;
  f.radiusDisk = Rd;
  f.aSph = Rs;
  f.invASph = Rs > 0.0f ? 1.0f / Rs : 0.0f;
  f.rhoSphPerMass = Rs > 0.0f ? g.invTwoPi / (Rs * Rs * Rs) : 0.0f;
  // Star-formation timescales (star_formation/timescales/dynamical_time.F90:121-189).
  auto timescale = [&](const gal_star_formation& sf, const Globals::Fast::Sf& s, float R) -> float {
    if (sf.timescale_type == GAL_SF_TIMESCALE_FIXED) return s.fixed;
    if (vvir <= 0.0f || s.efficiency == 0.0f) return 0.0f;
    const float t = g.tdynCoef * R / vvir;
    return fmaxf(t * powf(vvir * (1.0f / 200.0f), s.exponent) / s.efficiency, s.minimum);
  };
  const float tsD = timescale(p.sf_disk, g.sfDisk, Rd), tsS = timescale(p.sf_spheroid, g.sfSph, Rs);
  f.sfrDisk = tsD > 0.0f ? 1.0f / tsD : 0.0f;
  f.sfrSph = tsS > 0.0f ? 1.0f / tsS : 0.0f;
  // Outflow loading (power_law/_class.F90:118-164, fixed.F90) and rateLimit (rate_limit.F90).
  auto loading = [&](const gal_outflow& o, const Globals::Fast::Out& s) -> float {
    if (o.type == GAL_OUTFLOW_FIXED) return s.fraction;
    if (vvir <= 0.0f) return 0.0f;
    return powf(s.velocity / vvir, s.exponent);
  };
  auto limit = [&](const Globals::Fast::Out& s, float R) -> float {
    if (!(s.fractionalMinimum > 0.0f)) return -1.0f;
    const float t = (vvir <= 0.0f || R <= 0.0f) ? 1.0f : g.tdynCoef * R / vvir;
    return 1.0f / t / s.fractionalMinimum;
  };
  f.outDisk = loading(p.outflow_disk, g.outDisk);
  f.outSph = loading(p.outflow_spheroid, g.outSph);
  f.outDiskMax = limit(g.outDisk, Rd);
  f.outSphMax = limit(g.outSph, Rs);
  // Hot-halo Bondi accretion constants at the virial temperature.
  const float cs2 = g.csSquaredPerT * T, cs = sqrtf(cs2);
  f.bhRadiusHotCoef = T > 0.0f ? g.gravitationalConstant / cs2 : 0.0f;
  f.bhHotCoef = g.bhHotPrefactor * cs;
  f.bhHotMaxCoef = cs / (f.rOuter * g.tdynCoef);
  f.accretionRate = mdot > 0.0 ? g.accretionFraction * (float)mdot : 0.0f;
  f.reincorporationRate = g.reincorporationMultiplier * f.invTdyn;
}

// Absolute-tolerance scales of the components (scales() in FP32, from the
// FP32 copy of the state): hot-halo and outflowed components 1e-3 of the
// halo mass (hot_halo/standard/_class.F90:804-850), disk and spheroid
// masses and metals from the galaxy's total (disk :735-824, spheroid
// :804-897), the black hole from the seed and the spheroid (:195-257).
__device__ __forceinline__ void scales_fast(const float* y, float massHalo, float* s) {
  const float hot = massHalo * 1.0e-3f;
  s[GAL_Y_HOT_MASS] = s[GAL_Y_HOT_METALS] = s[GAL_Y_OUTFLOWED_MASS] = s[GAL_Y_OUTFLOWED_METALS] = hot;
  const float mass = fmaxf(fabsf(y[GAL_Y_DISK_GAS]) + fabsf(y[GAL_Y_SPHEROID_GAS]) + fabsf(y[GAL_Y_DISK_STARS]) +
                               fabsf(y[GAL_Y_SPHEROID_STARS]), 1.0f);
  const float metals = fmaxf(fabsf(y[GAL_Y_DISK_GAS_METALS]) + fabsf(y[GAL_Y_DISK_STARS_METALS]) +
                                 fabsf(y[GAL_Y_SPHEROID_GAS_METALS]),
                             fmaxf(mass * 1.0e-4f, 1.0f));
  s[GAL_Y_DISK_GAS] = s[GAL_Y_DISK_STARS] = s[GAL_Y_SPHEROID_GAS] = s[GAL_Y_SPHEROID_STARS] = mass;
  s[GAL_Y_DISK_GAS_METALS] = s[GAL_Y_DISK_STARS_METALS] = s[GAL_Y_SPHEROID_GAS_METALS] = metals;
  const float stars = y[GAL_Y_SPHEROID_STARS] > 0.0f ? y[GAL_Y_SPHEROID_STARS] : 0.0f;
  s[GAL_Y_BLACK_HOLE] = fmaxf(fmaxf(1.0f, 1.0e-4f * stars), y[GAL_Y_BLACK_HOLE]);
}

// FP32 copy of the CIE tables in shared memory: (ln Lambda, ln n_e/n_H)
// [nZ][nT], ln Z/Zsun [nZ], 1/(ln Z[i+1] - ln Z[i]) [nZ].
struct SmemF {
  const float2* tab;
  const float* lnZ;
  const float* invDlnZ;
  KmtTables<float> kmt;  // Krumholz (2009) tables (global memory)
};

struct CoolingValuesF {
  bool use;
  float lambda, electrons;
};

// cie_lookup() in FP32 (CIE_file.F90:238-317, 665-735): the metallicity
// cell by arithmetic on an evenly spaced grid (else by bisection), bilinear
// interpolation of the logs, exp.
__device__ __forceinline__ void cie_lookup_fast(const Globals& G, const SmemF& S, const NodeF& c, float zSolar, float& lambda,
                                               float& electrons) {
  zSolar = fminf(fmaxf(zSolar, G.f.Zmin), G.f.Zmax);  // "fix" extrapolation in metallicity
  const float zUse = fmaxf(zSolar, 0.0f);
  int iZ;
  float hZ;
  if (G.firstZero && zUse < G.f.firstNonZero) {
    iZ = 0;
    hZ = zUse * G.f.invFirstNonZero;
  } else {
    const float lnZ = __logf(zUse);
    const int last = G.nZ - 2;
    if (G.zUniform) {
      int j = G.zFirstLog + (int)floorf((lnZ - G.f.lnZFirst) * G.f.invDlnZ);
      iZ = j < G.zFirstLog ? G.zFirstLog : (j > last ? last : j);
    } else {
      int lo = G.zFirstLog, hi = G.nZ - 1;
      if (lnZ >= S.lnZ[hi]) lo = last;
      else
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (S.lnZ[mid] <= lnZ) lo = mid; else hi = mid;
        }
      iZ = lo;
    }
    hZ = (lnZ - S.lnZ[iZ]) * S.invDlnZ[iZ];
  }
  const int nT = G.nT;
  const float2 a = S.tab[iZ * nT + c.iT], b = S.tab[(iZ + 1) * nT + c.iT];
  const float2 d = S.tab[iZ * nT + c.iT + 1], e = S.tab[(iZ + 1) * nT + c.iT + 1];
  const float hT = c.hT;
  const float w00 = (1.0f - hT) * (1.0f - hZ), w01 = (1.0f - hT) * hZ, w10 = hT * (1.0f - hZ), w11 = hT * hZ;
  lambda = __expf(a.x * w00 + b.x * w01 + d.x * w10 + e.x * w11);
  electrons = __expf(a.y * w00 + b.y * w01 + d.y * w10 + e.y * w11);
}

// cooling_radius() in FP32: r = r_core sqrt(t_avail/t_cool(0) - 1) in
// [0, r_outer] (cooling_radius/simple.F90:313-427, cooling_time/simple.F90:128-179).
__device__ __forceinline__ float cooling_radius_fast(const Globals& G, const SmemF& S, const NodeF& c, float massHot, float zHot,
                                                    const CoolingValuesF& cv) {
  const float zs = zHot * (float)(1.0 / k::metallicitySolar);
  const float xH = fminf(fmaxf(zs * (float)(k::hydrogenByMassSolar - k::hydrogenByMassPrimordial) + (float)k::hydrogenByMassPrimordial,
                               0.7f),
                         (float)k::hydrogenByMassPrimordial);
  const float yHe = fminf(zs * (float)(k::heliumByMassSolar - k::heliumByMassPrimordial) + (float)k::heliumByMassPrimordial,
                          (float)k::heliumByMassPrimordial);
  float lambda, electrons;
  if (cv.use) {
    lambda = cv.lambda;
    electrons = cv.electrons;
  } else {
    cie_lookup_fast(G, S, c, zs, lambda, electrons);
  }
  const float num = c.coolingQCoef * lambda * massHot * xH * xH;
  const float den = xH * (1.0f + electrons) + yHe * (float)(k::atomicMassHydrogen / k::atomicMassHelium);
  const float q = massHot > 0.0f ? __fdividef(num, den) : 0.0f;
  if (q > c.onePlusXOuter2) return c.rOuter;
  if (q < 1.0f) return 0.0f;
  const float q1 = q - 1.0f;
  return c.rcore * (q1 * rsqrtf(q1));  // sqrt by the hardware reciprocal square root (~2 ulp)
}

__device__ __forceinline__ float mass_fraction_f(float metals, float mass, float invMass) {
  return metals > mass ? 1.0f : (metals <= 0.0f ? 0.0f : metals * invMass);
}

// rhs() in FP32: the node operators of nodeOperatorMulti
// (nodes/operators/multi.F90:313-332), branch by branch as in rhs().
template <bool KMT = false>
__device__ __forceinline__ void rhs_fast(const Globals& G, const SmemF& S, const NodeF& c, const float* y, float* dydt,
                                        const CoolingValuesF& cv = CoolingValuesF{false, 0.0f, 0.0f}) {
  const gal_params& p = G.p;
  const uint32_t ph = p.physics;
#pragma unroll
  for (int i = 0; i < GAL_NY; ++i) dydt[i] = 0.0f;
  const float oneMinusR = G.f.oneMinusR, yield = G.f.metalYield;
  const float massHot = y[GAL_Y_HOT_MASS], metalsHot = y[GAL_Y_HOT_METALS];
  const float gasDisk = y[GAL_Y_DISK_GAS], gasSph = y[GAL_Y_SPHEROID_GAS];
  // Reciprocals by the hardware approximation (~1 ulp): these are FP32 rates.
  const float invHot = massHot > 0.0f ? __fdividef(1.0f, massHot) : 0.0f;
  const float zHot = mass_fraction_f(metalsHot, massHot, invHot);
  bool coolingRadiusKnown = false;
  float rCool = 0.0f;

  // starFormationDisks (star_formation/disks.F90:200-324) + instantaneous populations
  // (stellar_populations/properties/instantaneous.F90:133-219).
  const bool diskOk = !(c.radiusDisk < 0.0f || gasDisk < 0.0f);
  float sfrDisk = 0.0f;
  if (diskOk) {
    if constexpr (KMT)
      sfrDisk = krumholz2009_rate<float>(S.kmt, G.f.kmtFrequency, G.f.kmtClumping, G.f.kmtSTruncation,
                                         p.krumholz_fast != 0, gasDisk, y[GAL_Y_DISK_GAS_METALS], c.radiusDisk);
    else
      sfrDisk = gasDisk * c.sfrDisk;
  }
  const float zDisk = mass_fraction_f(y[GAL_Y_DISK_GAS_METALS], gasDisk, gasDisk > 0.0f ? __fdividef(1.0f, gasDisk) : 0.0f);
  if ((ph & GAL_PHYS_STAR_FORMATION_DISK) && diskOk) {
    const float rateStars = oneMinusR * sfrDisk;
    const float rateMetals = zDisk * rateStars;
    dydt[GAL_Y_DISK_STARS] += rateStars;
    dydt[GAL_Y_DISK_GAS] += -rateStars;
    dydt[GAL_Y_DISK_STARS_METALS] += rateMetals;
    dydt[GAL_Y_DISK_GAS_METALS] += -rateMetals + yield * sfrDisk;
  }
  // starFormationSpheroids (star_formation/spheroids.F90:152-)
  const bool sphOk = !(c.aSph < 1.0e-12f || gasSph < 1.0e-6f);
  const float sfrSph = sphOk ? gasSph * c.sfrSph : 0.0f;
  const float invSph = gasSph > 0.0f ? __fdividef(1.0f, gasSph) : 0.0f;
  const float zSph = mass_fraction_f(y[GAL_Y_SPHEROID_GAS_METALS], gasSph, invSph);
  if ((ph & GAL_PHYS_STAR_FORMATION_SPHEROID) && sphOk) {
    const float rateStars = oneMinusR * sfrSph;
    dydt[GAL_Y_SPHEROID_STARS] += rateStars;
    dydt[GAL_Y_SPHEROID_GAS] += -rateStars;
    dydt[GAL_Y_SPHEROID_GAS_METALS] += -(zSph * rateStars) + yield * sfrSph;
  }
  // stellarFeedbackDisks (stellar_feedback/disks.F90:116-205); rateLimit caps at the maximum.
  if ((ph & GAL_PHYS_FEEDBACK_DISK) && diskOk) {
    float total = c.outDisk * sfrDisk;
    if (c.outDiskMax >= 0.0f) total = fminf(total, fmaxf(gasDisk * c.outDiskMax, 0.0f));
    if (total > 0.0f) {
      const float metals = gasDisk > 0.0f ? zDisk * total : 0.0f;
      dydt[GAL_Y_OUTFLOWED_MASS] += total;
      dydt[GAL_Y_DISK_GAS] += -total;
      dydt[GAL_Y_OUTFLOWED_METALS] += metals;
      dydt[GAL_Y_DISK_GAS_METALS] += -metals;
    }
  }
  // stellarFeedbackSpheroids (stellar_feedback/spheroids.F90:116-208)
  if ((ph & GAL_PHYS_FEEDBACK_SPHEROID) && sphOk) {
    float total = c.outSph * sfrSph;
    if (c.outSphMax >= 0.0f) total = fminf(total, fmaxf(gasSph * c.outSphMax, 0.0f));
    if (total > 0.0f) {
      const float metals = gasSph > 0.0f ? zSph * total : 0.0f;
      dydt[GAL_Y_OUTFLOWED_MASS] += total;
      dydt[GAL_Y_SPHEROID_GAS] += -total;
      dydt[GAL_Y_OUTFLOWED_METALS] += metals;
      dydt[GAL_Y_SPHEROID_GAS_METALS] += -metals;
    }
  }
  // blackHolesAccretion (black_holes/accretion.F90:113-174) with
  // blackHoleAccretionRateStandard (black_holes/accretion_rates/standard.F90:221-440).
  const float massBH = y[GAL_Y_BLACK_HOLE];
  if ((ph & GAL_PHYS_BLACK_HOLE_ACCRETION) && massBH > 0.0f) {
    const bool capped = G.f.capped;
    const float eddingtonCap = G.f.eddingtonOverEps * massBH;
    float rateSph = 0.0f;
    if (gasSph > 0.0f && c.aSph > 0.0f) {
      // Bondi-Hoyle from the spheroid gas (Hernquist density at max(r_BHL, Jeans length)).
      const float rAcc = fmaxf(G.f.bhRadiusSpheroidCoef * massBH, 0.0f);
      float xx = rAcc * c.invASph, opx = 1.0f + xx;
      float rho = __fdividef(gasSph * c.rhoSphPerMass, xx * opx * opx * opx);
      if (rho > 1.0f) {
        const float jeans = fminf(G.f.jeansPrefactor * rsqrtf(rho), c.aSph);
        if (jeans > rAcc) {
          xx = jeans * c.invASph;
          opx = 1.0f + xx;
          rho = __fdividef(gasSph * c.rhoSphPerMass, xx * opx * opx * opx);
        }
        rateSph = fmaxf(G.f.bhSpheroidCoef * massBH * massBH * rho, 0.0f);
        if (capped) rateSph = fminf(rateSph, eddingtonCap);
      }
    }
    float rateHot = 0.0f;
    {
      const float rAcc = fminf(c.bhRadiusHotCoef > 0.0f ? c.bhRadiusHotCoef * massBH : HUGE_VALF, c.rOuter);
      float fractionHot = 1.0f;
      if (p.bh_hot_mode_only) {
        // standardHotModeFraction (accretion_rates/standard.F90:442-468)
        rCool = cooling_radius_fast(G, S, c, massHot, zHot, cv);
        coolingRadiusKnown = true;
        const float xx = rCool * c.invRvir;
        if (xx < 0.9f) fractionHot = 1.0f;
        else if (xx > 1.0f) fractionHot = 0.0f;
        else {
          const float u = (xx - 0.9f) * 10.0f;
          fractionHot = u * u * (2.0f * u - 3.0f) + 1.0f;
        }
      }
      if (massHot > 0.0f && fractionHot > 0.0f) {
        const float xx = rAcc * c.invRcore;
        const float rho = __fdividef(fractionHot * massHot * c.rho0PerMass, 1.0f + xx * xx);
        if (rho > 1.0f) {
          rateHot = fmaxf(c.bhHotCoef * rAcc * rAcc * rho, 0.0f);
          rateHot = fminf(rateHot, fmaxf(massHot * c.bhHotMaxCoef, 0.0f));
          if (capped) rateHot = fminf(rateHot, eddingtonCap);
        }
      }
    }
    const float total = rateSph + rateHot;
    if (total > 0.0f) {
      dydt[GAL_Y_BLACK_HOLE] += total * G.f.bhRetained;
      // spheroid gas sink (spheroid/standard/_class.F90:638-671)
      if (rateSph != 0.0f && gasSph > 0.0f && gasSph + y[GAL_Y_SPHEROID_STARS] > 0.0f) {
        dydt[GAL_Y_SPHEROID_GAS] += -rateSph;
        dydt[GAL_Y_SPHEROID_GAS_METALS] += (-rateSph * invSph) * y[GAL_Y_SPHEROID_GAS_METALS];
      }
      // hot-halo mass sink (hot_halo/standard/_class.F90:771-799)
      if (rateHot != 0.0f && massHot > 0.0f) {
        dydt[GAL_Y_HOT_MASS] += -rateHot;
        dydt[GAL_Y_HOT_METALS] += metalsHot * (-rateHot * invHot);
      }
    }
  }
  // CGMAccretion (circumgalactic_medium/accretion.F90:517-593; accretion/halo/simple.F90:281-319)
  if (ph & GAL_PHYS_CGM_ACCRETION) dydt[GAL_Y_HOT_MASS] += c.accretionRate;
  // CGMOutflowReincorporation (circumgalactic_medium/outflow_reincorporation.F90:272-349;
  // hot_halo/outflow_reincorporation/halo_dynamical_time.F90:113-128).
  if (ph & GAL_PHYS_REINCORPORATION) {
    const float massOut = y[GAL_Y_OUTFLOWED_MASS];
    if (massOut > 0.0f) {
      const float rate = massOut * c.reincorporationRate;
      const float metals = y[GAL_Y_OUTFLOWED_METALS] * c.reincorporationRate;
      dydt[GAL_Y_OUTFLOWED_MASS] += -rate;
      dydt[GAL_Y_OUTFLOWED_METALS] += -metals;
      dydt[GAL_Y_HOT_MASS] += rate;
      dydt[GAL_Y_HOT_METALS] += metals;
    }
  }
  // CGMCoolingHeating (circumgalactic_medium/cooling_heating.F90:216-381) with
  // coolingRateWhiteFrenk1991 (cooling/cooling_rate/White-Frenk.F90:132-185).
  if ((ph & GAL_PHYS_COOLING) && massHot > 0.0f && c.rOuter > 0.0f) {
    float rate = 0.0f;
    if (c.coolingAllowed) {
      if (!coolingRadiusKnown) rCool = cooling_radius_fast(G, S, c, massHot, zHot, cv);
      if (rCool >= c.rOuter) {
        rate = massHot * c.invTdyn;
      } else if (rCool > 0.0f) {
        rate = massHot * c.coolingRateCoef * rCool;
      }
    }
    if (rate > 0.0f) {
      const float metals = rate * metalsHot * invHot;
      dydt[GAL_Y_HOT_MASS] += -rate;
      dydt[GAL_Y_HOT_METALS] += -metals;
      dydt[GAL_Y_DISK_GAS] += rate;
      dydt[GAL_Y_DISK_GAS_METALS] += metals;
    }
  }
}

}  // namespace gal
