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
// constants are the per-node constants of node_setup() rounded to FP32,
// grouped so that no intermediate leaves the FP32 range for halo masses of
// 1e6-1e16 Msun.
#pragma once

#include "galnode_physics.cuh"

namespace gal {

// FP32 copies of the per-node constants of NodeC.
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
  float sfrDisk, sfrSph;
  float outDisk, outSph, outDiskMax, outSphMax;
  float aSph, invASph, rhoSphPerMass, radiusDisk;
  float bhRadiusHotCoef, bhHotCoef, bhHotMaxCoef;
  float accretionRate, reincorporationRate;
};

__device__ __forceinline__ NodeF node_fast(const NodeC& c) {
  NodeF f;
  f.tdyn = (float)c.tdyn;
  f.invTdyn = (float)c.invTdyn;
  f.rcore = (float)c.rcore;
  f.invRcore = (float)c.invRcore;
  f.rho0PerMass = (float)c.rho0PerMass;
  f.rOuter = (float)c.rOuter;
  f.invRvir = (float)c.invRvir;
  f.onePlusXOuter2 = (float)c.onePlusXOuter2;
  f.coolingQCoef = (float)(c.tdyn * c.rho0PerMass / c.coolingTimeCoef);
  f.coolingRateCoef = (float)c.coolingRateCoef;
  f.hT = (float)c.hT;
  f.iT = c.iT;
  f.coolingAllowed = c.coolingAllowed;
  f.log10T = c.log10T;
  f.sfrDisk = (float)c.sfrDisk;
  f.sfrSph = (float)c.sfrSph;
  f.outDisk = (float)c.outDisk;
  f.outSph = (float)c.outSph;
  f.outDiskMax = (float)c.outDiskMax;
  f.outSphMax = (float)c.outSphMax;
  f.aSph = (float)c.aSph;
  f.invASph = (float)c.invASph;
  f.rhoSphPerMass = (float)c.rhoSphPerMass;
  f.radiusDisk = (float)c.radiusDisk;
  f.bhRadiusHotCoef = (float)c.bhRadiusHotCoef;
  f.bhHotCoef = (float)c.bhHotCoef;
  f.bhHotMaxCoef = (float)c.bhHotMaxCoef;
  f.accretionRate = (float)c.accretionRate;
  f.reincorporationRate = (float)c.reincorporationRate;
  return f;
}

// FP32 copy of the CIE tables in shared memory: (ln Lambda, ln n_e/n_H)
// [nZ][nT], ln Z/Zsun [nZ], 1/(ln Z[i+1] - ln Z[i]) [nZ].
struct SmemF {
  const float2* tab;
  const float* lnZ;
  const float* invDlnZ;
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
  const float sfrDisk = diskOk ? gasDisk * c.sfrDisk : 0.0f;
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
