// trees.cpp -- host merger-tree builder: Cole et al. (2000) binary-split
// trees with the Parkinson, Cole & Helly (2008, MNRAS 383, 557) branching
// rates, as the reference builds them (merger_trees/construct/builder/
// Cole2000/_class.F90:360-913, merger_trees/branching_probability/
// Parkinson_Cole_Helly.F90:265-634).
//
// Each tree is grown backwards in time from its root in the variable
// w = delta_c(z) = delta_c0 / D(z).  For a branch of mass M2 at w the
// progenitor mass function per unit w is (extended Press-Schechter, with the
// PCH modifier G)
//   dN/dq = (1/sqrt(2 pi)) q^-2 |dS1/dln M1| (S1 - S2)^-3/2 G,
//   G = G0 (sigma1/sigma2)^gamma1 (w/sigma2)^gamma2,   q = M1/M2,  S = sigma^2,
// so a step dw splits off a resolved progenitor (q in [q_res, 1/2]) with
// probability R dw, R = int dN/dq dq, and loses the fraction F dw of its mass
// to progenitors below the resolution,
//   F = (1/sqrt(2 pi)) int_{S_res}^inf (S1 - S2)^-3/2 G dS1
//     = (2/sqrt(2 pi)) int_0^{u_res} G du,   u = (S1 - S2)^-1/2.
// The step is limited so that R dw, F dw and dw / sqrt(2 (S(M2/2) - S2))
// stay below the accuracy parameters.  A split creates two progenitor nodes
// (the larger one first); a branch that drops below the resolution or
// reaches the maximum redshift ends in a leaf node.
//
// sigma(M) is that of a power law n_s times the transfer function squared,
// normalised to sigma8: by default the Eisenstein & Hu (1999) fit with
// massive-neutrino suppression, the reference's default (transfer_function/
// Eisenstein_Hu1999.F90), or the Eisenstein & Hu (1998) zero-baryon form;
// D(z) is the linear growth factor of a flat matter + Lambda model;
// delta_c0 = 3 (12 pi)^(2/3) / 20.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <random>
#include <vector>
#include <algorithm>
#include <chrono>

#include "../../include/galnode_forest.h"
#include "trees_internal.h"

namespace {

using gal::trees::GrownNode;

constexpr double kPi = 3.14159265358979323846;
constexpr double kGravity = 6.673e-11 * 1.98892e30 / 1.0e6 / (1.0e6 * 3.08567758135e16);  // km^2 s^-2 Mpc / Msun
constexpr double kMpcPerKmPerSToGyr = 1.0e6 * 3.08567758135e16 / 1.0e3 / (1.0e9 * 3.15581497635456e7);

struct Cosmo {
  double om, ol, ob, h0;  // h0 in km/s/Mpc
  double hubbleGyr() const { return h0 / kMpcPerKmPerSToGyr; }
  double time(double z) const {
    const double a = 1.0 / (1.0 + z);
    return 2.0 / (3.0 * hubbleGyr() * std::sqrt(ol)) * std::asinh(std::sqrt(ol / om) * std::pow(a, 1.5));
  }
  double redshift(double t) const {
    const double x = std::sinh(1.5 * hubbleGyr() * std::sqrt(ol) * t);
    const double a = std::pow(x / std::sqrt(ol / om), 2.0 / 3.0);
    return 1.0 / a - 1.0;
  }
};

Cosmo cosmo_of(const gal_params* p) { return Cosmo{p->omega_matter, p->omega_dark_energy, p->omega_baryon, p->hubble_constant}; }

// Eisenstein & Hu (1998) zero-baryon ("no wiggle") transfer function, k in 1/Mpc.
double transfer_no_wiggle(double k, const Cosmo& c, double tcmb) {
  const double h = c.h0 / 100.0;
  const double omh2 = c.om * h * h, obh2 = c.ob * h * h, fb = c.ob / c.om;
  const double theta = tcmb / 2.7;
  const double s = 44.5 * std::log(9.83 / omh2) / std::sqrt(1.0 + 10.0 * std::pow(obh2, 0.75));
  const double alpha = 1.0 - 0.328 * std::log(431.0 * omh2) * fb + 0.38 * std::log(22.3 * omh2) * fb * fb;
  const double ks = 0.43 * k * s;
  const double gammaEff = omh2 * (alpha + (1.0 - alpha) / (1.0 + ks * ks * ks * ks));  // Omega_m h^2 (...) per Mpc^-1
  const double q = k * theta * theta / gammaEff;
  const double l0 = std::log(2.0 * std::exp(1.0) + 1.8 * q);
  const double c0 = 14.2 + 731.0 / (1.0 + 62.5 * q);
  return l0 / (l0 + c0 * q * q);
}

// Eisenstein & Hu (1999, ApJ 511, 5) transfer function of cold dark matter,
// baryons and massive neutrinos, k in 1/Mpc, as the reference evaluates it
// (transfer_function/Eisenstein_Hu1999.F90:100-420): the shape parameter
// with the small-scale suppression alpha_nu (eqs. 15-16), the zero-baryon
// form L / (L + C q_eff^2) (eqs. 17-20) with beta_c (eq. 21), and the
// suppression near the neutrino free-streaming scale for 0 < f_nu <= 0.3.
struct EisensteinHu1999 {
  double omh2, theta, s, alphaNu, betaC, fNu, nEff;

  EisensteinHu1999(const Cosmo& c, const gal_pch_params& pch) {
    const double h = c.h0 / 100.0;
    omh2 = c.om * h * h;
    const double obh2 = c.ob * h * h;
    theta = pch.temperature_cmb / 2.7;
    const double zEq = 2.50e4 * omh2 / std::pow(theta, 4);
    const double b1 = 0.313 * std::pow(omh2, -0.419) * (1.0 + 0.607 * std::pow(omh2, 0.674));
    const double b2 = 0.238 * std::pow(omh2, 0.223);
    const double zDrag = 1291.0 * std::pow(omh2, 0.251) * (1.0 + b1 * std::pow(obh2, b2)) / (1.0 + 0.659 * std::pow(omh2, 0.828));
    const double yD = (1.0 + zEq) / (1.0 + zDrag);
    s = 44.5 * std::log(9.83 / omh2) / std::sqrt(1.0 + 10.0 * std::pow(obh2, 0.75));
    fNu = pch.neutrino_mass_summed / 94.0 / (h * h) / c.om;
    nEff = pch.neutrino_number_effective;
    const double fB = c.ob / c.om, fC = (c.om - c.ob) / c.om, fCB = fB + fC, fNuB = fNu + fB;
    const double pC = 0.25 * (5.0 - std::sqrt(1.0 + 24.0 * fC)), pCB = 0.25 * (5.0 - std::sqrt(1.0 + 24.0 * fCB));
    alphaNu = (fC / fCB) * ((5.0 - 2.0 * (pC + pCB)) / (5.0 - 4.0 * pCB)) *
              ((1.0 - 0.533 * fNuB + 0.126 * fNuB * fNuB * fNuB) * std::pow(1.0 + yD, pCB - pC) /
               (1.0 - 0.193 * std::sqrt(fNu * nEff) + 0.169 * fNu * std::pow(nEff, 0.2))) *
              (1.0 + 0.5 * (pC - pCB) * (1.0 + 1.0 / ((3.0 - 4.0 * pC) * (7.0 - 4.0 * pCB))) / (1.0 + yD));
    betaC = 1.0 / (1.0 - 0.949 * fNuB);
  }
  double operator()(double k) const {
    const double sa = std::sqrt(alphaNu);
    const double ks = 0.43 * k * s;
    const double gammaEff = omh2 * (sa + (1.0 - sa) / (1.0 + ks * ks * ks * ks));
    const double q = k * theta * theta / gammaEff;
    const double L = std::log(std::exp(1.0) + 1.84 * betaC * sa * q);
    const double C = 14.4 + 325.0 / (1.0 + 60.5 * std::pow(q, 1.11));
    double t = L / (L + C * q * q);
    if (fNu > 0.0 && fNu <= 0.3) {
      const double qNu = 3.92 * (k * theta * theta / omh2) * std::sqrt(nEff) / fNu;
      t *= 1.0 + 1.2 * std::pow(fNu, 0.64) * std::pow(nEff, 0.3 + 0.6 * fNu) / (std::pow(qNu, -1.6) + std::pow(qNu, 0.8));
    }
    return t;
  }
};

double transfer(double k, const Cosmo& c, const gal_pch_params& pch) {
  if (pch.transfer_function == GAL_TRANSFER_EISENSTEIN_HU_1998) return transfer_no_wiggle(k, c, pch.temperature_cmb);
  return EisensteinHu1999(c, pch)(k);
}

double window_top_hat(double x) {
  if (x < 1.0e-3) return 1.0 - x * x / 10.0;
  return 3.0 * (std::sin(x) - x * std::cos(x)) / (x * x * x);
}

// sigma(M) at z = 0 tabulated in ln M, with its logarithmic slope.
struct SigmaTable {
  double lnMin = 0.0, dlnM = 0.0;
  std::vector<double> lnSigma, slope;  // slope = dln sigma / dln M

  void build(const Cosmo& c, const gal_pch_params& pch) {
    const int nk = 8000;
    const double lnk0 = std::log(1.0e-6), lnk1 = std::log(1.0e4), dlnk = (lnk1 - lnk0) / (nk - 1);
    std::vector<double> kk(nk), pk(nk);
    const EisensteinHu1999 eh99(c, pch);
    for (int i = 0; i < nk; ++i) {
      kk[i] = std::exp(lnk0 + i * dlnk);
      const double t = pch.transfer_function == GAL_TRANSFER_EISENSTEIN_HU_1998
                           ? transfer_no_wiggle(kk[i], c, pch.temperature_cmb)
                           : eh99(kk[i]);
      pk[i] = std::pow(kk[i], pch.n_s) * t * t;
    }
    auto sigma2R = [&](double R) {
      double acc = 0.0;
      for (int i = 0; i < nk; ++i) {
        const double w = window_top_hat(kk[i] * R);
        const double f = kk[i] * kk[i] * kk[i] * pk[i] * w * w;
        acc += (i == 0 || i == nk - 1) ? 0.5 * f : f;
      }
      return acc * dlnk / (2.0 * kPi * kPi);
    };
    const double h = c.h0 / 100.0;
    const double norm = pch.sigma8 * pch.sigma8 / sigma2R(8.0 / h);
    const double rhoMean = c.om * 3.0 * c.h0 * c.h0 / (8.0 * kPi * kGravity);  // Msun/Mpc^3 (comoving, z = 0)
    const int n = 400;
    lnMin = std::log(1.0e4);
    const double lnMax = std::log(1.0e17);
    dlnM = (lnMax - lnMin) / (n - 1);
    lnSigma.resize(n);
    slope.resize(n);
    for (int i = 0; i < n; ++i) {
      const double M = std::exp(lnMin + i * dlnM);
      const double R = std::cbrt(3.0 * M / (4.0 * kPi * rhoMean));
      lnSigma[i] = 0.5 * std::log(norm * sigma2R(R));
    }
    for (int i = 0; i < n; ++i) {
      const int a = i == 0 ? 0 : i - 1, b = i == n - 1 ? n - 1 : i + 1;
      slope[i] = (lnSigma[b] - lnSigma[a]) / ((b - a) * dlnM);
    }
  }
  // ln sigma and its slope at mass M (linear interpolation; clamped).
  void at(double M, double& lns, double& sl) const {
    double x = (std::log(M) - lnMin) / dlnM;
    const int n = (int)lnSigma.size();
    if (x < 0.0) x = 0.0;
    if (x > n - 1.000001) x = n - 1.000001;
    const int i = (int)x;
    const double f = x - i;
    lns = lnSigma[i] + f * (lnSigma[i + 1] - lnSigma[i]);
    sl = slope[i] + f * (slope[i + 1] - slope[i]);
  }
  double sigma2(double M) const {
    double lns, sl;
    at(M, lns, sl);
    return std::exp(2.0 * lns);
  }
};

// w(z) = delta_c0 / D(z) tabulated in z for the inverse map.
struct GrowthTable {
  std::vector<double> z, w;
  void build(const Cosmo& c) {
    const int n = 4000;
    const double zMax = 40.0;
    auto E = [&](double a) { return std::sqrt(c.om / (a * a * a) + c.ol); };
    // D(a) = (5 om / 2) E(a) int_0^a da' / (a' E(a'))^3, by Simpson's rule in a'.
    auto growth = [&](double a) {
      const int m = 2000;  // even
      const double h = a / m;
      double acc = 0.0;
      for (int j = 0; j <= m; ++j) {
        const double x = j * h;
        double f = 0.0;
        if (x > 0.0) {
          const double ae = x * E(x);
          f = 1.0 / (ae * ae * ae);
        }
        acc += (j == 0 || j == m) ? f : (j % 2 ? 4.0 * f : 2.0 * f);
      }
      return 2.5 * c.om * E(a) * acc * h / 3.0;
    };
    const double d0 = growth(1.0);
    const double dc0 = 3.0 * std::pow(12.0 * kPi, 2.0 / 3.0) / 20.0;
    z.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
      z[i] = zMax * i / (n - 1);
      w[i] = dc0 * d0 / growth(1.0 / (1.0 + z[i]));
    }
  }
  double w_of_z(double zz) const {
    const double x = zz / z.back() * (z.size() - 1);
    const int i = std::min((int)x, (int)z.size() - 2);
    const double f = x - i;
    return w[i] + f * (w[i + 1] - w[i]);
  }
  double z_of_w(double ww) const {
    if (ww <= w.front()) return 0.0;
    const auto it = std::upper_bound(w.begin(), w.end(), ww);
    const int i = std::min((int)(it - w.begin()) - 1, (int)w.size() - 2);
    const double f = (ww - w[i]) / (w[i + 1] - w[i]);
    return z[i] + f * (z[i + 1] - z[i]);
  }
};

// Branching rates of the PCH algorithm for a branch of mass M2 at w.  The
// modifier G = G0 (sigma1/sigma2)^gamma1 (w/sigma2)^gamma2 factors into a
// part that depends on M2 alone and (w/sigma2)^gamma2, so the split rate R,
// the sub-resolution accretion rate F and the distribution of the split's
// mass ratio q are integrated once per mass on a grid in ln M2 (RateTable)
// and scaled by (w/sigma2)^gamma2 along each branch.
struct Rates {
  const SigmaTable& sig;
  gal_pch_params pch;
  double mRes;
  static constexpr int kNq = gal::trees::kNq;  // trapezoid points in ln q (1e-5 of the analytic rate)

  // G without its w factor: G0 (sigma1/sigma2)^gamma1.
  double modifier_mass(double s1, double s2) const { return pch.g0 * std::pow(s1 / s2, pch.gamma1); }

  // R / (w/sigma2)^gamma2 with its cumulative distribution over ln q on kNq
  // points from ln(mRes/M2) to ln 1/2:
  //   R = int q dN/dq dln q,  q dN/dq = (1/sqrt(2 pi)) |dS1/dln M1| q^-1 (S1 - S2)^-3/2 G.
  double split_rate(double M2, double* lnq, double* cdf) const {
    const double qRes = mRes / M2;
    if (qRes >= 0.5) {
      for (int i = 0; i < kNq; ++i) {
        lnq[i] = std::log(0.5);
        cdf[i] = 0.0;
      }
      return 0.0;
    }
    double lns2, sl2;
    sig.at(M2, lns2, sl2);
    const double S2 = std::exp(2.0 * lns2), s2 = std::sqrt(S2);
    const double a = std::log(qRes), b = std::log(0.5), d = (b - a) / (kNq - 1);
    double prev = 0.0;
    for (int i = 0; i < kNq; ++i) {
      lnq[i] = a + i * d;
      const double q = std::exp(lnq[i]);
      double lns1, sl1;
      sig.at(q * M2, lns1, sl1);
      const double S1 = std::exp(2.0 * lns1);
      const double dS1 = 2.0 * S1 * std::fabs(sl1);  // |dS1/dln M1|
      const double diff = S1 - S2;
      const double f = diff > 0.0 ? dS1 / q * std::pow(diff, -1.5) * modifier_mass(std::sqrt(S1), s2) / std::sqrt(2.0 * kPi) : 0.0;
      cdf[i] = i == 0 ? 0.0 : cdf[i - 1] + 0.5 * (prev + f) * d;
      prev = f;
    }
    return cdf[kNq - 1];
  }

  // F / (w/sigma2)^gamma2:
  //   F = (1/sqrt(2 pi)) int_{S_res}^inf (S1 - S2)^-3/2 G dS1 = (2/sqrt(2 pi)) int_0^{u_res} G du,
  // u = (S1 - S2)^-1/2, by the midpoint rule in v with u = u_res v^(1/(1-gamma1)),
  // which is exact for gamma1 = 0.
  double accretion_rate(double M2) const {
    const double S2 = sig.sigma2(M2), s2 = std::sqrt(S2);
    const double Sres = sig.sigma2(mRes);
    if (!(Sres > S2)) return 0.0;
    const double uRes = 1.0 / std::sqrt(Sres - S2);
    const double g1 = pch.gamma1, p = 1.0 / (1.0 - g1);
    const int nv = 32;
    double acc = 0.0;
    for (int j = 0; j < nv; ++j) {
      const double v = (j + 0.5) / nv;
      const double u = uRes * std::pow(v, p);
      const double dudv = uRes * p * std::pow(v, p - 1.0);
      const double s1 = std::sqrt(S2 + 1.0 / (u * u));
      acc += modifier_mass(s1, s2) * dudv;
    }
    return 2.0 / std::sqrt(2.0 * kPi) * acc / nv;
  }

  // (w/sigma2)^gamma2, the w-dependent factor of G.
  double modifier_w(double w, double s2) const { return std::pow(w / s2, pch.gamma2); }
};

// Rates on a grid in ln M2 (kPerDecade rows per decade from the resolution
// up): R and F interpolated linearly in ln M2, q drawn from the nearest row.
struct RateTable {
  static constexpr int kPerDecade = 256;
  double lnMin = 0.0, dlnM = 1.0, lnMRes = 0.0;
  int rows = 0;
  std::vector<double> R, F, lnq, cdf;  // R, F [rows]; lnq, cdf [rows][kNq] (cdf normalised to 1)

  void build(const Rates& r, double massMax) {
    lnMRes = std::log(r.mRes);
    lnMin = lnMRes;
    dlnM = std::log(10.0) / kPerDecade;
    rows = std::max(2, (int)std::ceil((std::log(massMax) - lnMin) / dlnM) + 2);
    R.resize(rows);
    F.resize(rows);
    lnq.resize((size_t)rows * Rates::kNq);
    cdf.resize((size_t)rows * Rates::kNq);
    for (int j = 0; j < rows; ++j) {
      const double M = std::exp(lnMin + j * dlnM);
      double* q = &lnq[(size_t)j * Rates::kNq];
      double* c = &cdf[(size_t)j * Rates::kNq];
      R[j] = r.split_rate(M, q, c);
      F[j] = r.accretion_rate(M);
      if (R[j] > 0.0)
        for (int i = 0; i < Rates::kNq; ++i) c[i] /= R[j];
    }
  }
  // Row coordinate of mass M (clamped to the grid).
  double coord(double M) const {
    double x = (std::log(M) - lnMin) / dlnM;
    return std::min(std::max(x, 0.0), rows - 1.000001);
  }
};

struct Builder {
  const SigmaTable& sig;
  gal_pch_params pch;
  double mRes, wMax;
  const RateTable& rt;
  using Node = GrownNode;

  // Grow one tree from its root.
  void grow(double rootMass, double rootW, std::mt19937_64& rng, std::vector<Node>& nodes) const {
    nodes.clear();
    nodes.push_back(Node{rootMass, rootW, -1, 0, 0});
    std::vector<int32_t> stack{0};
    std::uniform_real_distribution<double> U(0.0, 1.0);
    constexpr int nq = Rates::kNq;
    while (!stack.empty()) {
      const int32_t i = stack.back();
      stack.pop_back();
      double m = nodes[i].mass, w = nodes[i].w;
      double mPrev = m, wPrev = w;
      bool split = false;
      int guard = 0;
      while (w < wMax && m >= mRes && ++guard < 100000) {
        const double x = rt.coord(m);
        const int j = (int)x;
        const double fx = x - j;
        double lns2, sl2;
        sig.at(m, lns2, sl2);
        const double S2 = std::exp(2.0 * lns2), Sh = sig.sigma2(0.5 * m);
        const double wf = std::pow(w / std::sqrt(S2), pch.gamma2);
        const double R = m <= 2.0 * mRes ? 0.0 : wf * (rt.R[j] + fx * (rt.R[j + 1] - rt.R[j]));
        const double F = wf * (rt.F[j] + fx * (rt.F[j + 1] - rt.F[j]));
        double dw = pch.accuracy_second * std::sqrt(2.0 * std::max(Sh - S2, 0.0));
        if (R > 0.0) dw = std::min(dw, pch.accuracy_first / R);
        if (F > 0.0) dw = std::min(dw, pch.accuracy_first / F);
        if (!(dw > 0.0)) dw = 1.0e-3;
        bool last = false;
        if (w + dw >= wMax) {
          dw = wMax - w;
          last = true;
        }
        const double wNext = last ? wMax : w + dw;
        mPrev = m;
        wPrev = w;
        if (R > 0.0 && U(rng) < R * dw) {
          // Split: q from the tabulated distribution in ln q of the nearest
          // row with a resolved split (its q range is that row's).
          int row = fx < 0.5 ? j : j + 1;
          if (!(rt.R[row] > 0.0)) row = j + 1;
          const double* cdf = &rt.cdf[(size_t)row * nq];
          const double* lnq = &rt.lnq[(size_t)row * nq];
          const double target = U(rng);
          const int k = (int)(std::upper_bound(cdf, cdf + nq, target) - cdf);
          const int k1 = std::min(std::max(k, 1), nq - 1);
          const double f = (target - cdf[k1 - 1]) / std::max(cdf[k1] - cdf[k1 - 1], 1e-300);
          const double q = std::exp(lnq[k1 - 1] + f * (lnq[k1] - lnq[k1 - 1]));
          const double m1 = q * m;
          const double m2 = m * (1.0 - F * dw) - m1;
          const double wNew = wNext;
          const double big = std::max(m1, m2), small = std::min(m1, m2);
          const int32_t first = (int32_t)nodes.size();
          int32_t count = 0;
          if (big >= mRes) {
            nodes.push_back(Node{big, wNew, i, 0, 0});
            ++count;
          }
          if (small >= mRes) {
            nodes.push_back(Node{small, wNew, i, 0, 0});
            ++count;
          }
          nodes[i].childFirst = first;
          nodes[i].childCount = count;
          for (int32_t c = count - 1; c >= 0; --c) stack.push_back(first + c);
          split = true;
          break;
        }
        m *= 1.0 - F * dw;
        w = wNext;
        if (last) break;
      }
      if (!split) {
        // The branch ends: its earliest resolved halo is a leaf progenitor.
        double lm = m, lw = w;
        if (m < mRes) {
          lm = mPrev;
          lw = wPrev;
        }
        if (lw > nodes[i].w && lm >= mRes) {
          nodes[i].childFirst = (int32_t)nodes.size();
          nodes[i].childCount = 1;
          nodes.push_back(Node{lm, lw, i, 0, 0});
        }
      }
    }
  }
};

bool valid_transfer(const gal_pch_params& pch) {
  return (pch.transfer_function == GAL_TRANSFER_EISENSTEIN_HU_1999 ||
          pch.transfer_function == GAL_TRANSFER_EISENSTEIN_HU_1998) &&
         pch.neutrino_number_effective >= 0.0 && pch.neutrino_mass_summed >= 0.0;
}

uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Virial radius (Mpc) and velocity (km/s) of a halo of mass M at redshift z
// in the flat matter + Lambda cosmology, with the Bryan & Norman (1998)
// contrast relative to the mean density (the forest's segment constants use
// the same relation).
void virial(const Cosmo& c, double M, double z, double& r, double& v) {
  const double zp = (1.0 + z) * (1.0 + z) * (1.0 + z);
  const double omz = c.om * zp / (c.om * zp + c.ol);
  const double x = omz - 1.0;
  const double contrast = (18.0 * kPi * kPi + 82.0 * x - 39.0 * x * x) / (x + 1.0);
  const double rhoMean = c.om * 3.0 * c.h0 * c.h0 / (8.0 * kPi * kGravity) * zp;
  r = std::cbrt(3.0 * M / (4.0 * kPi * contrast * rhoMean));
  v = std::sqrt(kGravity * M / r);
}

// Jiang et al. (2008) merging time of a satellite on an orbit with radial
// and tangential velocities (ur, ut) at the host's virial radius, in units
// of the host's virial velocity (satelliteMergingTimescalesJiang2008%
// timeUntilMerging, satellites/merging/timescale/Jiang2008.F90): with the
// orbit's energy E = -1 + (ur^2 + ut^2) mu/2 (units of V_vir^2, mu =
// M_host/(M_host + M_sat) the specific reduced mass, as the reference's
// virial-orbit sampler forms it), the circular orbit of the same energy in
// a singular isothermal host truncated at r_vir (point mass beyond it) has
// radius r_c = r_vir exp(E + 1/2) (E <= -1/2) or r_vir/(-2E), and the
// orbit's circularity is its angular momentum r_vir ut V_vir over
// r_c V_c(r_c).  Negative for an unbound orbit.
double jiang2008_time(double tdyn, double q, double mu, double ur, double ut, double multiplier) {
  const double E = -1.0 + 0.5 * mu * (ur * ur + ut * ut);
  if (!(E < 0.0)) return -1.0;
  double rc, eps;
  if (E <= -0.5) {
    rc = std::exp(E + 0.5);
    eps = ut / rc;
  } else {
    rc = -0.5 / E;
    eps = ut * std::sqrt(1.0 / rc);
  }
  constexpr double C = 0.43, a = 0.94, b = 0.60, d = 0.60;  // Jiang et al. (2008), eq. 5
  if (!(q > 0.0)) return 0.0;
  return multiplier * tdyn * std::sqrt(rc) * ((a * std::pow(eps, b) + d) / (2.0 * C)) * q / std::log1p(q);
}

// An orbit from the Benson (2005, MNRAS 358, 551) distribution of radial and
// tangential velocities of infalling satellites at the host's virial radius
// (units of its virial velocity), by rejection as virialOrbitBenson2005%orbit
// does (satellites/merging/virial_orbits/Benson2005.F90): velocities uniform
// on [0, 3], accepted with probability f(ur, ut)/f_max, bound orbits only
// (E < -1e-4).  The fit's coefficients are the paper's.
void benson2005_orbit(std::mt19937_64& rng, double mu, double& ur, double& ut) {
  constexpr double pMax = 1.96797, velocityMax = 3.0;
  constexpr double a[9] = {3.90052, 2.47973, 10.2373, 0.683922, 0.353953, 1.07716, 0.509837, 0.206204, 0.314641};
  std::uniform_real_distribution<double> U(0.0, 1.0);
  for (int attempt = 0; attempt < 1000000; ++attempt) {
    ur = U(rng) * velocityMax;
    ut = U(rng) * velocityMax;
    const double y = pMax * U(rng);
    // Unbound orbits and points above g >= f (the factor exp(-b1 (ur -
    // b2)^2) <= 1 and rounding is monotone) are rejected before the rest of
    // f is evaluated: the same decisions as the full test, on the same draws.
    if (!(-1.0 + 0.5 * mu * (ur * ur + ut * ut) < -1.0e-4)) continue;
    const double g = a[0] * ut * std::exp(-a[1] * (ut - a[8]) * (ut - a[8]));
    if (!(y <= g)) continue;
    const double b1 = a[2] * std::exp(-a[3] * (ut - a[4]) * (ut - a[4]));
    const double b2 = a[5] * std::exp(-a[6] * (ut - a[7]) * (ut - a[7]));
    const double f = g * std::exp(-b1 * (ur - b2) * (ur - b2));
    if (y <= f) return;
  }
  ur = 0.0;  // not reached for the fit's distribution: a circular orbit
  ut = 1.0;
}

// One tree as built (children contiguous, primary first), with node times.
struct TreeIn {
  const std::vector<Builder::Node>* nodes;
  std::vector<double> time;
};

// A node of a tree with satellites before it is laid out.  Its
// progenitors form a list (primary first) linked through `next`, with its
// first and last entries and its length.
struct SatNode {
  double mass, time, spin;
  int32_t parent, satHost;  // satHost: the host at infall of a satellite phase, else -1
  int32_t first = -1, last = -1, next = -1, count = 0;
};

SatNode sat_node(double mass, double time, double spin, int32_t parent, int32_t satHost) {
  SatNode nd;
  nd.mass = mass;
  nd.time = time;
  nd.spin = spin;
  nd.parent = parent;
  nd.satHost = satHost;
  return nd;
}

// Append node c to the progenitors of node p.
void append_child(std::vector<SatNode>& out, int32_t p, int32_t c) {
  out[(size_t)c].next = -1;
  if (out[(size_t)p].last < 0)
    out[(size_t)p].first = c;
  else
    out[(size_t)out[(size_t)p].last].next = c;
  out[(size_t)p].last = c;
  ++out[(size_t)p].count;
}

// Satellites as the reference's tree evolver has them (merger_trees/
// evolver/standard.F90: a secondary progenitor becomes a satellite at its
// parent's time and merges when its merging time runs out): each secondary
// progenitor s of a node p gets a node S, its satellite phase (time t_p,
// its halo's mass, s as its only progenitor), and a merging time t_m = t_p
// + tau on a Benson (2005) orbit in the primary progenitor (its host at
// infall, satelliteMergingTimescalesJiang2008 with node%parent%firstChild as
// the host and q = M_host/M_sat).  The host at t_m is the node alive then
// on p's line of descendants (the halo that holds the satellite, through
// its own infall into a larger halo, as the reference moves satellites of
// satellites to the new host); that node is cut at t_m into the piece
// before and a piece from t_m on whose progenitors are the piece before
// (primary) and the satellites merging at t_m.  A satellite that outlives
// the tree ends in a root of its own at the tree's final time.  The host's
// mass line is kept: the piece from t_m starts at the mass its halo has
// reached by then.
void add_satellites(const TreeIn& in, const std::vector<double>& spin, const Cosmo& c, double multiplier,
                    std::mt19937_64& rng, std::vector<SatNode>& out) {
  const std::vector<Builder::Node>& tr = *in.nodes;
  const int32_t n = (int32_t)tr.size();
  const std::vector<double>& t = in.time;
  out.clear();
  out.reserve((size_t)n * 2);
  for (int32_t i = 0; i < n; ++i) out.push_back(sat_node(tr[i].mass, t[i], spin[i], tr[i].parent, -1));
  for (int32_t i = 0; i < n; ++i)
    for (int32_t k = 0; k < tr[i].childCount; ++k) append_child(out, i, tr[i].childFirst + k);
  // The halo mass a node reaches by time x (its mass line: a primary
  // progenitor grows by its parent's unresolved mass, others stay).
  auto massAt = [&](int32_t i, double x) {
    const int32_t p = tr[i].parent;
    if (p < 0 || tr[p].childFirst != i || !(t[p] > t[i])) return tr[i].mass;
    double brought = 0.0;
    for (int32_t k = 0; k < tr[p].childCount; ++k) brought += tr[tr[p].childFirst + k].mass;
    const double unresolved = std::max(tr[p].mass - brought, 0.0);
    return tr[i].mass + unresolved * (x - t[i]) / (t[p] - t[i]);
  };
  int32_t root = 0;
  while (tr[root].parent >= 0) root = tr[root].parent;
  const double tEnd = t[root];
  struct Event { double tm; int32_t sat; };
  std::vector<std::vector<Event>> events((size_t)n);  // merging events on each original node
  std::vector<int32_t> unmerged;
  // Ancestor jumps for large trees: up[k][i] is the 2^k-th ancestor of i
  // (-1 above the root); parents precede their progenitors in tr.
  int levels = 0;
  std::vector<int32_t> up;
  if (n > 512) {
    int32_t depth = 0;
    std::vector<int32_t> dep((size_t)n, 0);
    for (int32_t i = 0; i < n; ++i)
      if (tr[i].parent >= 0) depth = std::max(depth, dep[(size_t)i] = dep[(size_t)tr[i].parent] + 1);
    while ((1 << levels) <= depth) ++levels;
    up.assign((size_t)levels * n, -1);
    for (int32_t i = 0; i < n; ++i) {
      up[(size_t)i] = tr[i].parent;
      for (int k = 1; k < levels; ++k) {
        const int32_t a = up[(size_t)(k - 1) * n + i];
        up[(size_t)k * n + i] = a < 0 ? -1 : up[(size_t)(k - 1) * n + a];
      }
    }
  }
  for (int32_t p = 0; p < n; ++p) {
    if (tr[p].childCount < 2) continue;
    const int32_t c0 = tr[p].childFirst;
    double massSat = 0.0;
    for (int32_t k = 1; k < tr[p].childCount; ++k) massSat += tr[c0 + k].mass;
    // The host at infall: the primary progenitor at t_p.
    const double massHost = std::max(tr[p].mass - massSat, tr[c0].mass);
    double rv, vv;
    virial(c, massHost, std::max(c.redshift(t[p]), 0.0), rv, vv);
    const double tdyn = rv / vv * kMpcPerKmPerSToGyr;
    std::vector<int32_t> kept{c0};  // p's progenitors: the primary, and satellites that merge at once
    for (int32_t k = 1; k < tr[p].childCount; ++k) {
      const int32_t s = c0 + k;
      const double ms = tr[s].mass, mu = massHost / (massHost + ms);
      double ur, ut;
      benson2005_orbit(rng, mu, ur, ut);
      double tau = jiang2008_time(tdyn, massHost / ms, mu, ur, ut, multiplier);
      const double tm = tau < 0.0 ? HUGE_VAL : t[p] + tau;
      if (!(tm > t[p])) {
        kept.push_back(s);
        continue;
      }
      // The satellite phase S replaces s among p's progenitors.
      const int32_t S = (int32_t)out.size();
      out.push_back(sat_node(ms, t[p], spin[s], -1, p));
      append_child(out, S, s);
      out[s].parent = S;
      // The node alive at t_m on p's line of descendants: the highest
      // ancestor-or-self of p whose time is not after t_m (times grow
      // towards the root, so jumps of 2^k ancestors find it).
      int32_t d = p;
      if (up.empty()) {
        while (tr[d].parent >= 0 && !(tm < t[tr[d].parent])) d = tr[d].parent;
      } else {
        for (int k = levels - 1; k >= 0; --k) {
          const int32_t a = up[(size_t)k * n + d];
          if (a >= 0 && !(tm < t[a])) d = a;
        }
      }
      if (tr[d].parent < 0 && !(tm < tEnd)) unmerged.push_back(S);
      else events[d].push_back(Event{tm, S});
    }
    // The satellites' phases hang from their merging pieces.
    out[p].first = out[p].last = -1;
    out[p].count = 0;
    for (int32_t k : kept) append_child(out, p, k);
  }
  // Cut each host node at its merging times.
  for (int32_t d = 0; d < n; ++d) {
    std::vector<Event>& ev = events[d];
    if (ev.empty()) continue;
    std::stable_sort(ev.begin(), ev.end(), [](const Event& a, const Event& b) { return a.tm < b.tm; });
    const int32_t par = out[d].parent;
    const int32_t dNext = out[d].next;  // d's place among its parent's progenitors
    int32_t prev = d;
    size_t j = 0;
    // Mergers at the node's own time join its progenitors directly.
    while (j < ev.size() && !(ev[j].tm > t[d])) {
      out[ev[j].sat].parent = d;
      append_child(out, d, ev[j].sat);
      ++j;
    }
    if (j == ev.size()) continue;
    while (j < ev.size()) {
      const double tm = ev[j].tm;
      const int32_t J = (int32_t)out.size();
      out.push_back(sat_node(massAt(d, tm), tm, spin[d], -1, -1));
      append_child(out, J, prev);
      out[prev].parent = J;
      for (; j < ev.size() && ev[j].tm == tm; ++j) {
        out[ev[j].sat].parent = J;
        append_child(out, J, ev[j].sat);
      }
      prev = J;
    }
    // The last piece takes the node's place among its parent's progenitors.
    out[prev].parent = par;
    if (par >= 0) {
      out[prev].next = dNext;
      if (out[par].first == d) {
        out[par].first = prev;
      } else {
        int32_t q = out[par].first;
        while (out[q].next != d) q = out[q].next;
        out[q].next = prev;
      }
      if (out[par].last == d) out[par].last = prev;
    }
  }
  // Satellites that outlive the tree: a root of their own at its final time.
  for (int32_t S : unmerged) {
    if (!(tEnd > out[S].time)) continue;  // fell in at the final time: S is the root
    const int32_t E = (int32_t)out.size();
    out.push_back(sat_node(out[S].mass, tEnd, out[S].spin, -1, -1));
    append_child(out, E, S);
    out[S].parent = E;
  }
}

// Lay a tree with satellites out as the forest layout wants it: roots
// first (the tree's own root, then the roots of satellites that outlive
// it), then breadth first, so that each node's progenitors are contiguous
// with the primary first.  Returns the order of the nodes.
std::vector<int32_t> layout(const std::vector<SatNode>& nodes) {
  std::vector<int32_t> order;
  order.reserve(nodes.size());
  for (int32_t i = 0; i < (int32_t)nodes.size(); ++i)
    if (nodes[i].parent < 0) order.push_back(i);
  for (size_t q = 0; q < order.size(); ++q)
    for (int32_t ch = nodes[(size_t)order[q]].first; ch >= 0; ch = nodes[(size_t)ch].next) order.push_back(ch);
  return order;
}

}  // namespace

struct gal_forest {
  std::vector<int32_t> tree, parent, childFirst, childCount, satHost;
  std::vector<double> time, mass, spin;
  double stats[7] = {0, 0, 0, 0, 0, 0, 0};  // gal_forest_build_stats
};

namespace {

// The builder's tables as the device branching reads them.
gal::trees::BranchTables branch_tables(const SigmaTable& sig, const RateTable& rt, const Builder& B,
                                       const gal_pch_params& pch) {
  return gal::trees::BranchTables{sig.lnMin, sig.dlnM, (int32_t)sig.lnSigma.size(), sig.lnSigma.data(), rt.lnMin,
                                  rt.dlnM, rt.rows, rt.R.data(), rt.F.data(), rt.lnq.data(), rt.cdf.data(),
                                  B.mRes, B.wMax, pch.gamma2, pch.accuracy_first, pch.accuracy_second};
}

bool valid_spec(const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec) {
  return p && pch && spec && valid_transfer(*pch) && spec->n_trees >= 0 && spec->mass_resolution > 0.0 &&
         spec->root_mass_min >= spec->mass_resolution && spec->root_mass_max >= spec->root_mass_min &&
         spec->redshift_max > spec->root_redshift && spec->root_redshift >= 0.0 && spec->redshift_max <= 30.0 &&
         (spec->satellites == GAL_SATELLITES_NONE ||
          (spec->satellites == GAL_SATELLITES_JIANG2008 && spec->satellite_timescale_multiplier >= 0.0));
}

// The forest of spec: branches grown on the host (ctx == nullptr: one
// sequential stream per tree) or on the GPU of ctx (keyed streams).
int build_forest(gal_ctx* ctx, const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec,
                 gal_forest** out) {
  const auto tStart = std::chrono::steady_clock::now();
  auto since = [](std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  };
  double stats[7] = {0, 0, 0, 0, 0, 0, 0};
  if (!out) return GAL_ERR_ARGUMENT;
  *out = nullptr;
  if (!valid_spec(p, pch, spec)) return GAL_ERR_ARGUMENT;
  const Cosmo c = cosmo_of(p);
  SigmaTable sig;
  sig.build(c, *pch);
  GrowthTable gt;
  gt.build(c);
  RateTable rt;
  rt.build(Rates{sig, *pch, spec->mass_resolution}, spec->root_mass_max);
  const Builder B{sig, *pch, spec->mass_resolution, gt.w_of_z(spec->redshift_max), rt};
  stats[0] = since(tStart);
  const int64_t nTrees = spec->n_trees;
  const bool satellites = spec->satellites == GAL_SATELLITES_JIANG2008;
  std::vector<std::vector<Builder::Node>> trees((size_t)nTrees);
  std::vector<std::vector<double>> spins((size_t)nTrees);
  std::vector<std::vector<SatNode>> satTrees((size_t)(satellites ? nTrees : 0));
  const double s = spec->root_mass_slope;
  const double a = std::pow(spec->root_mass_min, s), b = std::pow(spec->root_mass_max, s);
  const double wRoot = gt.w_of_z(spec->root_redshift);
  const double tMaxTree = c.time(spec->redshift_max);
  // dN/dln M ~ M^s on [min, max]: the root mass of a tree is the inverse of
  // the cumulative M^s at the first draw of the tree's stream.
  auto root_mass = [&](std::mt19937_64& rng) {
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const double u = U(rng);
    return std::fabs(s) < 1e-12 ? spec->root_mass_min * std::pow(spec->root_mass_max / spec->root_mass_min, u)
                                : std::pow(a + u * (b - a), 1.0 / s);
  };
  auto tree_stream = [&](int64_t t) { return std::mt19937_64(splitmix64(spec->seed ^ splitmix64((uint64_t)t))); };
  if (ctx) {
    std::vector<double> roots((size_t)nTrees);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < nTrees; ++t) {
      std::mt19937_64 rng = tree_stream(t);
      roots[(size_t)t] = root_mass(rng);
    }
    const gal::trees::BranchTables tab = branch_tables(sig, rt, B, *pch);
    double g[3] = {0, 0, 0};
    const int rc = gal::trees::grow_forest_gpu(ctx, tab, roots.data(), nTrees, wRoot, spec->seed, trees, g);
    if (rc != GAL_OK) return rc;
    stats[1] = g[0];
    stats[2] = g[1];
    stats[5] = g[2];
  }
  const auto tLoop = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t t = 0; t < nTrees; ++t) {
    std::mt19937_64 rng = tree_stream(t);
    const double M = root_mass(rng);
    if (!ctx) B.grow(M, wRoot, rng, trees[(size_t)t]);
    // Spins: log-normal about the peak of the Bett et al. (2007) distribution.
    std::normal_distribution<double> N(0.0, 0.5);
    spins[(size_t)t].resize(trees[(size_t)t].size());
    for (double& x : spins[(size_t)t]) x = 0.04326 * std::exp(N(rng));
    if (satellites) {
      // Orbits drawn from the tree's stream after its spins.
      TreeIn in{&trees[(size_t)t], std::vector<double>(trees[(size_t)t].size())};
      for (size_t j = 0; j < in.time.size(); ++j) {
        const double w = trees[(size_t)t][j].w;
        in.time[j] = w >= B.wMax ? tMaxTree : c.time(gt.z_of_w(w));
      }
      add_satellites(in, spins[(size_t)t], c, spec->satellite_timescale_multiplier, rng, satTrees[(size_t)t]);
    }
  }
  stats[3] = since(tLoop);
  // Assembly, parallel over trees: each tree's nodes from its offset.
  const auto tAsm = std::chrono::steady_clock::now();
  gal_forest* f = new (std::nothrow) gal_forest();
  if (!f) return GAL_ERR_ARGUMENT;
  std::vector<size_t> first((size_t)nTrees + 1, 0);
  for (int64_t t = 0; t < nTrees; ++t)
    first[(size_t)t + 1] = first[(size_t)t] + (satellites ? satTrees[(size_t)t].size() : trees[(size_t)t].size());
  const size_t total = first[(size_t)nTrees];
  f->tree.resize(total);
  f->parent.resize(total);
  f->childFirst.resize(total);
  f->childCount.resize(total);
  f->time.resize(total);
  f->mass.resize(total);
  f->spin.resize(total);
  f->satHost.assign(total, -1);
  const double tMax = tMaxTree;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t t = 0; t < nTrees; ++t) {
    const size_t off = first[(size_t)t];
    if (satellites) {
      const std::vector<SatNode>& tr = satTrees[(size_t)t];
      const std::vector<int32_t> order = layout(tr);
      std::vector<int32_t> at(tr.size());
      for (size_t j = 0; j < order.size(); ++j) at[(size_t)order[j]] = (int32_t)j;
      for (size_t j = 0; j < order.size(); ++j) {
        const SatNode& nd = tr[(size_t)order[j]];
        const size_t g = off + j;
        f->tree[g] = (int32_t)t;
        f->parent[g] = nd.parent < 0 ? -1 : (int32_t)(off + at[(size_t)nd.parent]);
        f->childCount[g] = nd.count;
        f->childFirst[g] = nd.count == 0 ? 0 : (int32_t)(off + at[(size_t)nd.first]);
        f->time[g] = nd.time;
        f->mass[g] = nd.mass;
        f->spin[g] = nd.spin;
        f->satHost[g] = nd.satHost < 0 ? -1 : (int32_t)(off + at[(size_t)nd.satHost]);
      }
    } else {
      const auto& tr = trees[(size_t)t];
      for (size_t j = 0; j < tr.size(); ++j) {
        const size_t g = off + j;
        f->tree[g] = (int32_t)t;
        f->parent[g] = tr[j].parent < 0 ? -1 : (int32_t)(off + tr[j].parent);
        f->childFirst[g] = tr[j].childCount ? (int32_t)(off + tr[j].childFirst) : 0;
        f->childCount[g] = tr[j].childCount;
        // Nodes on the maximum-redshift boundary get exactly that time.
        f->time[g] = tr[j].w >= B.wMax ? tMax : c.time(gt.z_of_w(tr[j].w));
        f->mass[g] = tr[j].mass;
        f->spin[g] = spins[(size_t)t][j];
      }
    }
  }
  stats[4] = since(tAsm);
  stats[6] = since(tStart);
  std::memcpy(f->stats, stats, sizeof stats);
  *out = f;
  return GAL_OK;
}

}  // namespace

extern "C" {

void gal_pch_params_default(gal_pch_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->g0 = 0.57;
  p->gamma1 = 0.38;
  p->gamma2 = -0.01;
  p->accuracy_first = 0.1;
  p->accuracy_second = 0.1;
  p->sigma8 = 0.8;
  p->n_s = 0.96;
  p->temperature_cmb = 2.72548;
  p->transfer_function = GAL_TRANSFER_EISENSTEIN_HU_1999;
  p->neutrino_number_effective = 3.046;
  p->neutrino_mass_summed = 0.0;
}

double gal_cosmic_time(const gal_params* p, double z) { return p ? cosmo_of(p).time(z) : NAN; }
double gal_redshift(const gal_params* p, double t) { return p ? cosmo_of(p).redshift(t) : NAN; }

double gal_pch_transfer(const gal_params* p, const gal_pch_params* pch, double k) {
  if (!p || !pch || !(k > 0.0) || !valid_transfer(*pch)) return NAN;
  return transfer(k, cosmo_of(p), *pch);
}

double gal_pch_sigma(const gal_params* p, const gal_pch_params* pch, double mass) {
  if (!p || !pch || !(mass > 0.0) || !valid_transfer(*pch)) return NAN;
  SigmaTable s;
  s.build(cosmo_of(p), *pch);
  return std::sqrt(s.sigma2(mass));
}

int gal_pch_branching_rates(const gal_pch_params* pch, double alpha, double sigma_parent, double mass_parent,
                            double mass_resolution, double w, double* rate, double* accretion) {
  if (!pch || !rate || !accretion || !(sigma_parent > 0.0) || !(mass_parent > 0.0) || !(mass_resolution > 0.0) ||
      !(mass_resolution < mass_parent) || !(w > 0.0))
    return GAL_ERR_ARGUMENT;
  // sigma(M) = sigma_parent (M / mass_parent)^alpha on the builder's grid:
  // linear interpolation of ln sigma in ln M is exact for a power law.
  SigmaTable sig;
  const int n = 400;
  sig.lnMin = std::log(mass_resolution) - 8.0;
  sig.dlnM = (std::log(mass_parent) + 8.0 - sig.lnMin) / (n - 1);
  sig.lnSigma.resize(n);
  sig.slope.assign(n, alpha);
  for (int i = 0; i < n; ++i) sig.lnSigma[i] = std::log(sigma_parent) + alpha * (sig.lnMin + i * sig.dlnM - std::log(mass_parent));
  const Rates r{sig, *pch, mass_resolution};
  std::vector<double> lnq(Rates::kNq), cdf(Rates::kNq);
  const double wf = r.modifier_w(w, sigma_parent);
  *rate = wf * r.split_rate(mass_parent, lnq.data(), cdf.data());
  *accretion = wf * r.accretion_rate(mass_parent);
  return GAL_OK;
}

int gal_forest_build(const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec, gal_forest** out) {
  return build_forest(nullptr, p, pch, spec, out);
}

int gal_gpu_forest_build(gal_ctx* ctx, const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec,
                         gal_forest** out) {
  if (!ctx || !out || !valid_spec(p, pch, spec)) {
    if (out) *out = nullptr;
    return ctx ? gal::trees::record_error(ctx, GAL_ERR_ARGUMENT, "gal_gpu_forest_build: bad arguments")
               : GAL_ERR_ARGUMENT;
  }
  return build_forest(ctx, p, pch, spec, out);
}

int gal_pch_branch_tables(const gal_params* p, const gal_pch_params* pch, const gal_forest_spec* spec, int32_t* sizes,
                          double* meta, double* ln_sigma, double* rate, double* accretion, double* ln_q, double* cdf) {
  if (!p || !pch || !spec || !sizes || !meta || !valid_transfer(*pch) || !(spec->mass_resolution > 0.0) ||
      !(spec->root_mass_max >= spec->mass_resolution) || !(spec->redshift_max > spec->root_redshift) ||
      spec->root_redshift < 0.0 || spec->redshift_max > 30.0)
    return GAL_ERR_ARGUMENT;
  const Cosmo c = cosmo_of(p);
  SigmaTable sig;
  sig.build(c, *pch);
  GrowthTable gt;
  gt.build(c);
  RateTable rt;
  rt.build(Rates{sig, *pch, spec->mass_resolution}, spec->root_mass_max);
  const Builder B{sig, *pch, spec->mass_resolution, gt.w_of_z(spec->redshift_max), rt};
  const gal::trees::BranchTables t = branch_tables(sig, rt, B, *pch);
  sizes[0] = t.nSigma;
  sizes[1] = t.rows;
  const double m[10] = {t.sigLnMin, t.sigDlnM, t.rtLnMin, t.rtDlnM, t.mRes, t.wMax, t.gamma2, t.accuracyFirst,
                        t.accuracySecond, gt.w_of_z(spec->root_redshift)};
  std::memcpy(meta, m, sizeof m);
  auto put = [](double* dst, const double* src, size_t n) {
    if (dst) std::memcpy(dst, src, n * sizeof(double));
  };
  put(ln_sigma, t.lnSigma, (size_t)t.nSigma);
  put(rate, t.R, (size_t)t.rows);
  put(accretion, t.F, (size_t)t.rows);
  put(ln_q, t.lnq, (size_t)t.rows * gal::trees::kNq);
  put(cdf, t.cdf, (size_t)t.rows * gal::trees::kNq);
  return GAL_OK;
}

int gal_forest_build_stats(const gal_forest* f, double* stats) {
  if (!f || !stats) return GAL_ERR_ARGUMENT;
  std::memcpy(stats, f->stats, sizeof f->stats);
  return GAL_OK;
}

int64_t gal_forest_node_count(const gal_forest* f) { return f ? (int64_t)f->tree.size() : -1; }

int gal_forest_get(const gal_forest* f, int32_t* tree, int32_t* parent, int32_t* childFirst, int32_t* childCount,
                   double* time, double* mass, double* spin) {
  if (!f) return GAL_ERR_ARGUMENT;
  const size_t n = f->tree.size();
  auto put = [n](auto* dst, const auto& src) {
    if (dst) std::memcpy(dst, src.data(), n * sizeof(src[0]));
  };
  put(tree, f->tree);
  put(parent, f->parent);
  put(childFirst, f->childFirst);
  put(childCount, f->childCount);
  put(time, f->time);
  put(mass, f->mass);
  put(spin, f->spin);
  return GAL_OK;
}

int gal_forest_get_satellite_host(const gal_forest* f, int32_t* satellite_host) {
  if (!f || !satellite_host) return GAL_ERR_ARGUMENT;
  std::memcpy(satellite_host, f->satHost.data(), f->satHost.size() * sizeof(int32_t));
  return GAL_OK;
}

double gal_satellite_merging_time(const gal_params* p, double mass_host, double mass_satellite, double t,
                                  double velocity_radial, double velocity_tangential, double multiplier) {
  if (!p || !(mass_host > 0.0) || !(mass_satellite > 0.0)) return NAN;
  const Cosmo c = cosmo_of(p);
  double rv, vv;
  virial(c, mass_host, std::max(c.redshift(t), 0.0), rv, vv);
  const double mu = mass_host / (mass_host + mass_satellite);
  return jiang2008_time(rv / vv * kMpcPerKmPerSToGyr, mass_host / mass_satellite, mu, velocity_radial,
                        velocity_tangential, multiplier);
}

int gal_satellite_orbits(uint64_t seed, double mu, int64_t n, double* velocity_radial, double* velocity_tangential) {
  if (n < 0 || !(mu > 0.0 && mu <= 1.0) || (n > 0 && (!velocity_radial || !velocity_tangential))) return GAL_ERR_ARGUMENT;
  std::mt19937_64 rng(splitmix64(seed));
  for (int64_t i = 0; i < n; ++i) benson2005_orbit(rng, mu, velocity_radial[i], velocity_tangential[i]);
  return GAL_OK;
}

void gal_forest_free(gal_forest* f) { delete f; }

}  // extern "C"
