"""The oracle's right-hand side, one node operator at a time, against the
reference's formulas restated here independently (physics mask with a single
operator enabled; the constants are the reference's GSL MKSA values).

  reincorporation  haloDynamicalTime: dM_out/dt = -m M_out / t_dyn
                   (hot_halo/outflow_reincorporation/halo_dynamical_time.F90:113-128)
  star formation   timescale + dynamicalTime + instantaneous populations
                   (star_formation/rates/disks/timescale.F90:109-130,
                   star_formation/timescales/dynamical_time.F90:121-189,
                   stellar_populations/properties/instantaneous.F90:133-219)
  feedback         powerLaw under rateLimit (stellar_feedback/outflows/power_law/
                   _class.F90:118-164, rate_limit.F90)
  cooling          whiteFrenk1991: M_hot / t_dyn once the cooling radius reaches the
                   outer radius, the infall of the cooling radius below it
                   (cooling/cooling_rate/White-Frenk.F90:132-185,
                   cooling_radius/simple.F90:229-311), nothing above the velocity cut-off
  gas accretion    Omega_b / Omega_m of the halo's growth (accretion/halo/simple.F90:281-319)
  spheroids        star formation and feedback with the spheroid's parameters
  black holes      Bondi-Hoyle-Lyttleton accretion from the hot halo, capped by the hot
                   gas and the Eddington rate, and from the spheroid gas with the Jeans
                   length (accretion/Bondi_Hoyle_Lyttleton.F90:34-78,
                   black_holes/fundamentals.F90:123-138, accretion_rates/standard.F90:221-440)
"""

import math

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

# GSL MKSA constants as the reference uses them (numerical/constants).
MEGAPARSEC = 3.08567758135e22
GIGAYEAR = 3.15581497635456e16
MPC_PER_KMS_TO_GYR = MEGAPARSEC / 1.0e3 / GIGAYEAR
G_SI, M_H, SIGMA_T, C_LIGHT = 6.673e-11, 1.0078250322 * 1.660538782e-27, 6.65245893699e-29, 2.99792458e8


def node(mass=1e12, rvir=0.2, vvir=150.0, spin=0.04, mdot=0.0):
    p = np.zeros(_abi.NP)
    p[_abi.P_MASS], p[_abi.P_MASS_RATE], p[_abi.P_RADIUS_VIRIAL], p[_abi.P_VELOCITY_VIRIAL], p[_abi.P_SPIN] = \
        mass, mdot, rvir, vvir, spin
    return p


def only(mask):
    params = workloads.isolated_params()
    params.physics = mask
    return params


def test_reincorporation(oracle_mod, table):
    params = only(_abi.PHYS_REINCORPORATION)
    prm = node()
    y = np.zeros(_abi.NY)
    y[_abi.Y_OUTFLOWED_MASS], y[_abi.Y_OUTFLOWED_METALS] = 3e9, 4e7
    d = oracle_mod.rhs(params, table, prm, y)
    tdyn = prm[_abi.P_RADIUS_VIRIAL] / prm[_abi.P_VELOCITY_VIRIAL] * MPC_PER_KMS_TO_GYR
    rate = params.reincorporation_multiplier * y[_abi.Y_OUTFLOWED_MASS] / tdyn
    assert d[_abi.Y_OUTFLOWED_MASS] == pytest.approx(-rate, rel=1e-13)
    assert d[_abi.Y_HOT_MASS] == pytest.approx(rate, rel=1e-13)
    assert d[_abi.Y_HOT_METALS] == pytest.approx(rate * 4e7 / 3e9, rel=1e-13)
    others = [i for i in range(_abi.NY) if i not in (_abi.Y_OUTFLOWED_MASS, _abi.Y_OUTFLOWED_METALS,
                                                       _abi.Y_HOT_MASS, _abi.Y_HOT_METALS)]
    assert np.all(d[others] == 0.0)


def disk_timescale(params, prm):
    sf = params.sf_disk
    radius = params.radius_factor_disk * prm[_abi.P_SPIN] * prm[_abi.P_RADIUS_VIRIAL]
    v = prm[_abi.P_VELOCITY_VIRIAL]
    return max(MPC_PER_KMS_TO_GYR * radius / v * (v / 200.0) ** sf.exponent_velocity / sf.efficiency,
               sf.timescale_minimum), radius


def test_disk_star_formation(oracle_mod, table):
    params = only(_abi.PHYS_STAR_FORMATION_DISK)
    prm = node()
    y = np.zeros(_abi.NY)
    y[_abi.Y_DISK_GAS], y[_abi.Y_DISK_GAS_METALS] = 5e9, 5e7
    d = oracle_mod.rhs(params, table, prm, y)
    tau, _ = disk_timescale(params, prm)
    sfr = y[_abi.Y_DISK_GAS] / tau
    stars = (1.0 - params.recycled_fraction) * sfr
    z = y[_abi.Y_DISK_GAS_METALS] / y[_abi.Y_DISK_GAS]
    assert d[_abi.Y_DISK_STARS] == pytest.approx(stars, rel=1e-12)
    assert d[_abi.Y_DISK_GAS] == pytest.approx(-stars, rel=1e-12)
    assert d[_abi.Y_DISK_STARS_METALS] == pytest.approx(z * stars, rel=1e-12)
    assert d[_abi.Y_DISK_GAS_METALS] == pytest.approx(-z * stars + params.metal_yield * sfr, rel=1e-12)


@pytest.mark.parametrize("vvir", [40.0, 300.0])
def test_disk_feedback_with_rate_limit(oracle_mod, table, vvir):
    params = only(_abi.PHYS_STAR_FORMATION_DISK | _abi.PHYS_FEEDBACK_DISK)
    prm = node(vvir=vvir)
    y = np.zeros(_abi.NY)
    y[_abi.Y_DISK_GAS] = 5e9
    d_sf = oracle_mod.rhs(only(_abi.PHYS_STAR_FORMATION_DISK), table, prm, y)
    d = oracle_mod.rhs(params, table, prm, y)
    tau, radius = disk_timescale(params, prm)
    sfr = y[_abi.Y_DISK_GAS] / tau
    o = params.outflow_disk
    outflow = (o.velocity_characteristic / vvir) ** o.exponent * sfr
    limit = y[_abi.Y_DISK_GAS] / (MPC_PER_KMS_TO_GYR * radius / vvir) / o.timescale_fractional_minimum
    expected = min(outflow, limit)
    assert d[_abi.Y_OUTFLOWED_MASS] == pytest.approx(expected, rel=1e-12)
    assert d[_abi.Y_DISK_GAS] - d_sf[_abi.Y_DISK_GAS] == pytest.approx(-expected, rel=1e-12)


def test_rapid_cooling_and_the_velocity_cutoff(oracle_mod, table):
    params = only(_abi.PHYS_COOLING)
    # A dense, cool hot halo: the cooling radius reaches the virial radius.
    prm = node(mass=1e10, rvir=0.02, vvir=50.0)
    y = np.zeros(_abi.NY)
    y[_abi.Y_HOT_MASS], y[_abi.Y_HOT_METALS] = 1.5e9, 1.5e9 * 0.0188
    rcool = oracle_mod.cooling_radius(params, table, prm, y[_abi.Y_HOT_MASS], y[_abi.Y_HOT_METALS])
    assert rcool >= prm[_abi.P_RADIUS_VIRIAL]
    d = oracle_mod.rhs(params, table, prm, y)
    tdyn = prm[_abi.P_RADIUS_VIRIAL] / prm[_abi.P_VELOCITY_VIRIAL] * MPC_PER_KMS_TO_GYR
    rate = y[_abi.Y_HOT_MASS] / tdyn
    assert d[_abi.Y_HOT_MASS] == pytest.approx(-rate, rel=1e-12)
    assert d[_abi.Y_DISK_GAS] == pytest.approx(rate, rel=1e-12)
    assert d[_abi.Y_DISK_GAS_METALS] == pytest.approx(rate * 0.0188, rel=1e-12)
    # Above the cut-off velocity nothing cools.
    params.cooling_velocity_cutoff = 40.0
    assert np.all(oracle_mod.rhs(params, table, prm, y) == 0.0)


@pytest.mark.parametrize("enhancement,binding", [(None, "bondi"), (1.0e6, "eddington")])
def test_hot_mode_black_hole_accretion(oracle_mod, table, enhancement, binding):
    """Bondi-Hoyle-Lyttleton accretion from the hot halo at the accretion
    radius G M_BH / c_s^2 (Bondi_Hoyle_Lyttleton.F90:34-59), under the
    hot-gas and Eddington caps; with a large enhancement the Eddington rate
    binds."""
    params = only(_abi.PHYS_BLACK_HOLE_ACCRETION)
    if enhancement is not None:
        params.bh_enhancement_hot_halo = enhancement
    prm = node()
    rvir, v = prm[_abi.P_RADIUS_VIRIAL], prm[_abi.P_VELOCITY_VIRIAL]
    y = np.zeros(_abi.NY)
    y[_abi.Y_HOT_MASS], y[_abi.Y_BLACK_HOLE] = 1e11, 1e9
    # Hot mode throughout: the cooling radius is inside 0.9 r_vir.
    assert oracle_mod.cooling_radius(params, table, prm, y[_abi.Y_HOT_MASS], 0.0) < 0.9 * rvir
    d = oracle_mod.rhs(params, table, prm, y)
    amu, kB = 1.660538782e-27, 1.3806504e-23
    mu = 1.0 / (2.0 * 0.7514 / 1.0078250322 + 3.0 * 0.2486 / 4.0026032545)
    temperature = 0.5 * amu * mu * (1e3 * v) ** 2 / kB
    cs = math.sqrt(5.0 * kB * temperature / 3.0 / mu / amu) / 1e3
    g_internal = G_SI * 1.98892e30 / 1e6 / MEGAPARSEC
    r_acc = min(g_internal * y[_abi.Y_BLACK_HOLE] / cs ** 2, rvir)
    rc = params.core_radius_fraction * rvir
    x = rvir / rc
    rho = y[_abi.Y_HOT_MASS] / (4.0 * math.pi * rc ** 3) / (x - math.atan(x)) / (1.0 + (r_acc / rc) ** 2)
    bhl = 1e3 * GIGAYEAR / MEGAPARSEC * 4.0 * math.pi
    bondi = params.bh_enhancement_hot_halo * bhl * r_acc ** 2 * rho * cs
    hot_cap = y[_abi.Y_HOT_MASS] / (rvir / cs * MPC_PER_KMS_TO_GYR)
    eddington = y[_abi.Y_BLACK_HOLE] * 4.0 * math.pi * G_SI * M_H * GIGAYEAR / SIGMA_T / C_LIGHT \
        / params.bh_efficiency_radiative
    accreted = min(bondi, hot_cap, eddington)
    assert accreted == (bondi if binding == "bondi" else eddington)
    kept = 1.0 - params.bh_efficiency_radiative - params.bh_efficiency_jet
    assert d[_abi.Y_BLACK_HOLE] == pytest.approx(kept * accreted, rel=1e-12)
    assert d[_abi.Y_HOT_MASS] == pytest.approx(-accreted, rel=1e-12)


def test_slow_cooling_infall_rate(oracle_mod, table):
    """Below the outer radius the cooling rate is the infall of the cooling
    radius, 4 pi r^2 rho(r) dr/dt (White-Frenk.F90:132-185), with the
    growth rate of cooling_radius/simple.F90:229-311 for an isothermal
    beta = 2/3 profile and CIE cooling (d ln t_cool / d ln rho = -1):
    dr/dt = r / t_dyn / (2 x^2 / (1 + x^2)), x = r / r_core."""
    params = only(_abi.PHYS_COOLING)
    prm = node()
    rvir = prm[_abi.P_RADIUS_VIRIAL]
    y = np.zeros(_abi.NY)
    y[_abi.Y_HOT_MASS], y[_abi.Y_HOT_METALS] = 8e10, 8e10 * 0.003
    r = oracle_mod.cooling_radius(params, table, prm, y[_abi.Y_HOT_MASS], y[_abi.Y_HOT_METALS])
    assert 0.0 < r < rvir
    d = oracle_mod.rhs(params, table, prm, y)
    tdyn = rvir / prm[_abi.P_VELOCITY_VIRIAL] * MPC_PER_KMS_TO_GYR
    rc = params.core_radius_fraction * rvir
    xo, x = rvir / rc, r / rc
    rho = y[_abi.Y_HOT_MASS] / (4.0 * math.pi * rc ** 3) / (xo - math.atan(xo)) / (1.0 + x * x)
    rate = 4.0 * math.pi * r * r * rho * r / tdyn / (2.0 * x * x / (1.0 + x * x))
    assert d[_abi.Y_HOT_MASS] == pytest.approx(-rate, rel=1e-12)
    assert d[_abi.Y_DISK_GAS] == pytest.approx(rate, rel=1e-12)
    assert d[_abi.Y_DISK_GAS_METALS] == pytest.approx(rate * 0.003, rel=1e-12)


def test_cgm_accretion(oracle_mod, table):
    """Hot gas accretes the universal baryon fraction of the halo's growth,
    metal-free (circumgalactic_medium/accretion.F90:517-593,
    accretion/halo/simple.F90:281-319, failed fraction 0)."""
    params = only(_abi.PHYS_CGM_ACCRETION)
    d = oracle_mod.rhs(params, table, node(mdot=3e11), np.zeros(_abi.NY))
    assert d[_abi.Y_HOT_MASS] == pytest.approx(params.omega_baryon / params.omega_matter * 3e11, rel=1e-14)
    assert np.count_nonzero(d) == 1
    assert np.all(oracle_mod.rhs(params, table, node(mdot=-1e11), np.zeros(_abi.NY)) == 0.0)


@pytest.mark.parametrize("gas", [5e9, 5e-7])
def test_spheroid_star_formation_and_feedback(oracle_mod, table, gas):
    """The spheroid's own timescale and outflow parameters; below 1e-6 Msun
    of gas nothing forms (star_formation/spheroids.F90:152-)."""
    params = only(_abi.PHYS_STAR_FORMATION_SPHEROID | _abi.PHYS_FEEDBACK_SPHEROID)
    prm = node()
    y = np.zeros(_abi.NY)
    y[_abi.Y_SPHEROID_GAS], y[_abi.Y_SPHEROID_GAS_METALS] = gas, gas * 0.01
    d = oracle_mod.rhs(params, table, prm, y)
    if gas < 1e-6:
        assert np.all(d == 0.0)
        return
    sf, o = params.sf_spheroid, params.outflow_spheroid
    radius = params.radius_factor_spheroid * prm[_abi.P_SPIN] * prm[_abi.P_RADIUS_VIRIAL]
    v = prm[_abi.P_VELOCITY_VIRIAL]
    tau = max(MPC_PER_KMS_TO_GYR * radius / v * (v / 200.0) ** sf.exponent_velocity / sf.efficiency,
              sf.timescale_minimum)
    sfr = gas / tau
    stars = (1.0 - params.recycled_fraction) * sfr
    outflow = min((o.velocity_characteristic / v) ** o.exponent * sfr,
                  gas / (MPC_PER_KMS_TO_GYR * radius / v) / o.timescale_fractional_minimum)
    assert d[_abi.Y_SPHEROID_STARS] == pytest.approx(stars, rel=1e-12)
    assert d[_abi.Y_SPHEROID_GAS] == pytest.approx(-stars - outflow, rel=1e-12)
    assert d[_abi.Y_OUTFLOWED_MASS] == pytest.approx(outflow, rel=1e-12)
    assert d[_abi.Y_SPHEROID_GAS_METALS] == pytest.approx(
        -0.01 * stars + params.metal_yield * sfr - 0.01 * outflow, rel=1e-12)


def test_cooling_radius_from_the_cooling_time(oracle_mod, table):
    """coolingRadiusSimple: the radius where the cooling time equals the
    time available (coolingTimeAvailableWhiteFrenk1991 with ageFactor 0:
    the halo dynamical time).  The cooling time is (dof/2) k T n_tot /
    Lambda with n_tot = n_H / f_H + n_e (cooling_time/simple.F90:128-179;
    abundances.F90:781-883 for the hydrogen mass and number fractions); with
    CIE cooling it scales as 1/rho, so r = r_core sqrt(t_avail/t_cool(0) - 1).
    The table is interpolated here by the Python restatement."""
    from galacticus_gb300.cie_tables import _interp_ln
    params = workloads.isolated_params()
    prm = node()
    rvir, v = prm[_abi.P_RADIUS_VIRIAL], prm[_abi.P_VELOCITY_VIRIAL]
    mass_hot, z = 8e10, 0.003
    amu, kB, m_h = 1.660538782e-27, 1.3806504e-23, 1.0078250322 * 1.660538782e-27
    mu = 1.0 / (2.0 * 0.7514 / 1.0078250322 + 3.0 * 0.2486 / 4.0026032545)
    temperature = 0.5 * amu * mu * (1e3 * v) ** 2 / kB
    rc = params.core_radius_fraction * rvir
    xo = rvir / rc
    rho0 = mass_hot / (4.0 * math.pi * rc ** 3) / (xo - math.atan(xo))
    x_h = min(max(z / 0.0188 * (0.7070 - 0.7514) + 0.7514, 0.7), 0.7514)
    y_he = min(z / 0.0188 * (0.2740 - 0.2486) + 0.2486, 0.2486)
    f_h = (x_h / 1.0078250322) / (x_h / 1.0078250322 + y_he / 4.0026032545)
    n_h = rho0 * x_h * 1.98892e30 / m_h / 1e6 / MEGAPARSEC ** 3
    z_solar = z / 0.0188
    lam = table.interpolate_cooling(n_h, temperature, z_solar)
    n_e = _interp_ln(np.log(table.electron_density), np.log(table.temperature), table.metallicity,
                     np.log(temperature), z_solar) * n_h
    t_cool = params.cooling_degrees_of_freedom / 2.0 * kB * temperature * (n_h / f_h + n_e) / 1e-7 / lam / GIGAYEAR
    t_avail = rvir / v * MPC_PER_KMS_TO_GYR
    expected = min(max(rc * math.sqrt(max(t_avail / t_cool - 1.0, 0.0)), 0.0), rvir)
    assert 0.0 < expected < rvir
    closed = oracle_mod.cooling_radius(params, table, prm, mass_hot, mass_hot * z, brent=False)
    brent = oracle_mod.cooling_radius(params, table, prm, mass_hot, mass_hot * z, brent=True)
    assert closed == pytest.approx(expected, rel=1e-12)
    assert brent == pytest.approx(expected, rel=1e-6)


@pytest.mark.parametrize("mass_bh,jeans_branch", [(1e7, False), (1e4, True)])
def test_spheroid_black_hole_accretion(oracle_mod, table, mass_bh, jeans_branch):
    """Bondi-Hoyle-Lyttleton accretion from the spheroid gas at the
    spheroid temperature (accretion_rates/standard.F90:262-300): the
    Hernquist gas density at the accretion radius G M / c_s^2, or at the
    Jeans length c_s / sqrt(G rho) (limited to the spheroid radius) when that
    is larger (thermodynamics/ideal_gases.F90:34-69,
    accretion/Bondi_Hoyle_Lyttleton.F90:34-78)."""
    params = only(_abi.PHYS_BLACK_HOLE_ACCRETION)
    prm = node()
    y = np.zeros(_abi.NY)
    y[_abi.Y_SPHEROID_GAS], y[_abi.Y_SPHEROID_GAS_METALS], y[_abi.Y_BLACK_HOLE] = 1e9, 1e7, mass_bh
    d = oracle_mod.rhs(params, table, prm, y)
    amu, kB = 1.660538782e-27, 1.3806504e-23
    mu = 1.0 / (2.0 * 0.7514 / 1.0078250322 + 3.0 * 0.2486 / 4.0026032545)
    cs = math.sqrt(5.0 * kB * params.bh_temperature_spheroid / 3.0 / mu / amu) / 1e3
    g_internal = G_SI * 1.98892e30 / 1e6 / MEGAPARSEC
    a = params.radius_factor_spheroid * prm[_abi.P_SPIN] * prm[_abi.P_RADIUS_VIRIAL]

    def hernquist(r):
        x = r / a
        return y[_abi.Y_SPHEROID_GAS] / (2.0 * math.pi * a ** 3) / (x * (1.0 + x) ** 3)

    r_acc = g_internal * mass_bh / cs ** 2
    rho = hernquist(r_acc)
    assert rho > 1.0
    jeans = min(cs / math.sqrt(g_internal) / math.sqrt(rho), a)
    assert (jeans > r_acc) == jeans_branch
    if jeans > r_acc:
        rho = hernquist(jeans)
    rate = params.bh_enhancement_spheroid * 1e3 * GIGAYEAR / MEGAPARSEC * 4.0 * math.pi * (g_internal * mass_bh) ** 2 \
        * rho / cs ** 3
    eddington = mass_bh * 4.0 * math.pi * G_SI * M_H * GIGAYEAR / SIGMA_T / C_LIGHT / params.bh_efficiency_radiative
    rate = min(rate, eddington)
    kept = 1.0 - params.bh_efficiency_radiative - params.bh_efficiency_jet
    assert d[_abi.Y_BLACK_HOLE] == pytest.approx(kept * rate, rel=1e-12)
    assert d[_abi.Y_SPHEROID_GAS] == pytest.approx(-rate, rel=1e-12)
    assert d[_abi.Y_SPHEROID_GAS_METALS] == pytest.approx(-rate * 1e7 / 1e9, rel=1e-12)


def krumholz2009_rate(mass_gas, metals_gas, radius, frequency=0.385, clumping=5.0, fast=False):
    """The reference's disk star-formation rate with krumholz2009, restated
    with the exact functions (no tables) and an adaptive quadrature to 1e-10:
    2 pi int r nu Sigma f(Sigma) f_H2(s) dr over the exponential gas disk on
    [0, 10 R_d] (integrated_surface_density.F90:131-190; Krumholz2009.F90:
    312-414: chi = 0.77 (1 + 3.1 Z'^0.365), s = ln(1 + 0.6 chi + 0.01 chi^2)
    / (0.04 Z' X_H c Sigma/1e12), f = (X_H Sigma / 85e12 Msun/Mpc^2)^(+-0.33);
    utilities.F90:36-63 for f_H2)."""
    from scipy.integrate import quad
    zs = metals_gas / mass_gas / 0.0188
    if zs <= 0.0:
        return 0.0
    x_h = min(max(zs * (0.7070 - 0.7514) + 0.7514, 0.7), 0.7514)
    chi = 0.77 * (1.0 + 3.1 * zs ** 0.365)
    s_norm = math.log(1.0 + 0.6 * chi + 0.01 * chi * chi) / (0.04 * zs)
    sigma_norm = x_h * clumping / 1e12
    sigma0 = mass_gas / (2.0 * math.pi * radius ** 2)

    def f_h2(s):
        if fast:
            return 1.0 - 0.75 * s / (1.0 + 0.25 * s) if s < 2.0 else 0.0
        if s < 1e-6:
            return 1.0 - 0.75 * s
        if s >= 10.0:
            return 1.0 / (0.75 / 1.214008) ** 5 / 5.0 / s ** 5
        delta = 0.0712 / (0.1 / s + 0.675) ** 2.8
        return 1.0 - 1.0 / (1.0 + ((1.0 + delta) / 0.75 / s) ** 5) ** 0.2

    def integrand(r):
        sg = sigma0 * math.exp(-r / radius)
        sd = x_h * sg / 85e12
        return r * frequency * sg * (sd ** -0.33 if sd < 1.0 else sd ** 0.33) * f_h2(s_norm / (sigma_norm * sg))

    cut = [radius * math.log(x_h * sigma0 / 85e12)] if x_h * sigma0 / 85e12 > 1.0 else []
    cut += [radius * math.log(sigma0 * sigma_norm / s_norm * 10.0)] if sigma0 * sigma_norm / s_norm * 10.0 > 1.0 else []
    cut = sorted(c for c in cut if 0.0 < c < 10.0 * radius)
    value = quad(integrand, 0.0, 10.0 * radius, points=cut or None, limit=400, epsrel=1e-10, epsabs=0.0)[0]
    return 2.0 * math.pi * value


@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("mass,metallicity", [(1e10, 0.02), (1e9, 0.002), (3e10, 0.03), (5e10, 0.01), (1e11, 0.001)])
def test_krumholz2009_disk_star_formation(oracle_mod, table, fast, mass, metallicity):
    """Disk star formation with the reference's default rate class: the
    oracle (tables and QAG at relative tolerance 1e-3, as the reference)
    within 1e-4 of the exact integral, through the instantaneous
    populations."""
    params = only(_abi.PHYS_STAR_FORMATION_DISK)
    params.sf_disk_rate = _abi.SF_RATE_KRUMHOLZ2009
    params.krumholz_fast = 1 if fast else 0
    prm = node()
    y = np.zeros(_abi.NY)
    y[_abi.Y_DISK_GAS], y[_abi.Y_DISK_GAS_METALS] = mass, mass * metallicity
    d = oracle_mod.rhs(params, table, prm, y)
    radius = params.radius_factor_disk * prm[_abi.P_SPIN] * prm[_abi.P_RADIUS_VIRIAL]
    expected = krumholz2009_rate(mass, mass * metallicity, radius, fast=fast)
    assert expected > 0.0 or fast  # the fast fraction vanishes beyond s = 2: a thin, metal-poor disk forms no stars
    sfr = d[_abi.Y_DISK_STARS] / (1.0 - params.recycled_fraction)
    assert sfr == pytest.approx(expected, rel=1e-4, abs=1e-300)
    assert d[_abi.Y_DISK_GAS_METALS] == pytest.approx(-metallicity * d[_abi.Y_DISK_STARS] + params.metal_yield * sfr,
                                                      rel=1e-9)


def test_krumholz2009_needs_metals(oracle_mod, table):
    """Metal-free gas forms no molecules and no stars (Krumholz2009.F90:378-388)."""
    params = only(_abi.PHYS_STAR_FORMATION_DISK)
    params.sf_disk_rate = _abi.SF_RATE_KRUMHOLZ2009
    y = np.zeros(_abi.NY)
    y[_abi.Y_DISK_GAS] = 1e10
    assert np.all(oracle_mod.rhs(params, table, node(), y) == 0.0)
