"""Merger forests on the CPU: the tree builder's invariants and the oracle's
whole-forest evolution (baryon conservation through promotion and merging)."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, workloads


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


@pytest.fixture(scope="module")
def small_forest(params):
    return forest.build(params, n_trees=24, seed=3, root_mass_min=1e10, root_mass_max=1e12, mass_resolution=1e8)


def test_sigma_normalisation(params):
    """sigma(M) equals sigma8 at the mass of an 8/h Mpc sphere."""
    import ctypes
    lib = forest._declare(_abi.load_library())
    pch = forest.pch_params()
    h = params.hubble_constant / 100.0
    rho = params.omega_matter * 3.0 * params.hubble_constant ** 2 / (8.0 * np.pi * workloads.G_INTERNAL)
    m8 = 4.0 / 3.0 * np.pi * rho * (8.0 / h) ** 3
    s = lib.gal_pch_sigma(ctypes.byref(params), ctypes.byref(pch), m8)
    assert abs(s / pch.sigma8 - 1.0) < 2e-3
    assert lib.gal_pch_sigma(ctypes.byref(params), ctypes.byref(pch), 1e10) > s


def eisenstein_hu_1999(k, omega_matter, omega_baryon, h, t_cmb, n_eff=3.046, m_nu=0.0):
    """Eisenstein & Hu (1999, ApJ 511, 5) eqs. 2-4 and 15-22, written out
    independently of the builder, k in 1/Mpc."""
    omh2, obh2, theta = omega_matter * h * h, omega_baryon * h * h, t_cmb / 2.7
    z_eq = 2.5e4 * omh2 * theta ** -4
    b1 = 0.313 * omh2 ** -0.419 * (1 + 0.607 * omh2 ** 0.674)
    b2 = 0.238 * omh2 ** 0.223
    z_d = 1291 * omh2 ** 0.251 / (1 + 0.659 * omh2 ** 0.828) * (1 + b1 * obh2 ** b2)
    y_d = (1 + z_eq) / (1 + z_d)
    s = 44.5 * np.log(9.83 / omh2) / np.sqrt(1 + 10 * obh2 ** 0.75)
    f_nu = m_nu / (94 * h * h * omega_matter)
    f_b = omega_baryon / omega_matter
    f_c = 1 - f_b
    f_cb, f_nub = f_c + f_b, f_nu + f_b
    p_c, p_cb = (5 - np.sqrt(1 + 24 * f_c)) / 4, (5 - np.sqrt(1 + 24 * f_cb)) / 4
    alpha = (f_c / f_cb) * (5 - 2 * (p_c + p_cb)) / (5 - 4 * p_cb) \
        * (1 - 0.533 * f_nub + 0.126 * f_nub ** 3) / (1 - 0.193 * np.sqrt(f_nu * n_eff) + 0.169 * f_nu * n_eff ** 0.2) \
        * (1 + y_d) ** (p_cb - p_c) * (1 + (p_c - p_cb) / 2 * (1 + 1 / ((3 - 4 * p_c) * (7 - 4 * p_cb))) / (1 + y_d))
    gamma_eff = omh2 * (np.sqrt(alpha) + (1 - np.sqrt(alpha)) / (1 + (0.43 * k * s) ** 4))
    q_eff = k * theta ** 2 / gamma_eff
    beta_c = 1 / (1 - 0.949 * f_nub)
    big_l = np.log(np.e + 1.84 * beta_c * np.sqrt(alpha) * q_eff)
    big_c = 14.4 + 325 / (1 + 60.5 * q_eff ** 1.11)
    t = big_l / (big_l + big_c * q_eff ** 2)
    if 0 < f_nu <= 0.3:
        q_nu = 3.92 * k * theta ** 2 / omh2 * np.sqrt(n_eff) / f_nu
        t = t * (1 + 1.2 * f_nu ** 0.64 * n_eff ** (0.3 + 0.6 * f_nu) / (q_nu ** -1.6 + q_nu ** 0.8))
    return t


@pytest.mark.parametrize("m_nu", [0.0, 0.06])
def test_transfer_function_eisenstein_hu_1999(params, m_nu):
    """The builder's default transfer function is the reference's default,
    transferFunctionEisensteinHu1999 (structure_formation/transfer_function/
    Eisenstein_Hu1999.F90), with and without massive neutrinos (the
    reference's transfer-function test uses both, source/tests/
    transfer_functions.F90:65-78)."""
    import ctypes
    lib = forest._declare(_abi.load_library())
    pch = forest.pch_params()
    assert pch.transfer_function == forest.TRANSFER_EISENSTEIN_HU_1999
    assert pch.neutrino_number_effective == 3.046 and pch.neutrino_mass_summed == 0.0
    pch.neutrino_mass_summed = m_nu
    h = params.hubble_constant / 100.0
    for k in np.geomspace(1e-3, 1e2, 16):
        got = lib.gal_pch_transfer(ctypes.byref(params), ctypes.byref(pch), k)
        want = eisenstein_hu_1999(k, params.omega_matter, params.omega_baryon, h, pch.temperature_cmb, m_nu=m_nu)
        assert abs(got / want - 1.0) < 1e-12, (k, got, want)
    # Large scales are unsuppressed; the 1998 zero-baryon form stays a
    # selectable alternative and differs from the 1999 fit by percents.
    assert abs(lib.gal_pch_transfer(ctypes.byref(params), ctypes.byref(pch), 1e-5) - 1.0) < 2e-3
    eh98 = forest.pch_params()
    eh98.transfer_function = forest.TRANSFER_EISENSTEIN_HU_1998
    ratio = [lib.gal_pch_transfer(ctypes.byref(params), ctypes.byref(eh98), k) /
             lib.gal_pch_transfer(ctypes.byref(params), ctypes.byref(forest.pch_params()), k) for k in (0.1, 1.0, 10.0)]
    assert all(0.8 < r < 1.2 for r in ratio) and any(abs(r - 1.0) > 1e-3 for r in ratio)
    bad = forest.pch_params()
    bad.transfer_function = 7
    assert np.isnan(lib.gal_pch_transfer(ctypes.byref(params), ctypes.byref(bad), 1.0))


@pytest.mark.parametrize("w", [1.686, 4.0])
def test_branching_rates_match_reference_known_answers(w):
    """The builder's branching rates against the reference's known answers
    (source/tests/merger_tree_branching.F90:76-78, 185-191, 224-234,
    390-399): for sigma(M) proportional to M^(-1/3) (an n = -1 power
    spectrum with a sharp k-space filter) and the unmodified rates (G0 = 1,
    gamma1 = gamma2 = 0), a 1e12 Msun branch with resolution 1e11 Msun
    splits at 2.498324530964044/sigma and loses mass below the resolution
    at 0.4181139013841312/sigma per unit of the critical overdensity, at
    any w; tolerances as the reference's (1e-4 and 2e-3)."""
    pch = forest.pch_params()
    pch.g0, pch.gamma1, pch.gamma2 = 1.0, 0.0, 0.0
    for sigma in (0.7, 2.3):
        rate, accretion = forest.branching_rates(pch, -1.0 / 3.0, sigma, 1e12, 1e11, w=w)
        assert rate == pytest.approx(2.498324530964044 / sigma, rel=1e-4)
        assert accretion == pytest.approx(0.4181139013841312 / sigma, rel=2e-3)


def test_branching_rates_modifier():
    """With the PCH modifier G0 (sigma1/sigma2)^gamma1 (w/sigma2)^gamma2
    (Parkinson_Cole_Helly.F90:265-634), the w dependence is the factor
    (w/sigma2)^gamma2, and G0 scales both rates."""
    pch = forest.pch_params()
    pch.g0, pch.gamma1, pch.gamma2 = 0.57, 0.38, -0.01
    r1, a1 = forest.branching_rates(pch, -0.25, 1.5, 1e12, 1e10, w=1.0)
    r2, a2 = forest.branching_rates(pch, -0.25, 1.5, 1e12, 1e10, w=3.0)
    assert r2 / r1 == pytest.approx(3.0 ** -0.01, rel=1e-12)
    assert a2 / a1 == pytest.approx(3.0 ** -0.01, rel=1e-12)
    pch.g0 = 1.14
    r3, a3 = forest.branching_rates(pch, -0.25, 1.5, 1e12, 1e10, w=1.0)
    assert r3 / r1 == pytest.approx(2.0, rel=1e-12) and a3 / a1 == pytest.approx(2.0, rel=1e-12)


def test_tree_invariants(small_forest, params):
    f = small_forest
    roots = np.flatnonzero(f.parent < 0)
    assert len(roots) == 24
    t0 = forest._declare(_abi.load_library()).gal_cosmic_time(params, 0.0)
    np.testing.assert_array_equal(f.time[roots], t0)
    child = f.parent >= 0
    # A progenitor is earlier and lighter than its parent.
    assert np.all(f.time[child] < f.time[f.parent[child]])
    assert np.all(f.mass[child] <= f.mass[f.parent[child]] * (1 + 1e-12))
    # Progenitors are contiguous, primary (most massive) first, and list their parent.
    for i in np.flatnonzero(f.child_count > 0):
        kids = np.arange(f.child_first[i], f.child_first[i] + f.child_count[i])
        assert np.all(f.parent[kids] == i)
        assert np.all(np.diff(f.mass[kids]) <= 0)
    # Progenitor masses never exceed their parent's in total; all above resolution.
    brought = np.zeros(f.n)
    np.add.at(brought, f.parent[child], f.mass[child])
    assert np.all(brought <= f.mass * (1 + 1e-12))
    assert f.mass.min() >= 1e8
    # Branches end at the maximum redshift or below the resolution.
    zmax_time = forest._declare(_abi.load_library()).gal_cosmic_time(params, 8.0)
    assert f.time.min() >= zmax_time - 1e-12


def test_tree_builder_is_deterministic(params):
    a = forest.build(params, n_trees=6, seed=11, root_mass_min=1e11, root_mass_max=1e11)
    b = forest.build(params, n_trees=6, seed=11, root_mass_min=1e11, root_mass_max=1e11)
    np.testing.assert_array_equal(a.mass, b.mass)
    np.testing.assert_array_equal(a.parent, b.parent)
    c = forest.build(params, n_trees=6, seed=12, root_mass_min=1e11, root_mass_max=1e11)
    assert a.n != c.n or not np.array_equal(a.mass, c.mass)


def test_root_mass_distribution(params):
    """dN/dln M ~ M^-0.9 over 1e10-1e14: the median root sits near the
    analytic median of that distribution."""
    f = forest.build(params, n_trees=400, seed=5, root_mass_min=1e10, root_mass_max=1e14, mass_resolution=1e9)
    roots = f.mass[f.parent < 0]
    s = -0.9
    a, b = 1e10 ** s, 1e14 ** s
    median = (a + 0.5 * (b - a)) ** (1 / s)
    assert abs(np.log10(np.median(roots)) - np.log10(median)) < 0.15


def test_oracle_forest_conserves_baryons(small_forest, params, table, oracle_mod):
    """Leaves start at the universal baryon fraction and primaries accrete it
    on the mass their progenitors did not bring, so every root ends with
    f_b M_root in baryons, less the mass radiated by black-hole accretion
    (the reference's mass-conservation check is 1e-3;
    testSuite/test-mass-conservation-standard.py:82)."""
    f = small_forest
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    state, status, counters, snaps = oracle_mod.evolve_forest(params, table, f, state0, times)
    assert np.all(status == 0)
    roots = np.flatnonzero(f.parent < 0)
    masses = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
              _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]
    baryons = state[masses][:, roots].sum(axis=0)
    fb = params.omega_baryon / params.omega_matter
    rel = np.abs(baryons / (fb * f.mass[roots]) - 1.0)
    assert rel.max() < 1e-3, rel.max()
    # Stars formed, mergers built spheroids, and every node took steps.
    assert np.all(state[_abi.Y_DISK_STARS][roots] + state[_abi.Y_SPHEROID_STARS][roots] > 0)
    assert np.mean(state[_abi.Y_SPHEROID_STARS][roots] > 0) > 0.5
    assert counters[0][f.child_count == 0].min() > 0
    # One snapshot per (node, output inside or at the start of its interval).
    first, m = oracle_mod.forest_snapshots(f, times)
    assert snaps.shape == (_abi.NY, m)
    assert m >= len(roots)  # every root is at the last output


def test_oracle_forest_is_deterministic_across_threads(small_forest, params, table, oracle_mod):
    state0 = forest.initial_state(params, small_forest)
    times = forest.output_times(params)
    a = oracle_mod.evolve_forest(params, table, small_forest, state0, times, threads=1)
    b = oracle_mod.evolve_forest(params, table, small_forest, state0, times, threads=4)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[3], b[3])


def test_timestep_criterion_cuts_evolve_calls(params):
    """The tree evolver's evolve calls are limited by
    mergerTreeEvolveTimestepSimple (merger_trees/evolve/timesteps/
    simple.F90:124-161): a call from t ends no later than
    t + min(0.1 / H(t), 1 Gyr).  A two-node forest (a leaf at z = 3 whose
    parent is the root at z = 0) evolved by the oracle equals the chain of
    single evolve calls over exactly those pieces, each with the halo's mass
    and virial scales at its start and the step size carried over."""
    from galacticus_gb300.cie_tables import CieTable
    from oracle import oracle
    table = CieTable()
    cosmo = workloads.Cosmology()
    t_root, t_leaf = cosmo.time(0.0), cosmo.time(3.0)
    f = forest.Forest(np.array([0, 0], np.int32), np.array([-1, 0], np.int32), np.array([1, 0], np.int32),
                      np.array([1, 0], np.int32), np.array([t_root, t_leaf]), np.array([1e12, 3e11]),
                      np.array([0.04, 0.04]))
    state0 = forest.initial_state(params, f)
    got = oracle.evolve_forest(params, table, f, state0, np.array([]), brent=True)[0][:, 1]
    # The pieces: a_{k+1} = min(a_k + min(0.1/H(a_k), 1), t_root).
    cuts = [t_leaf]
    while cuts[-1] < t_root:
        a = cuts[-1]
        rate = cosmo.hubble_gyr * np.sqrt(cosmo.omega_matter * (1.0 + cosmo.redshift(a)) ** 3 + cosmo.omega_lambda)
        cuts.append(min(a + min(0.1 / rate, 1.0), t_root))
    assert len(cuts) > 8  # the 11 Gyr interval is cut many times
    y = state0[:, 1:2].copy()
    step = np.array([-1.0])
    rate_accretion = (1e12 - 3e11) / (t_root - t_leaf)
    for a, b in zip(cuts[:-1], cuts[1:]):
        m = 3e11 + rate_accretion * (a - t_leaf)
        r, v = cosmo.virial(np.array([m]), cosmo.redshift(np.array([a])))
        prm = np.array([[m], [rate_accretion], r, v, [0.04]])
        y, step, status, _ = oracle.evolve_batch(params, table, y, prm, np.array([a]), np.array([b]), step)
        assert status[0] == 0
    np.testing.assert_allclose(got, y[:, 0], rtol=1e-7, atol=1e-6)  # numpy vs C++ virial scales: 1e-15 in, ~1e-9 out
    # Without the limit (one call for the whole interval) the answer moves.
    q = workloads.isolated_params()
    q.timestep_relative, q.timestep_absolute = 0.0, 1e6
    single = oracle.evolve_forest(q, table, f, state0, np.array([]), brent=True)[0][:, 1]
    assert np.max(np.abs(single - got) / np.maximum(np.abs(got), 1.0)) > 1e-3


def merger_forest():
    """A root and two progenitors, 1 Gyr earlier."""
    return forest.Forest(np.array([0, 0, 0], np.int32), np.array([-1, 0, 0], np.int32), np.array([1, 0, 0], np.int32),
                         np.array([2, 0, 0], np.int32), np.array([13.0, 12.0, 12.0]), np.array([1e12, 6e11, 2e11]),
                         np.full(3, 0.04))


def merger_states(satellite_galaxy):
    """Progenitor states: a host with a disk and a small spheroid, and a
    satellite whose disk-plus-spheroid mass is `satellite_galaxy`."""
    s = np.zeros((_abi.NY, 3))
    s[:, 1] = [5e10, 1e8, 2e9, 1e7, 1e10, 2e8, 2e10, 3e8, 1e8, 1e6, 1e9, 1e6]
    s[:, 2] = [1e10, 5e7, 1e9, 1e7, 0.8 * satellite_galaxy, 1e7, 0.2 * satellite_galaxy, 2e7, 0.0, 0.0, 0.0, 2e5]
    return s


@pytest.mark.parametrize("satellite_galaxy,major", [(5e9, False), (1e10, True)])
def test_progenitors_merge_with_the_reference_mass_movements(params, table, oracle_mod, satellite_galaxy, major):
    """mergerMassMovementsSimple (satellites/merging/mass_movements/
    simple.F90): the host galaxy here is 3.11e10 Msun, so a satellite of
    5e9 Msun (ratio 0.16) merges as a minor merger -- its gas and stars to
    the host's spheroid, the host's disk unmoved -- and one of 1e10 Msun
    (0.32 >= 0.25) as a major merger, both galaxies into the spheroid.  With
    every operator off, the root's state is the merger's result exactly."""
    q = workloads.isolated_params()
    q.physics = 0
    f = merger_forest()
    s = merger_states(satellite_galaxy)
    state = oracle_mod.evolve_forest(q, table, f, s, np.array([]))[0]
    host, sat, root = s[:, 1], s[:, 2], state[:, 0]
    for v in (_abi.Y_HOT_MASS, _abi.Y_HOT_METALS, _abi.Y_OUTFLOWED_MASS, _abi.Y_OUTFLOWED_METALS, _abi.Y_BLACK_HOLE):
        assert root[v] == host[v] + sat[v]
    gas_sph = host[_abi.Y_SPHEROID_GAS] + (sat[_abi.Y_DISK_GAS] + sat[_abi.Y_SPHEROID_GAS])
    stars_sph = host[_abi.Y_SPHEROID_STARS] + (sat[_abi.Y_DISK_STARS] + sat[_abi.Y_SPHEROID_STARS])
    if major:
        assert root[_abi.Y_SPHEROID_GAS] == gas_sph + host[_abi.Y_DISK_GAS]
        assert root[_abi.Y_SPHEROID_STARS] == stars_sph + host[_abi.Y_DISK_STARS]
        assert np.all(root[[_abi.Y_DISK_GAS, _abi.Y_DISK_GAS_METALS, _abi.Y_DISK_STARS, _abi.Y_DISK_STARS_METALS]] == 0.0)
    else:
        assert root[_abi.Y_SPHEROID_GAS] == gas_sph and root[_abi.Y_SPHEROID_STARS] == stars_sph
        np.testing.assert_array_equal(root[_abi.Y_DISK_GAS:_abi.Y_DISK_STARS_METALS + 1],
                                      host[_abi.Y_DISK_GAS:_abi.Y_DISK_STARS_METALS + 1])
    # Gas, stars and black holes are conserved.
    masses = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
              _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]
    assert root[masses].sum() == pytest.approx(host[masses].sum() + sat[masses].sum(), rel=1e-15)
