"""The oracle against the reference's own known answers (CPU only).

These pin the CPU restatement before it is trusted as the GPU's checker:
closedBox/leakyBox reproducibility values, the ODE-solver unit-test values,
the CIE cooling-function normalisation and baryon mass conservation.
"""

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads
from cases import box_case, known_answers


@pytest.mark.parametrize("name", ["closedBox", "leakyBox"])
def test_box_models(oracle_mod, table, name):
    p, batch, expect, tol = box_case()[name]
    state, _, status, _ = oracle_mod.evolve_batch(p, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                  batch.step)
    assert status[0] == 0
    got = [state[_abi.Y_DISK_GAS, 0], state[_abi.Y_DISK_STARS, 0], state[_abi.Y_DISK_GAS_METALS, 0],
           state[_abi.Y_DISK_STARS_METALS, 0]]
    np.testing.assert_allclose(got, expect, rtol=tol)


def test_ode_sinusoid_forward_and_reversed(oracle_mod):
    ka = known_answers()["odeSinusoid"]
    for x in ka["xEnd"]:
        rc, y = oracle_mod.ode_test(1, 0.0, x, [0.0], 1e-9, 1e-9)
        assert rc == 0
        np.testing.assert_allclose(y[0], 1.0 - np.cos(x), atol=ka["toleranceAbsolute"], rtol=ka["toleranceRelative"])
        rc, y = oracle_mod.ode_test(1, x, 0.0, [1.0 - np.cos(x)], 1e-9, 1e-9)
        assert rc == 0
        np.testing.assert_allclose(y[0], 0.0, atol=ka["toleranceAbsolute"])


def test_ode_harmonic_oscillator_with_latent_integrals(oracle_mod):
    ka = known_answers()["odeHarmonicOscillator"]
    for i, x in enumerate(ka["xEnd"]):
        rc, y = oracle_mod.ode_test(2, 0.0, x, [1.0, 0.0, 0.0, 0.0], 1e-9, 1e-9)
        assert rc == 0
        np.testing.assert_allclose(y[:2], [np.cos(x), -np.sin(x)], rtol=ka["toleranceRelative"], atol=1e-9)
        np.testing.assert_allclose(y[2:], [ka["latent1"][i], ka["latent2"][i]], rtol=ka["toleranceRelative"])


def test_cie_normalisation(oracle_mod, table):
    ka = known_answers()["coolingFunctionCIE"]
    v = oracle_mod.lib().oracle_cooling_function(table.struct, ka["numberDensityHydrogen"], ka["temperature"],
                                                 ka["metallicitySolar"])
    assert abs(v / ka["value"] - 1.0) < ka["toleranceRelative"]
    v2 = table.interpolate_cooling(ka["numberDensityHydrogen"], ka["temperature"], ka["metallicitySolar"])
    assert abs(v2 / ka["value"] - 1.0) < ka["toleranceRelative"]


def test_cie_density_slope_is_two(oracle_mod, table):
    """cieFileCoolingFunctionDensityLogSlope = 2 (CIE_file.F90:514-533)."""
    l = oracle_mod.lib()
    for T, Z in [(1e5, 0.1), (3e6, 1.0), (2e4, 0.0), (1e8, 5.0)]:
        a = l.oracle_cooling_function(table.struct, 1e-3, T, Z)
        b = l.oracle_cooling_function(table.struct, 2e-3, T, Z)
        assert abs(b / a - 4.0) < 1e-12


def test_cie_extrapolation_rules(oracle_mod, table):
    """T beyond the grid is clamped ("extrapolate" implemented as a clamp,
    CIE_file.F90:257-274); Z beyond the grid is fixed (:276-292)."""
    l = oracle_mod.lib()
    assert l.oracle_cooling_function(table.struct, 1.0, 1e10, 1.0) == l.oracle_cooling_function(table.struct, 1.0, 1e9, 1.0)
    assert l.oracle_cooling_function(table.struct, 1.0, 1e6, 100.0) == l.oracle_cooling_function(table.struct, 1.0, 1e6, 30.0)
    # Z below the first non-zero row interpolates linearly in Z toward the Z=0 row.
    z1 = table.metallicity[1]
    a, b, m = (l.oracle_cooling_function(table.struct, 1.0, 1e6, z) for z in (0.0, z1, 0.5 * z1))
    assert abs(np.log(m) - 0.5 * (np.log(a) + np.log(b))) < 1e-12


def test_cooling_radius_closed_form_matches_root_finder(oracle_mod, table):
    """The closed-form cooling radius (used on the GPU) agrees with the
    reference's Brent root (relative tolerance 1e-6, cooling_radius/simple.F90:133)."""
    batch = workloads.isolated_halos(n=3000, seed=12)
    p = workloads.isolated_params()
    rng = np.random.default_rng(12)
    checked = 0
    for i in range(batch.n):
        prm = batch.param[:, i]
        # Hot-gas masses and metallicities spread around the workload's so that
        # interior roots, r_outer and zero are all reached.
        m = batch.state[_abi.Y_HOT_MASS, i] * 10.0 ** rng.uniform(-3.0, 0.3)
        z = m * 10.0 ** rng.uniform(-6.0, -1.0)
        rb = oracle_mod.cooling_radius(p, table, prm, m, z, brent=True)
        rc = oracle_mod.cooling_radius(p, table, prm, m, z, brent=False)
        if rb > 0 and rb < prm[_abi.P_RADIUS_VIRIAL]:
            checked += 1
        assert abs(rb - rc) <= 2e-6 * max(rb, 1e-30)
    assert checked > 300


def test_baryon_mass_conservation(oracle_mod, table):
    """Sum of baryonic reservoirs is conserved by every operator except
    black-hole radiative losses (test-mass-conservation-standard.py:82)."""
    ka = known_answers()["massConservation"]
    batch = workloads.isolated_halos(n=500, seed=13)
    p = workloads.isolated_params()
    p.physics = _abi.PHYS_ALL & ~_abi.PHYS_BLACK_HOLE_ACCRETION & ~_abi.PHYS_CGM_ACCRETION
    state, _, status, _ = oracle_mod.evolve_batch(p, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                  batch.step)
    assert np.all(status == 0)
    mass_idx = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
                _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]
    before = batch.state[mass_idx].sum(axis=0)
    after = state[mass_idx].sum(axis=0)
    np.testing.assert_allclose(after, before, rtol=ka["toleranceRelative"])
    # Halo accretion adds exactly f_b dM/dt dt to the reservoirs.
    p.physics = _abi.PHYS_CGM_ACCRETION
    b = batch.copy()
    b.param[_abi.P_MASS_RATE] = 1.0e10
    state, _, status, _ = oracle_mod.evolve_batch(p, table, b.state, b.param, b.t_start, b.t_end, b.step)
    gained = state[mass_idx].sum(axis=0) - b.state[mass_idx].sum(axis=0)
    np.testing.assert_allclose(gained, 0.045 / 0.3 * 1.0e10 * (b.t_end - b.t_start), rtol=1e-9)


def test_metals_never_exceed_gas_mass_fraction_one(oracle_mod, table):
    batch = workloads.isolated_halos(n=500, seed=14)
    p = workloads.isolated_params()
    state, _, status, _ = oracle_mod.evolve_batch(p, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                  batch.step)
    assert np.all(status == 0)
    for m, z in [(_abi.Y_HOT_MASS, _abi.Y_HOT_METALS), (_abi.Y_DISK_GAS, _abi.Y_DISK_GAS_METALS),
                 (_abi.Y_DISK_STARS, _abi.Y_DISK_STARS_METALS)]:
        assert np.all(state[z] <= state[m] * (1 + 1e-9) + 1e-3)


def test_oracle_threads_do_not_change_results(oracle_mod, table):
    batch = workloads.isolated_halos(n=300, seed=15)
    p = workloads.isolated_params()
    a = oracle_mod.evolve_batch(p, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, threads=1)
    b = oracle_mod.evolve_batch(p, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, threads=4)
    np.testing.assert_array_equal(a[0], b[0])
