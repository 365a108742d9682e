"""Spheroid physics on the GPU against the oracle.

The isolated-halo batches start with empty disks and spheroids, so there
the spheroid operators never act.  This batch (workloads.galaxy_halos) starts
every halo with a gaseous and stellar disk and spheroid, metals and a black
hole of 1e4-1e9 Msun, so that every operator runs from the first step:
spheroid star formation (nodes/operators/physics/star_formation/
spheroids.F90:152-), spheroid feedback under the rate limit
(stellar_feedback/spheroids.F90:116-208) and Bondi-Hoyle accretion from the
spheroid gas, at the accretion radius or at the Jeans length
(black_holes/accretion_rates/standard.F90:262-300).  The plain form (FP64)
and the FP32-rate form are checked with the bound of the other parity tests:
ten times the ODE tolerance in the solver's mixed norm (oracle/compare.py);
for the FP32-rate form, halos whose oracle answer itself moves by more than
that bound when the tolerance changes by 10% must lie within twice that
movement.
"""

import math

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

N_HALOS = 8192


def jeans_branch(params, batch):
    """Per halo, at the initial state: whether the spheroid gas density
    enters the Bondi-Hoyle rate at the Jeans length (True) or at the
    accretion radius G M / c_s^2 (False), as the reference decides it."""
    amu, kB = 1.660538782e-27, 1.3806504e-23
    mu = 1.0 / (2.0 * 0.7514 / 1.0078250322 + 3.0 * 0.2486 / 4.0026032545)
    cs = math.sqrt(5.0 * kB * params.bh_temperature_spheroid / 3.0 / mu / amu) / 1e3
    g = 6.673e-11 * 1.98892e30 / 1e6 / (1e6 * 3.08567758135e16)
    a = params.radius_factor_spheroid * batch.param[_abi.P_SPIN] * batch.param[_abi.P_RADIUS_VIRIAL]
    r_acc = g * batch.state[_abi.Y_BLACK_HOLE] / cs ** 2
    x = r_acc / a
    rho = batch.state[_abi.Y_SPHEROID_GAS] / (2.0 * np.pi * a ** 3) / (x * (1.0 + x) ** 3)
    jeans = np.minimum(cs / np.sqrt(g) / np.sqrt(rho), a)
    return (rho > 1.0) & (jeans > r_acc)


@pytest.fixture(scope="module")
def reference(table, oracle_mod):
    params = workloads.isolated_params()
    batch = workloads.galaxy_halos(n=N_HALOS, seed=12)
    ref, ref_step, ref_status, ref_counters = oracle_mod.evolve_batch(params, table, batch.state, batch.param,
                                                                      batch.t_start, batch.t_end, batch.step)
    moved = []
    for factor in (0.9, 1.1):
        q = workloads.isolated_params(tolerance_relative=1e-3 * factor)
        moved.append(oracle_mod.evolve_batch(q, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                             batch.step)[0])
    sensitivity = np.maximum(np.abs(moved[0] - ref), np.abs(moved[1] - ref))
    return params, batch, ref, ref_status, ref_counters, sensitivity


def test_batch_exercises_every_spheroid_branch(reference):
    """The batch is what this module needs: both sides of the Jeans-length
    condition, and spheroid star formation, feedback and black-hole growth
    that change the masses by more than the tolerance."""
    params, batch, ref, ref_status, _, _ = reference
    assert np.all(ref_status == 0)
    branch = jeans_branch(params, batch)
    assert 0.05 < branch.mean() < 0.95, branch.mean()
    grew = ref[_abi.Y_SPHEROID_STARS] / batch.state[_abi.Y_SPHEROID_STARS] - 1.0
    assert np.mean(grew > 1e-2) > 0.25
    fed = ref[_abi.Y_BLACK_HOLE] / batch.state[_abi.Y_BLACK_HOLE] - 1.0
    assert np.mean(fed[branch] > 1e-2) > 0.25 and np.mean(fed[~branch] > 1e-2) > 0.25


@pytest.mark.parametrize("rates", ["fp64", "fp32"])
def test_spheroid_physics_parity(table, reference, rates):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params, batch, ref, ref_status, ref_counters, sensitivity = reference
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
    g = batch.copy()
    status, counters = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True, counters=True)
    ev.close()
    assert np.all(status == 0)
    ratio = compare.parity_ratio(g.state, ref, batch.state, batch.param, params)
    branch = jeans_branch(params, batch)
    if rates == "fp64":
        # The reference's arithmetic: every value of every halo within the bound.
        assert ratio.max() <= 1.0, f"worst parity ratio {ratio.max():.3g}"
        assert np.mean((counters[0] == ref_counters[0]) & (counters[1] == ref_counters[1])) > 0.99
    else:
        bound = compare.parity_bound(ref, batch.state, batch.param, params)
        ok = (ratio <= 1.0) | (np.abs(g.state - ref) <= bound + 2.0 * sensitivity)
        bad = np.argwhere(~ok)
        assert len(bad) == 0, [(int(v), int(i), float(g.state[v, i]), float(ref[v, i])) for v, i in bad[:5]]
        assert np.mean(np.all(ratio <= 1.0, axis=0)) > 0.995
    # Both sides of the Jeans-length condition hold the bound on their own.
    for side in (branch, ~branch):
        assert np.all(ratio[:, side] <= 1.0) or rates == "fp32"
        assert np.mean(np.all(ratio[:, side] <= 1.0, axis=0)) > 0.99
    # The spheroid values themselves.
    for idx in (_abi.Y_SPHEROID_GAS, _abi.Y_SPHEROID_GAS_METALS, _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE):
        assert np.mean(ratio[idx] <= 1.0) > 0.995
