"""Forests with satellites on the GPU against the oracle: satellite phases
(frozen halo mass and virial scales, no accretion) evolved by the same
persistent forest kernel as every other node, merged into the piece of the
host's branch that starts at their merging time (Jiang et al. 2008 on a
Benson 2005 orbit).  The plain form within ten times the tolerance of the
oracle, node by node and at every output; the FP32-rate and surrogate
forms within the bounds of the forests without satellites."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, output, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


@pytest.fixture(scope="module")
def case(params, table, oracle_mod):
    f = forest.build(params, n_trees=48, seed=3, root_mass_min=1e10, root_mass_max=3e12, mass_resolution=1e8,
                     satellites=forest.SATELLITES_JIANG2008)
    assert np.sum(f.satellite_host >= 0) > 500
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    ref = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)
    return f, state0, times, ref


@pytest.fixture(scope="module")
def sensitivity(case, table, oracle_mod):
    """How far the oracle's answers move under a 10% change of the relative
    tolerance (as for the forests without satellites)."""
    f, state0, times, (ref, _, _, ref_snaps) = case
    moved = [oracle_mod.evolve_forest(workloads.isolated_params(1e-3 * k), table, f, state0, times, brent=False)
             for k in (0.9, 1.1)]
    return (np.max([np.abs(m[0] - ref) for m in moved], axis=0), np.max([np.abs(m[3] - ref_snaps) for m in moved], axis=0))


def _evolver(params, table, rates):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    return MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)


def _bound(ref, params, f, nodes=None):
    from oracle import compare
    nodes = np.arange(f.n) if nodes is None else nodes
    param = np.zeros((_abi.NP, len(nodes)))
    param[_abi.P_MASS] = f.mass[nodes]
    return compare.parity_bound(ref, ref, param, params)


def test_plain_forest_with_satellites_matches_oracle(case, sensitivity, params, table, oracle_mod):
    f, state0, times, (ref, ref_status, ref_counters, ref_snaps) = case
    sens, sens_snaps = sensitivity
    ev = _evolver(params, table, "fp64")
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status, counters, snaps, snap_node, snap_out = fe.results()
    assert np.all(status == 0) and np.all(ref_status == 0)
    bound = _bound(ref, params, f)
    within = np.abs(state - ref) <= bound
    conditioned = np.all(within | (np.abs(state - ref) <= bound + 2.0 * sens), axis=0)
    assert np.mean(conditioned) >= 0.999
    assert np.mean(np.all(within, axis=0)) > 0.998
    # The satellite phases themselves, every one.
    phases = f.satellite_host >= 0
    assert np.all(conditioned[phases])
    first, m = oracle_mod.forest_snapshots(f, times)
    expected_node = np.repeat(np.arange(f.n), np.diff(np.append(first, m)))
    np.testing.assert_array_equal(snap_node, expected_node)
    sbound = _bound(ref_snaps, params, f, expected_node) + 2.0 * sens_snaps
    assert np.mean(np.all(np.abs(snaps - ref_snaps) <= sbound, axis=0)) >= 0.999
    assert np.mean(np.all(counters == ref_counters, axis=0)) > 0.97
    # Baryons over each tree's roots (the central and the satellites that
    # outlive the tree) at f_b M_root.
    roots = np.flatnonzero(f.parent < 0)
    baryons = np.bincount(f.tree[roots], weights=state[[_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS,
                                                       _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS, _abi.Y_SPHEROID_STARS,
                                                       _abi.Y_BLACK_HOLE]][:, roots].sum(axis=0),
                          minlength=f.n_trees)
    main = np.array([roots[f.tree[roots] == t][np.argmax(f.mass[roots][f.tree[roots] == t])] for t in range(f.n_trees)])
    fb = params.omega_baryon / params.omega_matter
    assert np.max(np.abs(baryons / (fb * f.mass[main]) - 1.0)) < 1e-3
    # The outputs mark the satellites.
    out = output.layout(params, f, times, snaps, snap_node, snap_out)
    last = f"Outputs/Output{len(times)}/nodeData"
    idx = out[f"{last}/nodeIndex"]
    np.testing.assert_array_equal(out[f"{last}/nodeIsIsolated"], np.where(f.satellite_host[idx] >= 0, 0, 1))
    fe.close()
    ev.close()


@pytest.mark.parametrize("rates", ["fp32", "surrogate"])
def test_fast_forest_with_satellites_within_tolerance(case, params, table, rates, request):
    f, state0, times, (ref, _, _, _) = case
    ev = _evolver(params, table, "fp32")
    if rates == "surrogate":
        # The shared network with its own error map (other modules rely on it).
        request.getfixturevalue("trained").install(ev)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status, _, _, _, _ = fe.results()
    assert np.all(status == 0)
    within = np.all(np.abs(state - ref) <= _bound(ref, params, f), axis=0)
    assert within.mean() > 0.995, within.mean()
    roots = f.parent < 0
    stars = state[_abi.Y_DISK_STARS][roots] + state[_abi.Y_SPHEROID_STARS][roots]
    stars_ref = ref[_abi.Y_DISK_STARS][roots] + ref[_abi.Y_SPHEROID_STARS][roots]
    assert abs(stars.sum() / stars_ref.sum() - 1.0) < 1e-4
    fe.close()
    ev.close()
