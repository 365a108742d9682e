"""The tree builder's branching on the GPU (gal_gpu_forest_build) against
the oracle's restatement of its walk: on the same roots and tables, every
tree is the oracle's bit for bit (topology, masses; the walk uses only
IEEE-defined operations and neither side contracts to FMA), and its times
are a function of the oracle's w.  Builds are deterministic, agree with the
host builder in distribution, and forests with satellites come out valid
and evolve."""

import numpy as np
import pytest

from galacticus_gb300 import forest, workloads

pytestmark = pytest.mark.gpu

SPEC = dict(seed=3, root_mass_min=1e10, root_mass_max=1e13, mass_resolution=1e8)


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


@pytest.fixture(scope="module")
def evolver(params, table):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32")
    yield ev
    ev.close()


@pytest.fixture(scope="module")
def built(params, evolver):
    return forest.build(params, n_trees=1024, gpu=evolver, **SPEC)


def _tree_slices(f):
    starts = np.flatnonzero(np.diff(np.append(-1, f.tree)) != 0)
    return starts, np.append(starts[1:], f.n)


def test_gpu_branching_matches_the_oracle(built, params, oracle_mod):
    f = built
    starts, ends = _tree_slices(f)
    assert len(starts) == 1024 and np.all(f.parent[starts] == -1)
    tables = forest.branch_tables(params, **SPEC)
    mass, w, parent, child_first, child_count, tree_first = oracle_mod.grow_trees(tables, SPEC["seed"], f.mass[starts])
    o_ends = np.append(tree_first[1:], len(mass))
    assert f.n == len(mass)
    np.testing.assert_array_equal(starts, tree_first)
    local = np.repeat(starts, ends - starts)
    np.testing.assert_array_equal(np.where(f.parent >= 0, f.parent - local, -1), parent)
    np.testing.assert_array_equal(f.child_count, child_count)
    has = child_count > 0  # (a split with both progenitors unresolved leaves the oracle's first index set)
    np.testing.assert_array_equal((f.child_first - local)[has], child_first[has])
    np.testing.assert_array_equal(f.mass, mass)
    # Times are a decreasing function of w (w = delta_c0/D grows into the
    # past), equal w giving equal times.
    order = np.argsort(w, kind="stable")
    assert np.all(np.diff(f.time[order]) <= 0.0)
    assert np.all(np.diff(f.time[order])[np.diff(w[order]) == 0.0] == 0.0)


def test_gpu_branching_is_deterministic(built, params, evolver):
    again = forest.build(params, n_trees=1024, gpu=evolver, **SPEC)
    for name in ("parent", "child_first", "child_count", "mass", "time", "spin"):
        np.testing.assert_array_equal(getattr(again, name), getattr(built, name))


def test_gpu_branching_agrees_with_the_host_builder_in_distribution(built, params):
    host = forest.build(params, n_trees=1024, **SPEC)
    np.testing.assert_array_equal(host.mass[host.parent < 0], built.mass[built.parent < 0])
    assert abs(built.n / host.n - 1.0) < 0.03, (built.n, host.n)
    bins = np.linspace(8.0, 13.0, 11)
    h_host = np.histogram(np.log10(host.mass[host.child_count == 0]), bins)[0]
    h_gpu = np.histogram(np.log10(built.mass[built.child_count == 0]), bins)[0]
    ok = (h_host + h_gpu) > 50
    chi2 = np.sum((h_host - h_gpu)[ok] ** 2 / (h_host + h_gpu)[ok])
    assert chi2 < 2.0 * ok.sum() + 10, (h_host, h_gpu)


def test_gpu_built_forest_with_satellites_evolves(params, evolver, table, oracle_mod):
    """A GPU-built forest with satellites through the whole pipeline: the
    FP32-rate forest evolution against the oracle's evolution of the same
    forest, node by node within the FP32-rate forms' bound."""
    from oracle import compare
    from galacticus_gb300 import _abi
    f = forest.build(params, n_trees=64, gpu=evolver, satellites=forest.SATELLITES_JIANG2008, **SPEC)
    host = f.satellite_host
    phases = np.flatnonzero(host >= 0)
    assert len(phases) > 100
    assert np.all(f.time[phases] == f.time[host[phases]])
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    fe = forest.ForestEvolver(evolver, f, state0, times)
    fe.evolve()
    state, status = fe.results()[:2]
    fe.close()
    assert np.all(status == 0)
    ref, ref_status = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)[:2]
    assert np.all(ref_status == 0)
    param = np.zeros((_abi.NP, f.n))
    param[_abi.P_MASS] = f.mass
    within = np.all(np.abs(state - ref) <= compare.parity_bound(ref, ref, param, params), axis=0)
    assert within.mean() > 0.995, within.mean()


def test_gpu_branching_grows_its_node_arrays(built, params, evolver, monkeypatch):
    """A first capacity far below the forest's size: the growth overflows,
    repeats with larger arrays and ends with the same forest."""
    monkeypatch.setenv("GALNODE_BRANCH_CAPACITY", str(built.n // 6))
    again = forest.build(params, n_trees=1024, gpu=evolver, **SPEC)
    for name in ("parent", "child_first", "child_count", "mass", "time", "spin"):
        np.testing.assert_array_equal(getattr(again, name), getattr(built, name))


@pytest.mark.parametrize("case", [
    dict(pch=dict(g0=1.0, gamma1=0.0, gamma2=0.0), spec=dict(mass_resolution=1e9)),           # plain EPS rates
    dict(pch=dict(accuracy_first=0.05, accuracy_second=0.05), spec=dict(redshift_max=12.0)),  # finer steps
    dict(pch=dict(gamma2=-0.1), spec=dict(root_redshift=1.0, root_mass_max=1e12)),             # roots at z = 1
])
def test_gpu_branching_matches_the_oracle_for_other_parameters(case, params, evolver, oracle_mod):
    pch = forest.pch_params()
    for k, v in case["pch"].items():
        setattr(pch, k, v)
    spec = dict(seed=9, root_mass_min=1e11, root_mass_max=1e13, mass_resolution=1e8, redshift_max=8.0)
    spec.update(case["spec"])
    root_redshift = spec.pop("root_redshift", 0.0)
    f = forest.build(params, n_trees=128, gpu=evolver, pch=pch, root_redshift=root_redshift, **spec)
    starts, ends = _tree_slices(f)
    tables = forest.branch_tables(params, pch=pch, root_redshift=root_redshift, **spec)
    mass, w, parent, child_first, child_count, tree_first = oracle_mod.grow_trees(tables, spec["seed"], f.mass[starts])
    assert f.n == len(mass) and np.array_equal(starts, tree_first)
    local = np.repeat(starts, ends - starts)
    np.testing.assert_array_equal(np.where(f.parent >= 0, f.parent - local, -1), parent)
    np.testing.assert_array_equal(f.child_count, child_count)
    np.testing.assert_array_equal(f.mass, mass)


def test_gpu_built_forest_plain_form_matches_the_oracle(params, evolver, table, oracle_mod):
    """The plain FP64 form on a GPU-built forest with satellites: every node
    within ten times the tolerance of the oracle (allowing, as for the host
    builder's forests, for nodes whose oracle answer itself moves with the
    tolerance), the snapshot labels exactly."""
    from oracle import compare
    from galacticus_gb300 import _abi
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    f = forest.build(params, n_trees=32, gpu=evolver, satellites=forest.SATELLITES_JIANG2008, **SPEC)
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    plain = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp64")
    fe = forest.ForestEvolver(plain, f, state0, times)
    fe.evolve()
    state, status, _, snaps, snap_node, _ = fe.results()
    fe.close()
    plain.close()
    ref, ref_status, _, ref_snaps = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)
    assert np.all(status == 0) and np.all(ref_status == 0)
    first, m = oracle_mod.forest_snapshots(f, times)
    np.testing.assert_array_equal(snap_node, np.repeat(np.arange(f.n), np.diff(np.append(first, m))))
    param = np.zeros((_abi.NP, f.n))
    param[_abi.P_MASS] = f.mass
    within = np.all(np.abs(state - ref) <= compare.parity_bound(ref, ref, param, params), axis=0)
    assert within.mean() > 0.998, within.mean()
