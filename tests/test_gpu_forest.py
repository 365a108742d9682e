"""Whole-forest evolution on the GPU (one CUDA graph per evolution) against the
oracle's restatement of the tree evolver: final states, snapshots at the
output times, counters, replay determinism, the autotuner, and baryon
conservation."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, workloads

pytestmark = pytest.mark.gpu

MASSES = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
          _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


@pytest.fixture(scope="module")
def case(params, table, oracle_mod):
    f = forest.build(params, n_trees=48, seed=3, root_mass_min=1e10, root_mass_max=3e12, mass_resolution=1e8)
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    # The oracle with the closed-form cooling radius the kernels use (the
    # Brent root it replaces agrees to 1e-6; tests/test_oracle_golden.py).
    ref = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)
    return f, state0, times, ref


@pytest.fixture(scope="module")
def sensitivity(case, table, oracle_mod):
    """How far the oracle's own final states and snapshots move when the
    relative tolerance changes by 10%: the conditioning of each value.
    Mergers build spheroids in these trees, and a spheroid black hole that
    grows by Bondi-Hoyle accretion (rate ~ M^2) towards its Eddington limit
    can end anywhere between hundreds and 5e5 Msun with such a change (or
    with the last bits of the host's libm)."""
    f, state0, times, (ref, _, _, ref_snaps) = case
    moved = [oracle_mod.evolve_forest(workloads.isolated_params(1e-3 * k), table, f, state0, times, brent=False)
             for k in (0.9, 1.1)]
    params = workloads.isolated_params()
    moved.append(oracle_mod.evolve_forest(params, table, f, state0, times, brent=True))
    moved.append(oracle_mod.evolve_forest(params, table, f, state0 * (1.0 + 1e-12), times, brent=False))
    return (np.max([np.abs(m[0] - ref) for m in moved], axis=0), np.max([np.abs(m[3] - ref_snaps) for m in moved], axis=0))


def _evolver(params, table, rates="fp64"):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    return MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)


def _bound(ref, params, f, nodes=None):
    """Ten times the tolerance in the solver's mixed norm (oracle/compare.py),
    with the absolute-tolerance scales of each node's state and halo mass."""
    from oracle import compare
    nodes = np.arange(f.n) if nodes is None else nodes
    param = np.zeros((_abi.NP, len(nodes)))
    param[_abi.P_MASS] = f.mass[nodes]
    return compare.parity_bound(ref, ref, param, params)


def _worst(a, ref, bound):
    bad = np.argwhere(np.abs(a - ref) > bound)
    return [(int(v), int(i), float(a[v, i]), float(ref[v, i])) for v, i in bad[:5]]


def test_plain_forest_matches_oracle(case, sensitivity, params, table, oracle_mod):
    f, state0, times, (ref, ref_status, ref_counters, ref_snaps) = case
    sens, sens_snaps = sensitivity
    ev = _evolver(params, table)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status, counters, snaps, snap_node, snap_out = fe.results()
    assert np.all(status == 0) and np.all(ref_status == 0)
    # The plain form is the reference's FP64 arithmetic: every final mass and
    # metal mass of every node within ten times the tolerance of the oracle
    # (in practice to rounding), or, for the values whose oracle answer moves
    # by more than that under a 10% change of the tolerance, within twice
    # that movement.
    # A black hole at the edge of its runaway can land on either side of it
    # whatever probe is tried (the outcome turns on the last bits of the
    # arithmetic): at most one node in a thousand may differ beyond that.
    bound = _bound(ref, params, f)
    within = np.abs(state - ref) <= bound
    conditioned = np.all(within | (np.abs(state - ref) <= bound + 2.0 * sens), axis=0)
    assert np.mean(conditioned) >= 0.999, _worst(state, ref, bound + 2.0 * sens)
    assert np.mean(np.all(within, axis=0)) > 0.998
    assert np.median(np.abs(state - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-12
    # Snapshots: same slots, same values.
    first, m = oracle_mod.forest_snapshots(f, times)
    assert snaps.shape == ref_snaps.shape == (_abi.NY, m)
    expected_node = np.repeat(np.arange(f.n), np.diff(np.append(first, m)))
    sbound = _bound(ref_snaps, params, f, expected_node) + 2.0 * sens_snaps
    assert np.mean(np.all(np.abs(snaps - ref_snaps) <= sbound, axis=0)) >= 0.999, _worst(snaps, ref_snaps, sbound)
    np.testing.assert_array_equal(snap_node, expected_node)
    assert np.all(times[snap_out] >= f.time[snap_node])
    # Same step sequences for almost every node: a rounding-level difference
    # (the short FP64 log/exp of the kernels against the C library's) that
    # flips one step decision is inherited by every later node of the branch.
    same = np.all(counters == ref_counters, axis=0)
    assert same.mean() > 0.97
    assert fe.accepted_steps() == int(counters[0].sum())
    fe.close()
    ev.close()
    # The device snapshots in the reference's output layout: the last output
    # holds every root, with the snapshot values under the reference's names.
    from galacticus_gb300 import output
    out = output.layout(params, f, times, snaps, snap_node, snap_out)
    last = f"Outputs/Output{len(times)}"
    roots = np.flatnonzero(f.parent < 0)
    np.testing.assert_array_equal(np.sort(out[f"{last}/nodeData/nodeIndex"]), roots)
    idx = out[f"{last}/nodeData/nodeIndex"]
    slot = {int(n): j for j, n in enumerate(snap_node) if snap_out[j] == len(times) - 1}
    np.testing.assert_array_equal(out[f"{last}/nodeData/diskMassStellar"],
                                  snaps[_abi.Y_DISK_STARS, [slot[int(n)] for n in idx]])
    assert out[f"{last}/mergerTreeCount"].sum() == roots.size


def test_graph_replays_are_identical(case, params, table):
    f, state0, times, _ = case
    ev = _evolver(params, table)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    a = fe.results()
    fe.evolve()
    fe.evolve()
    b = fe.results()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    fe.close()
    ev.close()


def test_fast_forest_within_tolerance(case, params, table):
    f, state0, times, (ref, _, _, _) = case
    ev = _evolver(params, table, "fp32")
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


def test_autotune_picks_a_built_shape(case, params, table):
    f, state0, times, _ = case
    ev = _evolver(params, table, "fp32")
    fe = forest.ForestEvolver(ev, f, state0, times)
    t = fe.autotune(repeats=2)
    valid = t > 0
    assert valid.sum() >= 3 and t[0] < 0  # 64 threads is not built for the FP32 form
    shapes = [(64, 1), (128, 1), (128, 2), (256, 1), (256, 2), (512, 1)]
    best = shapes[int(np.argmin(np.where(valid, t, np.inf)))]
    assert ev.get_launch() == best
    fe.evolve()
    assert np.all(fe.results()[1] == 0)
    fe.close()
    ev.close()


def test_forest_matches_reference_root_finder(case, sensitivity, params, table, oracle_mod):
    """Against the oracle with the reference's Brent cooling radius: within
    ten times the tolerance everywhere (ill-conditioned values: within twice
    the oracle's own movement beyond it)."""
    f, state0, times, _ = case
    ref, _, _, _ = oracle_mod.evolve_forest(params, table, f, state0, times, brent=True)
    ev = _evolver(params, table)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state = fe.results()[0]
    bound = _bound(ref, params, f) + 2.0 * sensitivity[0]
    assert np.mean(np.all(np.abs(state - ref) <= bound, axis=0)) >= 0.999, _worst(state, ref, bound)
    fe.close()
    ev.close()


def test_surrogate_forest_conserves_baryons(case, params, table, trained):
    from galacticus_gb300 import surrogate
    f, state0, times, (ref, _, _, _) = case
    ev = _evolver(params, table, "fp32")
    trained.install(ev)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status, _, _, _, _ = fe.results()
    assert np.all(status == 0)
    network, tab = surrogate.stats(ev)
    assert network > 0
    roots = np.flatnonzero(f.parent < 0)
    fb = params.omega_baryon / params.omega_matter
    baryons = state[MASSES][:, roots].sum(axis=0)
    assert np.abs(baryons / (fb * f.mass[roots]) - 1.0).max() < 1e-3
    fe.close()
    ev.close()


def test_forest_rejects_bad_topology(params, table):
    ev = _evolver(params, table)
    f = forest.build(params, n_trees=2, seed=1, root_mass_min=1e10, root_mass_max=1e10)
    bad = forest.Forest(f.tree.copy(), f.parent.copy(), f.child_first.copy(), f.child_count.copy(), f.time.copy(),
                        f.mass.copy(), f.spin.copy())
    i = int(np.flatnonzero(bad.parent >= 0)[0])
    bad.time[i] = bad.time[bad.parent[i]] + 1.0  # a progenitor after its parent
    with pytest.raises(RuntimeError, match="inconsistent forest topology"):
        forest.ForestEvolver(ev, bad, forest.initial_state(params, bad), forest.output_times(params))
    # A node whose parent does not list it among its progenitors.
    orphan = forest.Forest(f.tree.copy(), f.parent.copy(), f.child_first.copy(), f.child_count.copy(), f.time.copy(),
                           f.mass.copy(), f.spin.copy())
    p = int(np.flatnonzero(orphan.child_count > 1)[0])
    orphan.child_count[p] -= 1
    with pytest.raises(RuntimeError, match="progenitors must be contiguous"):
        forest.ForestEvolver(ev, orphan, forest.initial_state(params, orphan), forest.output_times(params))
    # The context stays usable.
    fe = forest.ForestEvolver(ev, f, forest.initial_state(params, f), forest.output_times(params))
    fe.evolve()
    assert np.all(fe.results()[1] == 0)
    fe.close()
    ev.close()


def test_small_cpu_configuration(table, oracle_mod):
    """The reference's small plain configuration: 32 PCH trees (seed 1), roots
    log-uniform 1e10-1e12 Msun, resolution 1e9, z=8 to 0, relative tolerance
    1e-2: the GPU forest against the oracle's, node by node."""
    params = workloads.isolated_params(tolerance_relative=1e-2)
    f = forest.build(params, n_trees=32, seed=1, root_mass_min=1e10, root_mass_max=1e12, root_mass_slope=0.0,
                     mass_resolution=1e9)
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    ref, ref_status, _, _ = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)
    ev = _evolver(params, table)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status = fe.results()[:2]
    assert np.all(status == 0) and np.all(ref_status == 0)
    bound = _bound(ref, params, f)
    assert np.all(np.abs(state - ref) <= bound), _worst(state, ref, bound)
    fe.close()
    ev.close()


def test_forest_needs_a_built_form(params, table, trained):
    """A surrogate with FP64 rates has no forest kernel: a clear error, and
    the context stays usable once the rates are FP32."""
    ev = _evolver(params, table, "fp64")
    trained.install(ev)
    f = forest.build(params, n_trees=2, seed=2, root_mass_min=1e10, root_mass_max=1e10)
    fe = forest.ForestEvolver(ev, f, forest.initial_state(params, f), forest.output_times(params))
    with pytest.raises(RuntimeError, match="FP32"):
        fe.evolve()
    ev.set_rate_precision("fp32")
    fe.evolve()
    assert np.all(fe.results(snapshots=False)[1] == 0)
    fe.close()
    ev.close()


@pytest.mark.parametrize("rates", ["fp64", "fp32"])
@pytest.mark.parametrize("satellite_galaxy", [5e9, 1e10])
def test_progenitors_merge_as_in_the_oracle(table, oracle_mod, rates, satellite_galaxy):
    """The GPU's merger of two progenitors (mergerMassMovementsSimple, a minor
    and a major case) equals the oracle's bit for bit with every operator
    off: the merge is the same sequence of FP64 additions."""
    import test_forest_cpu as cpu
    q = workloads.isolated_params()
    q.physics = 0
    f = cpu.merger_forest()
    s = cpu.merger_states(satellite_galaxy)
    ev = _evolver(q, table, rates)
    fe = forest.ForestEvolver(ev, f, s, np.array([]))
    fe.evolve()
    state, status = fe.results(snapshots=False)[:2]
    fe.close()
    ev.close()
    ref = oracle_mod.evolve_forest(q, table, f, s, np.array([]))[0]
    assert np.all(status == 0)
    np.testing.assert_array_equal(state[:, 0], ref[:, 0])
