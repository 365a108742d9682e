"""Forest snapshots written in the reference's output layout
(merger_trees/outputter/standard.F90), from the oracle's forest evolution."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, output, workloads


@pytest.fixture(scope="module")
def evolved(table, oracle_mod):
    params = workloads.isolated_params()
    f = forest.build(params, n_trees=6, seed=11, root_mass_min=1e10, root_mass_max=1e12, mass_resolution=1e9)
    times = forest.output_times(params, n=5, redshift_max=3.0)
    state0 = forest.initial_state(params, f)
    _, status, _, snap = oracle_mod.evolve_forest(params, table, f, state0, times)
    assert np.all(status == 0)
    first, m = oracle_mod.forest_snapshots(f, times)
    # The oracle's slots: each node's outputs in increasing order from its
    # first slot; recover (node, output) of every slot.
    node = np.repeat(np.arange(f.n), np.diff(np.append(first, m)))
    outputs = np.zeros(m, dtype=np.int64)
    for i in range(f.n):
        t0 = f.time[i]
        t1 = f.time[f.parent[i]] if f.parent[i] >= 0 else t0
        ks = [k for k, t in enumerate(times) if (t == t0 and (f.parent[i] < 0 or t0 < t1)) or t0 < t < t1]
        assert len(ks) == np.count_nonzero(node == i)
        outputs[node == i] = ks
    return params, f, times, snap, node, outputs


def test_layout_and_values(tmp_path, evolved):
    params, f, times, snap, node, outputs = evolved
    path = tmp_path / "galacticus.npz"
    output.write(path, params, f, times, snap, node, outputs)
    out = output.read(path)
    groups = out["Outputs"]
    assert out["Outputs"]["attrs"]["outputCount"] == len(times)
    for k, t in enumerate(times):
        g = groups[f"Output{k + 1}"]
        assert g["attrs"]["outputTime"] == t
        z = forest.redshift(params, t)
        assert abs(g["attrs"]["outputExpansionFactor"] * (1.0 + z) - 1.0) < 1e-14
        d = g["nodeData"]
        # Every node alive at the output time, once: the node's own time is
        # at or before it and its parent's after it (roots up to the end).
        alive = [i for i in range(f.n) if f.time[i] <= t and
                 (f.parent[i] < 0 and t == f.time[i] or f.parent[i] >= 0 and t < f.time[f.parent[i]])]
        assert sorted(d["nodeIndex"].tolist()) == sorted(alive)
        # Trees one after another, located by the per-tree datasets.
        tree_of = f.tree[d["nodeIndex"]]
        assert np.all(np.diff(tree_of) >= 0)
        for tr, s, c in zip(g["mergerTreeIndex"], g["mergerTreeStartIndex"], g["mergerTreeCount"]):
            assert np.all(tree_of[s:s + c] == tr)
        assert g["mergerTreeCount"].sum() == len(alive)
        # Values: the snapshot of each node at this output, under the
        # reference's property names.
        for j, i in enumerate(d["nodeIndex"]):
            slot = np.flatnonzero((node == i) & (outputs == k))[0]
            for y, name in output.PROPERTY_NAMES.items():
                assert d[name][j] == snap[y, slot]
        assert np.all(d["parentIndex"] == f.parent[d["nodeIndex"]])
        assert np.all(d["nodeIsIsolated"] == 1)
        assert np.allclose(d["basicMass"], output.halo_mass(f, d["nodeIndex"], t), rtol=0, atol=0)
    # The final output holds the roots at z = 0 with the reference's names.
    last = groups[f"Output{len(times)}"]["nodeData"]
    assert sorted(last["nodeIndex"].tolist()) == sorted(np.flatnonzero(f.parent < 0).tolist())
    assert np.allclose(last["basicMass"], f.mass[last["nodeIndex"]], rtol=1e-15)
    for name in ("diskMassStellar", "diskAbundancesGasMetals", "hotHaloMass", "blackHoleMass", "spheroidMassStellar"):
        assert name in last


def test_halo_mass_interpolates_along_primary_branches(evolved):
    """A primary progenitor's halo grows by its parent's unresolved mass (the
    parent's mass beyond all its progenitors'), linearly in time, as the
    reference's dmoInterpolate operator has it; secondaries keep theirs."""
    _, f, _, _, _, _ = evolved
    prim = [i for i in range(f.n) if f.parent[i] >= 0 and f.child_first[f.parent[i]] == i and
            f.time[f.parent[i]] > f.time[i] and f.child_count[f.parent[i]] > 1]
    i = prim[0]
    p = f.parent[i]
    unresolved = f.mass[p] - f.mass[f.child_first[p]:f.child_first[p] + f.child_count[p]].sum()
    assert unresolved > 0.0
    mid = 0.5 * (f.time[i] + f.time[p])
    assert output.halo_mass(f, [i], f.time[i])[0] == f.mass[i]
    assert abs(output.halo_mass(f, [i], mid)[0] - (f.mass[i] + 0.5 * unresolved)) < 1e-9 * f.mass[p]
    assert abs(output.halo_mass(f, [i], f.time[p])[0] - (f.mass[p] - (f.mass[p] - f.mass[i] - unresolved))) < \
        1e-9 * f.mass[p]
    secondary = [i for i in range(f.n) if f.parent[i] >= 0 and f.child_first[f.parent[i]] != i]
    if secondary:
        s = secondary[0]
        assert output.halo_mass(f, [s], f.time[s])[0] == f.mass[s]


def test_rejects_bad_snapshots(tmp_path, evolved):
    params, f, times, snap, node, outputs = evolved
    with pytest.raises(ValueError):
        output.write(tmp_path / "a.npz", params, f, times[::-1], snap, node, outputs)
    bad = outputs.copy()
    bad[0] = len(times)
    with pytest.raises(ValueError):
        output.write(tmp_path / "b.npz", params, f, times, snap, node, bad)
    with pytest.raises(ValueError):
        output.write(tmp_path / "c.npz", params, f, times, snap[:, :-1], node, outputs)
