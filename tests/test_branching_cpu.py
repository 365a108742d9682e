"""The GPU tree builder's branching, on the CPU: the oracle's restatement of
its walk with keyed per-branch streams (the GPU kernel's specification)
against the host builder, which draws each tree from one sequential stream.
The two differ only in where their random numbers come from, so on the
same roots their trees must agree in distribution: node counts, leaf mass
functions, the main branch's earliest mass.  The builder's tables exported
for the restatement are checked for their own invariants, and the GPU entry
point refuses a missing context without touching a GPU."""

import ctypes

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, workloads


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


SPEC = dict(seed=7, root_mass_min=1e11, root_mass_max=1e13, mass_resolution=1e9)


@pytest.fixture(scope="module")
def pair(params, oracle_mod):
    """800 host-built trees and the oracle's keyed trees on the same roots."""
    host = forest.build(params, n_trees=800, **SPEC)
    tables = forest.branch_tables(params, **{k: v for k, v in SPEC.items()})
    roots = host.mass[host.parent < 0]
    keyed = oracle_mod.grow_trees(tables, SPEC["seed"], roots)
    return host, keyed, tables


def _main_branch_end(mass, child_first, child_count, first, offset=0):
    """Mass of the earliest node of the main branch of the tree whose root
    is node `first` (child_first relative to `offset`)."""
    i = first
    while child_count[i] > 0:
        i = offset + child_first[i]
    return mass[i]


def test_branch_tables(pair):
    _, _, t = pair
    rows = t["sizes"][1]
    cdf = t["cdf"].reshape(rows, 96)
    lnq = t["ln_q"].reshape(rows, 96)
    split = t["rate"] > 0
    assert split.sum() > 0.9 * rows
    assert np.all(np.diff(cdf[split], axis=1) >= 0.0)
    np.testing.assert_allclose(cdf[split][:, -1], 1.0, rtol=1e-12)
    np.testing.assert_allclose(lnq[split][:, -1], np.log(0.5), rtol=1e-12)
    assert np.all(t["accretion"] >= 0.0)
    s_ln_m0, s_dln_m, r_ln_m0, r_dln_m, m_res, w_max, gamma2, acc1, acc2, w_root = t["meta"]
    assert r_ln_m0 == pytest.approx(np.log(m_res)) and m_res == SPEC["mass_resolution"]
    assert w_max > w_root > 1.6 and gamma2 == -0.01 and acc1 == acc2 == 0.1
    # sigma(M) decreases with mass.
    assert np.all(np.diff(t["ln_sigma"]) < 0.0)


def test_keyed_trees_are_valid(pair):
    _, (mass, w, parent, child_first, child_count, tree_first), t = pair
    m_res = t["meta"][4]
    n = len(mass)
    assert np.all(mass >= m_res)
    local = np.arange(n) - np.repeat(tree_first, np.diff(np.append(tree_first, n)))
    for i in np.flatnonzero(child_count > 0):
        g = i - local[i]
        kids = g + child_first[i] + np.arange(child_count[i])
        assert np.all(parent[kids] == local[i])
        assert np.all(w[kids] > w[i])
        assert mass[kids].sum() <= mass[i] * (1 + 1e-12)
        if child_count[i] == 2:
            assert mass[kids[0]] >= mass[kids[1]]


def test_keyed_trees_match_the_host_builder_in_distribution(pair):
    host, (mass, w, parent, child_first, child_count, tree_first), t = pair
    n_keyed, n_host = len(mass), host.n
    # Node counts: 800 trees of a few hundred nodes each.
    assert abs(n_keyed / n_host - 1.0) < 0.03, (n_keyed, n_host)
    # Leaf mass functions (log-mass histograms) agree within their Poisson errors.
    bins = np.linspace(np.log10(SPEC["mass_resolution"]), 13.0, 13)
    h_host = np.histogram(np.log10(host.mass[host.child_count == 0]), bins)[0]
    h_keyed = np.histogram(np.log10(mass[child_count == 0]), bins)[0]
    ok = (h_host + h_keyed) > 50
    chi2 = np.sum((h_host - h_keyed)[ok] ** 2 / (h_host + h_keyed)[ok])
    assert chi2 < 2.0 * ok.sum() + 10, (h_host, h_keyed)
    # The main branch's earliest mass over the root's, tree by tree on the
    # same roots: the same distribution (two-sample Kolmogorov-Smirnov).
    from scipy import stats
    roots = np.flatnonzero(host.parent < 0)
    f_host = np.array([_main_branch_end(host.mass, host.child_first, host.child_count, r) / host.mass[r]
                       for r in roots])
    f_keyed = np.array([_main_branch_end(mass, child_first, child_count, tree_first[k], tree_first[k]) /
                        mass[tree_first[k]] for k in range(len(roots))])
    assert stats.ks_2samp(f_host, f_keyed).pvalue > 1e-3
    assert abs(np.median(f_keyed) / np.median(f_host) - 1.0) < 0.15


def test_gpu_build_needs_a_context(params):
    lib = forest._declare(_abi.load_library())
    spec = forest._spec(2, 1, 1e11, 1e11, -0.9, 8.0, 1e9, forest.SATELLITES_NONE, 0.75)
    pch = forest.pch_params()
    out = ctypes.c_void_p(1)
    rc = lib.gal_gpu_forest_build(None, ctypes.byref(params), ctypes.byref(pch), ctypes.byref(spec), ctypes.byref(out))
    assert rc == _abi.ERR_ARGUMENT and not out.value


def test_walk_math_accuracy(oracle_mod):
    """The walk's FP32 ln and exp against numpy's FP64: ln to half an FP32
    ulp of e ln 2 plus the mantissa's truncation, exp to ~2 FP32 ulp (the
    rounded 2^(j/32) table entry and two products)."""
    rng = np.random.default_rng(1)
    x = np.exp(rng.uniform(np.log(1e-3), np.log(1e17), 100_000))
    y = rng.uniform(-20.0, 20.0, 100_000).astype(np.float32)
    lx, ey = oracle_mod.branch_math(x, y)
    err = np.abs(lx.astype(np.float64) - np.log(x))
    assert np.all(err <= 2.5e-7 + 6.5e-8 * np.abs(np.log(x))), err.max()
    assert np.max(np.abs(ey / np.exp(y.astype(np.float64)) - 1.0)) < 2.5e-7


def test_build_stats(params):
    """Where a host build's time went: every phase timed, none of them the
    GPU's, and the phases within the total."""
    f = forest.build(params, n_trees=64, seed=5, root_mass_min=1e10, root_mass_max=1e12,
                     satellites=forest.SATELLITES_JIANG2008)
    s = f.build_stats
    assert s["gpu_growth_s"] == 0.0 and s["download_renumber_s"] == 0.0 and s["generations"] == 0
    assert s["tables_s"] > 0.0 and s["per_tree_s"] > 0.0 and s["assembly_s"] > 0.0
    assert s["tables_s"] + s["per_tree_s"] + s["assembly_s"] <= s["total_s"] * (1 + 1e-9)
