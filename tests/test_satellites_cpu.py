"""Satellites in the merger forests, on the CPU: the merging time against a
restatement of Jiang et al. (2008) on a Benson (2005) orbit
(satellites/merging/timescale/Jiang2008.F90, satellites/merging/
virial_orbits/Benson2005.F90), the trees the builder makes with satellite
phases, and the oracle's evolution of them (baryons conserved over each
tree's roots)."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, forest, output, workloads


@pytest.fixture(scope="module")
def params():
    return workloads.isolated_params()


@pytest.fixture(scope="module")
def pair(params):
    """The same trees without and with satellites (the orbits are drawn after
    the trees, so the trees themselves are the same)."""
    kw = dict(n_trees=24, seed=3, root_mass_min=1e10, root_mass_max=1e12, mass_resolution=1e8)
    return (forest.build(params, **kw),
            forest.build(params, satellites=forest.SATELLITES_JIANG2008, **kw))


def jiang2008(params, m_host, m_sat, t, ur, ut, multiplier):
    """The merging time restated from the paper's fit and the orbit's
    equivalent circular radius in an isothermal host (point mass outside
    r_vir), with the host's virial scales from the Bryan & Norman (1998)
    contrast."""
    cos = workloads.Cosmology(params.omega_matter, params.omega_dark_energy, params.omega_baryon,
                              params.hubble_constant)
    r, v = cos.virial(m_host, max(float(cos.redshift(t)), 0.0))
    tdyn = r / v * workloads.MPC_PER_KM_PER_S_TO_GYR
    mu = m_host / (m_host + m_sat)
    energy = -1.0 + 0.5 * mu * (ur ** 2 + ut ** 2)
    if energy >= 0.0:
        return -1.0
    if energy <= -0.5:
        rc = np.exp(energy + 0.5)
        circularity = ut / rc
    else:
        rc = -0.5 / energy
        circularity = ut / np.sqrt(rc)
    q = m_host / m_sat
    return multiplier * tdyn * np.sqrt(rc) * (0.94 * circularity ** 0.60 + 0.60) / (2.0 * 0.43) * q / np.log1p(q)


@pytest.mark.parametrize("m_host,m_sat,z,ur,ut", [
    (1e12, 1e11, 0.5, 0.9, 0.7),   # a typical bound orbit, inside the isothermal part
    (1e11, 1e9, 2.0, 0.3, 1.0),    # nearly circular
    (3e12, 3e11, 0.0, 1.1, 0.6),   # energy above -1/2: the point-mass part
    (1e12, 9e11, 1.0, 0.5, 0.5),   # a near-equal-mass merger
])
def test_merging_time_matches_jiang2008(params, m_host, m_sat, z, ur, ut):
    t = forest.satellite_merging_time(params, 1.0, 1.0, 1.0, 0.0, 1.0)  # warm the library declarations
    assert t > 0.0
    cos = workloads.Cosmology(params.omega_matter, params.omega_dark_energy, params.omega_baryon,
                              params.hubble_constant)
    tt = float(cos.time(z))
    got = forest.satellite_merging_time(params, m_host, m_sat, tt, ur, ut, 0.75)
    want = jiang2008(params, m_host, m_sat, tt, ur, ut, 0.75)
    assert got == pytest.approx(want, rel=1e-12)
    # The fit's scalings: linear in the multiplier, q/ln(1+q) in the mass ratio.
    assert forest.satellite_merging_time(params, m_host, m_sat, tt, ur, ut, 1.5) == pytest.approx(2.0 * got, rel=1e-14)


def test_unbound_orbits_never_merge(params):
    assert forest.satellite_merging_time(params, 1e12, 1e11, 5.0, 2.0, 2.0, 0.75) < 0.0


def test_satellite_trees(pair):
    """Each secondary progenitor becomes a satellite phase whose host at
    infall is the node it fell into; it merges later, into a piece of the
    host's line that starts at the merging time, whose primary progenitor
    is the line before the merger and whose halo mass continues that line;
    or it outlives the tree as a root of its own."""
    base, sat = pair
    n_secondary = int(np.sum(np.maximum(base.child_count - 1, 0)))
    host = sat.satellite_host
    phases = np.flatnonzero(host >= 0)
    assert len(phases) > 0.9 * n_secondary  # a few merge at once (zero time)
    assert len(phases) <= n_secondary
    # The layout: parents later, progenitors contiguous with the primary first.
    for i in range(sat.n):
        p = sat.parent[i]
        if p >= 0:
            assert sat.time[p] > sat.time[i]
            assert sat.child_first[p] <= i < sat.child_first[p] + sat.child_count[p]
        assert sat.tree[i] == sat.tree[sat.child_first[i]] or sat.child_count[i] == 0
    # A phase: the infalling halo as its only progenitor, the host's time and tree.
    for s in phases:
        assert sat.child_count[s] == 1
        assert sat.time[s] == sat.time[host[s]]
        assert sat.tree[s] == sat.tree[host[s]]
        assert sat.mass[s] == sat.mass[sat.child_first[s]]
        p = sat.parent[s]
        if p >= 0 and sat.child_first[p] != s:
            # Merged: the piece from the merger on continues its primary's mass line.
            c0 = sat.child_first[p]
            assert host[c0] < 0
            line = output.halo_mass(sat, [c0], sat.time[p])[0]
            assert abs(sat.mass[p] - line) <= 1e-12 * sat.mass[p] or sat.child_count[c0] == 0
    # The leaves (the halos the trees start from) are the same.
    leaves = lambda f: np.sort(f.mass[f.child_count == 0])
    np.testing.assert_array_equal(leaves(base), leaves(sat))
    # Satellites merge later than they fall in: merging times of order of
    # the host's dynamical time times the mass ratio.
    merged = [s for s in phases if sat.parent[s] >= 0 and host[sat.parent[s]] < 0]
    delay = np.array([sat.time[sat.parent[s]] - sat.time[s] for s in merged])
    assert np.all(delay > 0.0)
    assert 0.1 < np.median(delay) < 20.0


def test_oracle_conserves_baryons_with_satellites(pair, params, table, oracle_mod):
    """Every tree ends with f_b M_root in baryons over its roots -- the
    central's and those of satellites that outlive the tree -- less what
    black-hole accretion radiates (the reference's mass-conservation bar,
    1e-3; testSuite/test-mass-conservation-standard.py:82)."""
    _, f = pair
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    state, status, counters, snaps = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)
    assert np.all(status == 0)
    roots = np.flatnonzero(f.parent < 0)
    masses = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
              _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]
    baryons = np.bincount(f.tree[roots], weights=state[masses][:, roots].sum(axis=0), minlength=f.n_trees)
    main = np.array([roots[(f.tree[roots] == t)][np.argmax(f.mass[roots][f.tree[roots] == t])]
                     for t in range(f.n_trees)])
    fb = params.omega_baryon / params.omega_matter
    rel = np.abs(baryons / (fb * f.mass[main]) - 1.0)
    assert rel.max() < 1e-3, rel.max()
    # Satellite phases evolved (they form stars on their own) and the
    # outputs mark them as satellites.
    phases = np.flatnonzero(f.satellite_host >= 0)
    assert counters[0][phases].sum() > 0
    first, m = oracle_mod.forest_snapshots(f, times)
    node = np.repeat(np.arange(f.n), np.diff(np.append(first, m)))
    out_idx = np.zeros(m, np.int64)
    for i in range(f.n):
        k0 = first[i]
        k1 = first[i + 1] if i + 1 < f.n else m
        t_in = [k for k, t in enumerate(times) if (t == f.time[i] and (f.parent[i] < 0 or f.time[i] < f.time[f.parent[i]]))
                or (f.parent[i] >= 0 and f.time[i] < t < f.time[f.parent[i]])]
        out_idx[k0:k1] = t_in
    d = output.layout(params, f, times, snaps, node, out_idx)
    iso = np.concatenate([d[f"Outputs/Output{k + 1}/nodeData/nodeIsIsolated"] for k in range(len(times))])
    idx = np.concatenate([d[f"Outputs/Output{k + 1}/nodeData/nodeIndex"] for k in range(len(times))])
    assert np.all(iso[f.satellite_host[idx] >= 0] == 0) and np.all(iso[f.satellite_host[idx] < 0] == 1)
    assert np.any(iso == 0)


def benson2005_density(ur, ut):
    """The Benson (2005) fit to the distribution of infall velocities (units
    of the host's virial velocity), unnormalised."""
    a = [3.90052, 2.47973, 10.2373, 0.683922, 0.353953, 1.07716, 0.509837, 0.206204, 0.314641]
    b1 = a[2] * np.exp(-a[3] * (ut - a[4]) ** 2)
    b2 = a[5] * np.exp(-a[6] * (ut - a[7]) ** 2)
    return a[0] * ut * np.exp(-a[1] * (ut - a[8]) ** 2) * np.exp(-b1 * (ur - b2) ** 2)


@pytest.mark.parametrize("mu", [1.0, 0.6])
def test_orbit_sampler_follows_benson2005(mu):
    """The builder's orbits against the published distribution restricted to
    bound orbits (mu (ur^2 + ut^2)/2 < 1 - 1e-4), integrated on a grid: the
    means and spreads of both velocities and the share of each quadrant of
    the velocity plane."""
    ur, ut = forest.satellite_orbits(400_000, mu=mu, seed=11)
    assert np.all(0.5 * mu * (ur ** 2 + ut ** 2) < 1.0 - 1e-4)
    assert np.all((ur >= 0) & (ur <= 3) & (ut >= 0) & (ut <= 3))
    g = (np.arange(1200) + 0.5) * 3.0 / 1200
    R, T = np.meshgrid(g, g, indexing="ij")
    w = benson2005_density(R, T) * (0.5 * mu * (R ** 2 + T ** 2) < 1.0 - 1e-4)
    w /= w.sum()
    for sample, grid in ((ur, R), (ut, T)):
        mean = (w * grid).sum()
        sd = np.sqrt((w * (grid - mean) ** 2).sum())
        assert abs(sample.mean() - mean) < 4 * sd / np.sqrt(len(sample)) + 1e-3
        assert abs(sample.std() - sd) < 0.01 * sd
    for r0 in (0.5, 1.0):
        for t0 in (0.5, 1.0):
            share = np.mean((ur < r0) & (ut < t0))
            assert abs(share - w[(R < r0) & (T < t0)].sum()) < 0.005
