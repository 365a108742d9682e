"""Krumholz (2009) disk star formation on the GPU against the oracle.

The reference's default disk star-formation rate integrates the Krumholz,
McKee & Tumlinson (2009) surface density law over the exponential gas disk
(star_formation/rates/disks/integrated_surface_density.F90:131-190,
star_formation/rate_surface_density/disks/Krumholz2009.F90:312-620) with
GSL's adaptive Gauss-Kronrod quadrature.  The GPU forms run the same
algorithm per lane (galnode_krumholz.cuh); here they are checked against the
oracle on halos with gaseous disks (workloads.galaxy_halos) and on a small
forest whose gas carries metals, with the bound of the other parity tests:
ten times the ODE tolerance in the solver's mixed norm (oracle/compare.py),
and for the FP32-rate form the conditioning exemption of the fast-form test.
"""

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu


def krumholz_params(tolerance_relative=1.0e-3):
    p = workloads.isolated_params(tolerance_relative)
    p.sf_disk_rate = _abi.SF_RATE_KRUMHOLZ2009
    return p


@pytest.fixture(scope="module")
def reference(table, oracle_mod):
    params = krumholz_params()
    batch = workloads.galaxy_halos(n=4096, seed=12)
    ref, _, ref_status, ref_counters = oracle_mod.evolve_batch(params, table, batch.state, batch.param, batch.t_start,
                                                               batch.t_end, batch.step)
    moved = [oracle_mod.evolve_batch(krumholz_params(1e-3 * f), table, batch.state, batch.param, batch.t_start,
                                     batch.t_end, batch.step)[0] for f in (0.9, 1.1)]
    sensitivity = np.maximum(np.abs(moved[0] - ref), np.abs(moved[1] - ref))
    return params, batch, ref, ref_status, ref_counters, sensitivity


def test_the_rate_class_matters(table, reference, oracle_mod):
    """The batch forms stars at rates that differ from the timescale class."""
    params, batch, ref, ref_status, _, _ = reference
    assert np.all(ref_status == 0)
    timescale = oracle_mod.evolve_batch(workloads.isolated_params(), table, batch.state, batch.param, batch.t_start,
                                        batch.t_end, batch.step)[0]
    change = np.abs(ref[_abi.Y_DISK_STARS] / timescale[_abi.Y_DISK_STARS] - 1.0)
    assert np.mean(change > 1e-2) > 0.25


@pytest.mark.parametrize("rates", ["fp64", "fp32"])
def test_krumholz_batch_parity(table, reference, rates):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params, batch, ref, ref_status, ref_counters, sensitivity = reference
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
    assert ev.get_launch()[0] == 128
    g = batch.copy()
    status, counters = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True, counters=True)
    ev.close()
    assert np.all(status == 0)
    ratio = compare.parity_ratio(g.state, ref, batch.state, batch.param, params)
    if rates == "fp64":
        assert ratio.max() <= 1.0, f"worst parity ratio {ratio.max():.3g}"
        assert np.mean(counters[0] == ref_counters[0]) > 0.99
    else:
        bound = compare.parity_bound(ref, batch.state, batch.param, params)
        ok = (ratio <= 1.0) | (np.abs(g.state - ref) <= bound + 2.0 * sensitivity)
        assert np.all(ok), np.argwhere(~ok)[:5]
        assert np.mean(np.all(ratio <= 1.0, axis=0)) > 0.995


@pytest.mark.parametrize("rates", ["fp64", "fp32"])
def test_krumholz_forest_parity(table, oracle_mod, rates):
    """A forest of 8 trees whose hot gas carries metals, so that its disks
    form stars, in one graph launch."""
    from galacticus_gb300 import forest
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params = krumholz_params()
    f = forest.build(params, n_trees=8, seed=3, root_mass_min=1e10, root_mass_max=1e11)
    state0 = forest.initial_state(params, f)
    state0[_abi.Y_HOT_METALS] = 1e-3 * state0[_abi.Y_HOT_MASS]
    times = forest.output_times(params)
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
    fe = forest.ForestEvolver(ev, f, state0, times)
    fe.evolve()
    state, status = fe.results(snapshots=False)[:2]
    fe.close()
    ev.close()
    ref, ref_status = oracle_mod.evolve_forest(params, table, f, state0, times, brent=False)[:2]
    assert np.all(status == 0) and np.all(ref_status == 0)
    roots = f.parent < 0
    assert np.all(ref[_abi.Y_DISK_STARS, roots] + ref[_abi.Y_SPHEROID_STARS, roots] > 0.0)
    param = np.zeros((_abi.NP, f.n))
    param[_abi.P_MASS] = f.mass
    within = np.abs(state - ref) <= compare.parity_bound(ref, ref, param, params)
    assert np.mean(np.all(within, axis=0)) > (0.999 if rates == "fp64" else 0.99)


def test_krumholz_needs_a_form_without_the_surrogate(table, trained):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=krumholz_params(), table=table, ratePrecision="fp32")
    with pytest.raises(RuntimeError):
        trained.install(ev)
    ev.close()
