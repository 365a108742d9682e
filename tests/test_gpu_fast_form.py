"""The fast form (FP32 rates; FP64 state, error norm and step control)
against the FP64 oracle: the same parity bound as the plain form (ten times
the ODE tolerance in the solver's mixed norm), and final stellar and cold-gas
masses within 1e-3 relative of the oracle for (almost) every halo."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fast(table):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=workloads.isolated_params(), table=table, ratePrecision="fp32")
    yield ev
    ev.close()


@pytest.fixture(scope="module")
def reference(table, oracle_mod):
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=8192, seed=2)
    ref, ref_step, ref_status, ref_counters = oracle_mod.evolve_batch(params, table, batch.state, batch.param,
                                                                      batch.t_start, batch.t_end, batch.step)
    # How far the oracle's own answer moves under an admissible change of the
    # integration (relative tolerance x0.9 and x1.1): the conditioning of
    # each value at the working tolerance.
    moved = []
    for factor in (0.9, 1.1):
        q = workloads.isolated_params(tolerance_relative=1e-3 * factor)
        moved.append(oracle_mod.evolve_batch(q, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                             batch.step)[0])
    sensitivity = np.maximum(np.abs(moved[0] - ref), np.abs(moved[1] - ref))
    return batch, ref, ref_status, ref_counters, sensitivity


def test_fast_form_parity(fast, reference):
    """Every final mass and metal mass within ten times the ODE tolerance of
    the oracle -- or, on the few ill-conditioned halos whose oracle answer
    itself moves by more than that when the tolerance changes by 10%, within
    twice that movement."""
    from oracle import compare
    batch, ref, ref_status, ref_counters, sensitivity = reference
    g = batch.copy()
    status, counters = fast.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True, counters=True)
    assert np.all(status == 0) and np.all(ref_status == 0)
    ratio = compare.parity_ratio(g.state, ref, batch.state, batch.param, fast.params)
    within = ratio <= 1.0
    bound = compare.parity_bound(ref, batch.state, batch.param, fast.params)
    conditioned = np.abs(g.state - ref) <= bound + 2.0 * sensitivity
    bad = np.argwhere(~(within | conditioned))
    assert len(bad) == 0, [(int(v), int(i), float(g.state[v, i]), float(ref[v, i]), float(sensitivity[v, i]))
                           for v, i in bad[:5]]
    assert np.mean(np.all(within, axis=0)) > 0.995, f"halos within 10x tolerance: {np.mean(np.all(within, axis=0)):.5f}"
    # FP32 rates move the step sequence only at the rounding level of the
    # error estimate: accepted-step counts agree within one step nearly everywhere.
    assert np.mean(np.abs(counters[0].astype(int) - ref_counters[0].astype(int)) <= 1) > 0.99
    for idx in (_abi.Y_DISK_STARS, _abi.Y_DISK_GAS):
        big = ref[idx] > 1e6
        rel = np.abs(g.state[idx][big] / ref[idx][big] - 1.0)
        assert np.median(rel) < 1e-5, f"median {np.median(rel):.2e}"
        assert np.mean(rel < 1e-3) > 0.998, f"share within 1e-3: {np.mean(rel < 1e-3):.5f}"


@pytest.mark.parametrize("n", [1, 33, 1000])
def test_fast_form_ragged_sizes(fast, table, oracle_mod, n):
    from oracle import compare
    batch = workloads.isolated_halos(n=n, seed=11)
    g = batch.copy()
    status = fast.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True)
    ref, _, ref_status, _ = oracle_mod.evolve_batch(fast.params, table, batch.state, batch.param, batch.t_start,
                                                    batch.t_end, batch.step)
    assert np.all(status == ref_status)
    assert compare.parity_ratio(g.state, ref, batch.state, batch.param, fast.params).max() <= 1.0


def test_fast_form_launch_shapes(fast):
    """Blocks per SM and grid size never change a result (same kernel
    binary); the block-size instantiations are compiled separately and may
    contract FP32 multiply-adds differently, so they agree to rounding."""
    batch = workloads.isolated_halos(n=3000, seed=9)
    outs = {}
    for threads, blocks in [(128, 1), (128, 2), (256, 1), (512, 1)]:
        fast.set_launch(threads, blocks)
        g = batch.copy()
        fast.evolve(g.state, g.param, g.t_start, g.t_end, g.step)
        outs[(threads, blocks)] = g.state
    fast.set_launch(128, 1)
    np.testing.assert_array_equal(outs[(128, 2)], outs[(128, 1)])
    for key in [(256, 1), (512, 1)]:
        np.testing.assert_allclose(outs[key], outs[(128, 1)], rtol=1e-9, atol=0.0)


def test_rate_precision_switch(fast):
    assert fast.lib.gal_gpu_get_rate_precision(fast.ctx) == _abi.RATES_FP32
    with pytest.raises(KeyError):
        fast.set_rate_precision("fp16")
    assert fast.lib.gal_gpu_set_rate_precision(fast.ctx, 7) == _abi.ERR_ARGUMENT
    assert fast.lib.gal_gpu_get_rate_precision(fast.ctx) == _abi.RATES_FP32
