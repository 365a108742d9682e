"""Interrupts on the GPU against the oracle (gal_gpu_evolve_batch_interrupt).

mergerTreeNodeEvolver%evolve returns `interrupted` and `functionInterrupt`
(node_evolver/_class.F90:41-57; standard.F90:729-737): a node whose rates
reach a component it does not have stops at the earliest such evaluation
(odeSolverInterrupt, numerical/ODE_solver/error_codes.F90:33), and the host
creates the component and evolves it on.  Here halos without a disk start to
cool during the step (workloads.disk_creation_halos): cooling into the
missing disk interrupts them at the start, part way through, or never.  The
GPU's statuses, tasks, interrupt times and states must match the oracle's,
the states within ten times the ODE tolerance (oracle/compare.py), and the
resumed evolution after creating the disk too.
"""

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def evolver(table):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=workloads.isolated_params(), table=table)
    yield ev
    ev.close()


def run_gpu(ev, batch, comps, t_start=None, state=None, step=None):
    g = batch.copy()
    if state is not None:
        g.state[:] = state
    if step is not None:
        g.step[:] = step
    t0 = batch.t_start if t_start is None else t_start
    status, reached, task, cnt = ev.evolve_interruptible(g.state, g.param, t0, g.t_end, g.step, comps, counters=True)
    return g.state, g.step, status, reached, task, cnt


def test_disk_creation_interrupts_match_oracle(evolver, table, oracle_mod):
    from oracle import compare
    params = evolver.params
    batch, comps = workloads.disk_creation_halos(n=8192)
    st, step, status, reached, task, cnt = run_gpu(evolver, batch, comps)
    ref, ref_step, ref_status, ref_cnt, ref_reached, ref_task = oracle_mod.evolve_batch_interrupt(
        params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, comps)
    interrupted = ref_status == _abi.STATUS_INTERRUPTED
    inside = interrupted & (ref_reached > batch.t_start) & (ref_reached < batch.t_end)
    assert inside.sum() > 200 and (~interrupted).sum() > 200
    # Same outcome node by node (an interrupt found one stage earlier or
    # later is the same decision made at a rounding-level difference).
    assert np.mean(status == ref_status) > 0.999
    assert np.mean(task == ref_task) > 0.999
    same = status == ref_status
    # The interrupt time is a stage time t + c h of the step sequence: equal
    # to rounding where the step sequences agree.
    span = batch.t_end - batch.t_start
    dt = np.abs(reached - ref_reached) / span
    assert np.mean(dt[same] < 1e-12) > 0.99
    assert np.all(step[same & interrupted] == -1.0)
    # States at the time reached.
    ratio = compare.parity_ratio(st, ref, batch.state, batch.param, params)
    close = np.all(ratio <= 1.0, axis=0)
    assert np.mean(close[same]) > 0.995
    assert np.all(st[[_abi.Y_DISK_GAS, _abi.Y_DISK_GAS_METALS, _abi.Y_DISK_STARS, _abi.Y_DISK_STARS_METALS]] == 0.0)


def test_resume_after_creating_the_disk(evolver, table, oracle_mod):
    """The host protocol on the GPU: create the disk of every interrupted
    node and evolve again from the time reached; all reach the end, within
    the bound of the oracle doing the same."""
    from oracle import compare
    params = evolver.params
    batch, comps = workloads.disk_creation_halos(n=4096, seed=23)
    st, step, status, reached, task, _ = run_gpu(evolver, batch, comps)
    comps2 = comps | np.where(task & _abi.INTERRUPT_CREATE_DISK, _abi.COMPONENT_DISK, 0).astype(np.int32)
    st2, _, status2, reached2, task2, _ = run_gpu(evolver, batch, comps2, t_start=reached, state=st, step=step)
    assert np.all(status2 == _abi.STATUS_SUCCESS) and np.all(task2 == 0)
    np.testing.assert_array_equal(reached2, batch.t_end)
    # The oracle, through the same two calls.
    r1 = oracle_mod.evolve_batch_interrupt(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                           batch.step, comps)
    c2 = comps | np.where(r1[5] & _abi.INTERRUPT_CREATE_DISK, _abi.COMPONENT_DISK, 0).astype(np.int32)
    r2 = oracle_mod.evolve_batch_interrupt(params, table, r1[0], batch.param, r1[4], batch.t_end, r1[1], c2)
    same = (status == r1[2]) & (task == r1[5])
    ratio = compare.parity_ratio(st2, r2[0], batch.state, batch.param, params)
    assert np.mean(np.all(ratio <= 1.0, axis=0)[same]) > 0.995


def test_no_missing_component_matches_the_plain_evolution(evolver, table):
    """With every component present the interrupt form is the plain
    evolution: nothing interrupts and the states agree within the bound."""
    from oracle import compare
    batch = workloads.galaxy_halos(n=4096, seed=12)
    comps = np.full(batch.n, _abi.COMPONENT_ALL, np.int32)
    st, _, status, reached, task, _ = run_gpu(evolver, batch, comps)
    g = batch.copy()
    plain = evolver.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True)
    assert np.all(status == 0) and np.all(plain == 0) and np.all(task == 0)
    np.testing.assert_array_equal(reached, batch.t_end)
    assert compare.parity_ratio(st, g.state, batch.state, batch.param, evolver.params).max() <= 1e-3


def test_interrupts_need_the_fp64_form(table):
    from galacticus_gb300.evolver import GalnodeError, MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=workloads.isolated_params(), table=table, ratePrecision="fp32")
    batch, comps = workloads.disk_creation_halos(n=8)
    with pytest.raises(GalnodeError):
        ev.evolve_interruptible(batch.state.copy(), batch.param, batch.t_start, batch.t_end, batch.step.copy(), comps)
    ev.close()
