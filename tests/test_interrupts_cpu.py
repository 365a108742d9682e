"""Interrupts in the oracle (the checker of gal_gpu_evolve_batch_interrupt).

The reference interrupts a node's integration when a rate reaches a
component the node does not have (node_evolver/standard.F90:895-945,
numerical/ODE_solver/solver.F90:608-620): the evolution stops at the
earliest such evaluation and reports its time and task.  These tests pin
the oracle's restatement on the CPU."""

import numpy as np

from galacticus_gb300 import _abi, workloads


def test_no_missing_component_means_no_interrupt(table, oracle_mod):
    """With every component present nothing interrupts, and the interrupt
    form (which evaluates f(t+h, y_new) on every attempt, as GSL's rkck)
    gives the plain evolution bit for bit."""
    params = workloads.isolated_params()
    batch = workloads.galaxy_halos(n=2048, seed=12)
    comps = np.full(batch.n, _abi.COMPONENT_ALL, np.int32)
    st, step, status, cnt, reached, task = oracle_mod.evolve_batch_interrupt(
        params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, comps)
    ref, ref_step, ref_status, ref_cnt = oracle_mod.evolve_batch(params, table, batch.state, batch.param,
                                                                 batch.t_start, batch.t_end, batch.step)
    np.testing.assert_array_equal(status, ref_status)
    np.testing.assert_array_equal(st, ref)
    np.testing.assert_array_equal(step, ref_step)
    np.testing.assert_array_equal(cnt[:2], ref_cnt[:2])
    assert np.all(task == 0) and np.all(reached == batch.t_end)


def test_disk_creation_interrupts(table, oracle_mod):
    params = workloads.isolated_params()
    batch, comps = workloads.disk_creation_halos(n=4096)
    st, step, status, cnt, reached, task = oracle_mod.evolve_batch_interrupt(
        params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, comps)
    interrupted = status == _abi.STATUS_INTERRUPTED
    assert set(np.unique(status)) <= {_abi.STATUS_SUCCESS, _abi.STATUS_INTERRUPTED}
    at_start = interrupted & (reached == batch.t_start)
    inside = interrupted & (reached > batch.t_start) & (reached < batch.t_end)
    # All three outcomes occur: cooling from the start, from part way, never.
    assert at_start.sum() > 100 and inside.sum() > 100 and (~interrupted).sum() > 100
    assert np.all(task[interrupted] == _abi.INTERRUPT_CREATE_DISK) and np.all(task[~interrupted] == 0)
    assert np.all(step[interrupted] == -1.0)
    np.testing.assert_array_equal(reached[~interrupted], batch.t_end[~interrupted])
    # No rate reaches the missing disk before the interrupt.
    disk = [_abi.Y_DISK_GAS, _abi.Y_DISK_GAS_METALS, _abi.Y_DISK_STARS, _abi.Y_DISK_STARS_METALS]
    assert np.all(st[disk] == 0.0)
    # Interrupted at the start: nothing moves.
    np.testing.assert_array_equal(st[:, at_start], batch.state[:, at_start])
    # Against the ordinary evolution (every component present): a node that
    # never interrupts is the same integration bit for bit, and did not
    # cool; a node that interrupts does cool in the ordinary evolution.
    comps_all = np.full(batch.n, _abi.COMPONENT_ALL, np.int32)
    ref = oracle_mod.evolve_batch_interrupt(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                            batch.step, comps_all)[0]
    np.testing.assert_array_equal(st[:, ~interrupted], ref[:, ~interrupted])
    assert np.all(ref[_abi.Y_DISK_GAS, ~interrupted] == 0.0)
    assert np.all(ref[_abi.Y_DISK_GAS, interrupted] > 0.0)


def test_resuming_after_creating_the_disk(table, oracle_mod):
    """The host protocol: create the component named by the task and evolve
    again from the time reached; every node then reaches the end."""
    params = workloads.isolated_params()
    batch, comps = workloads.disk_creation_halos(n=1024, seed=22)
    st, step, status, _, reached, task = oracle_mod.evolve_batch_interrupt(
        params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, comps)
    comps = comps | np.where(task & _abi.INTERRUPT_CREATE_DISK, _abi.COMPONENT_DISK, 0).astype(np.int32)
    st2, _, status2, _, reached2, task2 = oracle_mod.evolve_batch_interrupt(
        params, table, st, batch.param, reached, batch.t_end, step, comps)
    assert np.all(status2 == _abi.STATUS_SUCCESS) and np.all(task2 == 0)
    np.testing.assert_array_equal(reached2, batch.t_end)
    moved = status == _abi.STATUS_INTERRUPTED
    assert np.all(st2[_abi.Y_DISK_GAS, moved] > 0.0)
