"""The cooling surrogate held to the per-halo final-mass bar.

The target of the surrogate form: final stellar and cold-gas masses within
1e-3 relative of the FP64 oracle, halo by halo.  On the whole 65,536-halo
isolated-step batch (the benchmark's), these tests
  * check that the FP32-rate form with the table meets that bar;
  * choose the error-map gate of the surrogate as the benchmark does (the
    loosest gate at which 99.5% of the well-conditioned halos meet the bar;
    none when only the table does) and hold that form to the bar and, for
    every final mass and metal mass, to ten times the ODE tolerance in the
    solver's mixed norm (oracle/compare.py);
  * pin the precision of Lambda that the bar needs, from the oracle alone.
A halo is ill-conditioned when its oracle masses move by more than 1e-3
under a 10% change of the tolerance or a 1e-4 dex change of Lambda; such
halos must lie within twice that movement instead.
"""

import numpy as np
import pytest

from galacticus_gb300 import surrogate, workloads

pytestmark = pytest.mark.gpu

GATES = (0.01, 0.003, 0.001, 0.0003, 0.0001)


@pytest.fixture(scope="module")
def halos(table, oracle_mod):
    from oracle import compare
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=65536, seed=2)
    ref = oracle_mod.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step)[0]
    movement, sensitivity = compare.conditioning(oracle_mod, params, table, batch, ref)
    return params, batch, ref, movement, sensitivity


def evolve(ev, batch):
    g = batch.copy()
    status = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True)
    assert np.all(status == 0)
    return g.state


def test_table_form_meets_the_bar(table, halos):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params, batch, ref, movement, _ = halos
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32")
    bar = compare.bar_shares(evolve(ev, batch), ref, movement)
    ev.close()
    assert bar["min_conditioned"] >= 0.995, bar
    assert bar["ill_conditioned"] < 0.05, bar


def test_surrogate_form_at_the_chosen_gate(trained, table, halos):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params, batch, ref, movement, sensitivity = halos
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32")
    states = {}

    def run(gate):
        if gate is None:
            trained.uninstall(ev)
            states[gate] = evolve(ev, batch)
            return states[gate], 0.0
        trained.build_error_map(table, tolerance=gate)
        trained.install(ev)
        a = surrogate.stats(ev)
        states[gate] = evolve(ev, batch)
        b = surrogate.stats(ev)
        return states[gate], (b[0] - a[0]) / max(1, (b[0] - a[0]) + (b[1] - a[1]))

    chosen, results = compare.select_gate(run, ref, movement, GATES + (None,))
    ev.close()
    # The table alone always meets the bar, so a gate (or the table) is chosen.
    assert results[None]["meets_bar"]
    rec = results[chosen]
    assert rec["meets_bar"] and rec["min_conditioned"] >= 0.995
    # Every final mass and metal mass of the chosen form: within ten times
    # the tolerance, or (ill-conditioned values) within twice the oracle's
    # own movement beyond it.
    state = states[chosen]
    ratio = compare.parity_ratio(state, ref, batch.state, batch.param, params)
    bound = compare.parity_bound(ref, batch.state, batch.param, params)
    ok = (ratio <= 1.0) | (np.abs(state - ref) <= bound + 2.0 * sensitivity)
    assert np.all(ok), np.argwhere(~ok)[:5]
    # A looser gate than the chosen one never meets the bar (the choice is
    # the loosest that does).
    for gate in GATES:
        if chosen is not None and gate <= chosen:
            break
        assert not results[gate]["meets_bar"]


def test_lambda_precision_the_bar_needs(table, halos, oracle_mod):
    """From the oracle alone: how precisely Lambda must be known for the
    bar.  A systematic error of 3e-4 dex (0.07%) in every cooling rate
    already breaks it on the well-conditioned halos, and one of 1e-3 dex
    for more than half of them; at 1e-4 dex 95% of all halos still meet it.
    A network used in a halo's cells shifts that halo's Lambda by about its
    deployed error there, so the gate that meets the bar lies at or below
    1e-4 dex."""
    from oracle import compare
    params, batch, ref, movement, _ = halos
    bars = {}
    for dex in (1e-4, 3e-4, 1e-3):
        moved = oracle_mod.evolve_batch(params, compare.perturbed_table(table, dex), batch.state, batch.param,
                                        batch.t_start, batch.t_end, batch.step)[0]
        bars[dex] = compare.bar_shares(moved, ref, movement)
    assert bars[1e-4]["min_all"] >= 0.95
    assert bars[3e-4]["min_conditioned"] < 0.995
    assert bars[1e-3]["min_conditioned"] < 0.5
