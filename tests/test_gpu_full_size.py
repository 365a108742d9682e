"""Full-size checks of the batched isolated-halo step.

At the benchmark's size (65,536 halos, seed 2) the plain form is compared with
the oracle halo by halo.  At 1,048,576 halos, sixteen times that, a
size-independent property is checked in every form instead: mass
conservation.  Every node operator moves mass between reservoirs except
black-hole accretion, which keeps 1 - eps_rad - eps_jet of what it removes
from the spheroid gas and the hot halo, so

    sum of the seven masses + eps / (1 - eps) * M_BH

is constant along the exact solution; an embedded Runge-Kutta step preserves
a linear invariant of its right-hand side up to rounding, so the final states
keep it to FP64 rounding in the FP64 form (the oracle: 6e-16) and to the FP32
rounding of the rates' increments in the FP32-rate forms.
"""

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

MASSES = [_abi.Y_HOT_MASS, _abi.Y_OUTFLOWED_MASS, _abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS,
          _abi.Y_SPHEROID_STARS, _abi.Y_BLACK_HOLE]


def invariant(params, state):
    eps = params.bh_efficiency_radiative + params.bh_efficiency_jet
    return state[MASSES].sum(axis=0) + eps / (1.0 - eps) * state[_abi.Y_BLACK_HOLE]


def test_benchmark_batch_parity(table, oracle_mod):
    from oracle import compare
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=65536, seed=2)
    ev = MergerTreeNodeEvolverStandard(params=params, table=table)
    gpu = batch.copy()
    status = ev.evolve(gpu.state, gpu.param, gpu.t_start, gpu.t_end, gpu.step, return_status=True)
    ev.close()
    ref, _, ref_status, _ = oracle_mod.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                    batch.step)
    assert np.all(status == 0) and np.all(ref_status == 0)
    ratio = compare.parity_ratio(gpu.state, ref, batch.state, batch.param, params)
    assert ratio.max() <= 1.0, f"worst parity ratio {ratio.max():.3g}"


@pytest.mark.parametrize("form,bound", [("plain", 1e-12), ("fast", 1e-5), ("surrogate", 1e-5)])
def test_mass_conservation_at_one_million_halos(table, trained, form, bound):
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=1 << 20, seed=2)
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp64" if form == "plain" else "fp32")
    if form == "surrogate":
        trained.install(ev)  # the network with its own error map (the invariant holds at any gate)
    gpu = batch.copy()
    status = ev.evolve(gpu.state, gpu.param, gpu.t_start, gpu.t_end, gpu.step, return_status=True)
    ev.close()
    assert np.all(status == 0)
    assert np.all(np.isfinite(gpu.state))
    before, after = invariant(params, batch.state), invariant(params, gpu.state)
    rel = np.abs(after - before) / before
    assert rel.max() < bound, f"{form}: worst relative change of the mass invariant {rel.max():.3g}"
    # The halos did evolve: gas cooled onto the disks and formed stars.
    assert np.mean(gpu.state[_abi.Y_DISK_STARS] > 0.0) > 0.5
