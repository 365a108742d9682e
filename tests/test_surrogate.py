"""GPU checks of the learned cooling surrogate: gradients of the training
kernels against the FP64 CPU reference, tensor-core inference against FP32,
training, the error map, and evolution with the surrogate installed."""

import numpy as np
import pytest

from galacticus_gb300 import _abi, surrogate, workloads

pytestmark = pytest.mark.gpu


def test_training_gradients_match_cpu_oracle():
    from oracle import mlp_reference
    rng = np.random.default_rng(11)
    p = surrogate.init_params(11)
    x = rng.uniform(-1, 1, (256, 3)).astype(np.float32)
    y = rng.normal(size=256).astype(np.float32)
    loss, g = surrogate.gradient(p, x, y)
    ref_loss, ref_g = mlp_reference.loss_and_gradient(p, x, y)
    assert abs(loss / ref_loss - 1.0) < 1e-5
    # FP32 accumulation over 256 samples: relative to the gradient's scale.
    scale = np.abs(ref_g).max()
    assert np.abs(g - ref_g).max() < 1e-5 * scale


def test_training_converges(trained):
    h = trained.history
    assert h[-1, 1] < 0.02 * h[0, 1] or h[-1, 1] < 1e-4
    assert trained.rms_dex < 0.01, f"validation rms {trained.rms_dex:.4f} dex"


def test_tensor_core_inference_matches_fp32(trained, table):
    x, _ = surrogate.cooling_samples(table, 20000, seed=21)
    a = trained.predict(x, tensor_cores=True)
    b = trained.predict(x, tensor_cores=False)
    # Split-BF16 products (hi*hi + hi*lo + lo*hi) keep ~16 significant bits.
    assert np.abs(a - b).max() < 2e-3
    assert np.abs(a - b).mean() < 3e-4


def test_error_map_bounds_the_deployed_error(trained, table):
    x, y = surrogate.cooling_samples(table, 50000, seed=22)
    pred = trained.predict(x)
    it = ((x[:, 0] - trained.map_lo[0]) / trained.map_step[0]).astype(int).clip(0, trained.use_table.shape[0] - 1)
    iz = ((x[:, 1] - trained.map_lo[1]) / trained.map_step[1]).astype(int).clip(0, trained.use_table.shape[1] - 1)
    served = trained.use_table[it, iz] == 0
    assert served.mean() > 0.5
    assert np.abs(pred - y)[served].max() < 2 * trained.tolerance


@pytest.mark.parametrize("rates", ["fp64", "fp32"])
def test_evolution_with_surrogate(trained, table, oracle_mod, rates):
    """The surrogate forms against the FP64 oracle on the isolated-halo step,
    and what the network gains: the share of cooling evaluations it serves
    and its error against the untrained network it started from."""
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=8192, seed=2)
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
    trained.install(ev)
    g = batch.copy()
    status = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True)
    network, tab = surrogate.stats(ev)
    ev.close()
    assert np.all(status == 0)
    assert network > 0.5 * (network + tab), f"network served {network} of {network + tab}"
    ref, _, ref_status, _ = oracle_mod.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                    batch.step)
    for idx in (_abi.Y_DISK_STARS, _abi.Y_DISK_GAS):
        big = ref[idx] > 1e6
        rel = np.abs(g.state[idx][big] / ref[idx][big] - 1.0)
        assert np.median(rel) < 1e-3, f"median rel error {np.median(rel):.2e}"
    # The gain of training: the untrained network misses the table by far more.
    untrained = surrogate.CoolingSurrogate(surrogate.init_params(4), trained.in_mean, trained.in_scale, trained.y_mean,
                                           trained.y_scale)
    x, y = surrogate.cooling_samples(table, 20000, seed=23)
    assert np.abs(untrained.predict(x) - y).mean() > 50 * np.abs(trained.predict(x) - y).mean()
