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
def test_evolution_with_surrogate_against_the_table(trained, table, oracle_mod, rates):
    """The surrogate forms at the configuration's gate (0.01 dex) against
    the same rates with the table (the method without the network), both
    against the FP64 oracle on the isolated-halo step: the network takes
    most cooling evaluations off the table, and the price is accuracy --
    per halo, the table form keeps more halos' stellar and cold-gas masses
    within 1e-3 of the oracle than the surrogate form does (the per-halo
    bar itself is held in test_surrogate_bar.py)."""
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import compare
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=8192, seed=2)
    ref, _, ref_status, _ = oracle_mod.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                    batch.step)
    out = {}
    for name in ("table", "network"):
        ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
        if name == "network":
            trained.build_error_map(table, tolerance=0.01)
            trained.install(ev)
        g = batch.copy()
        status = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True)
        if name == "network":
            network, tab = surrogate.stats(ev)
        ev.close()
        assert np.all(status == 0)
        out[name] = compare.bar_shares(g.state, ref, np.zeros(batch.n))
    assert network > 0.5 * (network + tab), f"network served {network} of {network + tab}"
    assert out["table"]["min_all"] >= 0.995
    assert out["network"]["min_all"] < out["table"]["min_all"]
    # Still a close approximation: the median halo within 1e-3.
    errs = compare.relative_mass_errors(g.state, ref)
    for name, (rel, big) in errs.items():
        assert np.median(rel[big]) < 1e-3, f"{name}: median rel error {np.median(rel[big]):.2e}"


def test_split_launch_matches_one_kernel(trained, table):
    """The surrogate form's split launch (the nodes the network may serve on
    the network kernel, the others on the kernel without it, at once) against
    one network kernel over all nodes: every node succeeds, nearly every node
    is bit for bit the same (a node may use the network in the one-kernel
    launch once its metallicity reaches a served cell), and the evaluation
    counts add up to the RHS evaluations."""
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=8192, seed=2)
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32")
    trained.build_error_map(table, tolerance=0.003)
    trained.install(ev)
    out = {}
    for split in (True, False):
        surrogate.set_split(ev, split)
        a = surrogate.stats(ev)
        g = batch.copy()
        status, counters = ev.evolve(g.state, g.param, g.t_start, g.t_end, g.step, return_status=True, counters=True)
        b = surrogate.stats(ev)
        assert np.all(status == 0)
        out[split] = (g.state, counters, (b[0] - a[0], b[1] - a[1]))
    ev.close()
    same = np.all(out[True][0] == out[False][0], axis=0)
    assert same.mean() > 0.95
    # Every node was taken exactly once from the split lists (the table list
    # is filled from both ends: long integrations at its front).
    assert np.all(out[True][1][2] > 0)
    np.testing.assert_allclose(out[True][1][0].sum(), out[False][1][0].sum(), rtol=0.01)
    for split in (True, False):
        net, tab = out[split][2]
        assert net + tab == int(out[split][1][2].sum())
        assert net > 0.2 * (net + tab)
