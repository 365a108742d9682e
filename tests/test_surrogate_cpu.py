"""CPU checks of the surrogate's data and of its FP64 reference network."""

import numpy as np

from galacticus_gb300 import surrogate


def test_training_targets_follow_the_reference_interpolation(oracle_mod, table):
    """The vectorised sample generator reproduces the oracle's restatement of
    cieFileCoolingFunction (CIE_file.F90:238-317) point by point."""
    rng = np.random.default_rng(3)
    x = surrogate.DOMAIN_LO + (surrogate.DOMAIN_HI - surrogate.DOMAIN_LO) * rng.random((500, 3))
    x[::50, 1] = -12.0  # metallicities below the first non-zero row
    got = surrogate.cie_log10_lambda(table, x[:, 0], x[:, 1], x[:, 2])
    lib = oracle_mod.lib()
    ref = np.array([np.log10(lib.oracle_cooling_function(table.struct, 10 ** c, 10 ** a, 10 ** b)) for a, b, c in x])
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)


def test_reference_gradient_matches_finite_differences():
    from oracle import mlp_reference
    rng = np.random.default_rng(5)
    p = surrogate.init_params(9).astype(np.float64)
    x = rng.uniform(-1, 1, (40, 3))
    y = rng.normal(size=40)
    loss, g = mlp_reference.loss_and_gradient(p, x, y)
    for i in rng.choice(len(p), 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (mlp_reference.loss_and_gradient(p + e, x, y)[0] - mlp_reference.loss_and_gradient(p - e, x, y)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8
