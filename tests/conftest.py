import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgalnode.so")


@pytest.fixture(scope="session")
def table():
    from galacticus_gb300.cie_tables import CieTable
    return CieTable()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def trained(table):
    """The cooling surrogate trained on the GPU in the full configuration
    (2M samples, 90/10 split, Adam from 1e-3, 20 epochs), shared by the
    GPU test modules that need it."""
    from galacticus_gb300 import surrogate
    return surrogate.train(table, n_samples=2_000_000, epochs=20)
