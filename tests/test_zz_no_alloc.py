"""The no-allocation entry point against the regular one.

gal_gpu_evolve_batch_noalloc exists for callers that cannot let a library
allocate device memory (a host code whose own pool allocator owns the
device memory, or one that must not take the device-wide synchronisation of
cudaMalloc/cudaFree).  Its kernel scratch lives in one fixed static device
array.  This test drives it through the C ABI on caller-owned device arrays,
twice in a row with tables of different sizes (the second call finds the
first call's contents in the shared scratch and must replace them), and
checks each result against gal_gpu_evolve_batch_device on a context built
from the same table, within the parity tolerance of the other GPU tests.  It is collected last so
that a stop-at-first-failure run has already run everything else.
"""

import ctypes

import numpy as np
import pytest

from galacticus_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu


def _device_copy(torch, dev, batch):
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
    return {
        "state": t(batch.state), "param": t(batch.param), "t0": t(batch.t_start), "t1": t(batch.t_end),
        "step": t(batch.step), "status": torch.zeros(batch.n, dtype=torch.int32, device=dev),
        "counters": torch.zeros((3, batch.n), dtype=torch.int32, device=dev),
    }


def _ptrs(d):
    return [d[k].data_ptr() for k in ("state", "param", "t0", "t1", "step", "status", "counters")]


def _regular(lib, torch, dev, params, table, batch):
    """State and status from the regular entry point (context-owned scratch)."""
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    ev = MergerTreeNodeEvolverStandard(params=params, table=table)
    ref = _device_copy(torch, dev, batch)
    assert lib.gal_gpu_evolve_batch_device(ev.ctx, batch.n, *_ptrs(ref), None) == 0
    torch.cuda.synchronize()
    out = ref["state"].cpu().numpy(), ref["status"].cpu().numpy()
    ev.close()
    return out


def test_noalloc_matches_regular_entry_point_twice(table):
    """Two calls in a row, the second with a coarser table (every other
    temperature: 131 instead of 261), so that the second call must restage
    the shared scratch with a different layout; each is checked against a
    context built from its own table."""
    torch = pytest.importorskip("torch")
    from galacticus_gb300.cie_tables import CieTable
    from oracle import compare

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lib = _abi.load_library()
    params = workloads.isolated_params()
    batch = workloads.isolated_halos(n=5000, seed=31)
    coarse = CieTable(table.temperature[::2], table.metallicity, table.cooling_rate[:, ::2],
                      table.electron_density[:, ::2])
    assert len(coarse.temperature) == 131

    for call, tab in enumerate((table, coarse)):
        ref_state, ref_status = _regular(lib, torch, dev, params, tab, batch)
        d = _device_copy(torch, dev, batch)
        rc = lib.gal_gpu_evolve_batch_noalloc(ctypes.byref(params), ctypes.byref(tab.struct), batch.n, *_ptrs(d), None)
        if rc:
            buf = ctypes.create_string_buffer(512)
            lib.gal_gpu_last_error(None, buf, 512)
            pytest.fail(f"call {call}: gal_gpu_evolve_batch_noalloc returned {rc}: {buf.value.decode()}")
        torch.cuda.synchronize()
        status = d["status"].cpu().numpy()
        state = d["state"].cpu().numpy()
        np.testing.assert_array_equal(status, ref_status)
        assert np.all(status == 0)
        ratio = compare.parity_ratio(state, ref_state, batch.state, batch.param, params)
        assert ratio.max() <= 1.0, f"call {call}: worst ratio {ratio.max():.3g}"


def test_noalloc_rejects_tables_beyond_its_scratch(table):
    from galacticus_gb300.cie_tables import CieTable
    lib = _abi.load_library()
    params = workloads.isolated_params()
    n_t = 4000  # 24 x 4000 cells need far more than the 128 KiB scratch
    temperature = np.logspace(2.5, 9.0, n_t)
    big = CieTable(temperature, table.metallicity, np.ones((len(table.metallicity), n_t)) * 1e-23,
                   np.ones((len(table.metallicity), n_t)))
    rc = lib.gal_gpu_evolve_batch_noalloc(ctypes.byref(params), ctypes.byref(big.struct), 1,
                                          *([ctypes.c_void_p(8)] * 7), None)
    assert rc == _abi.ERR_TOO_LARGE
    buf = ctypes.create_string_buffer(512)
    lib.gal_gpu_last_error(None, buf, 512)
    assert b"128 KiB" in buf.value
    # A shape whose cell count overflows 32-bit arithmetic is rejected on
    # its size before any table value is read.
    huge = _abi.CieTable(70000, 70000, table.struct.temperature, table.struct.metallicity,
                         table.struct.cooling_rate, table.struct.electron_density)
    rc = lib.gal_gpu_evolve_batch_noalloc(ctypes.byref(params), ctypes.byref(huge), 1,
                                          *([ctypes.c_void_p(8)] * 7), None)
    assert rc == _abi.ERR_TOO_LARGE
