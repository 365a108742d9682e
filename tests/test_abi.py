"""C ABI checks that need no GPU: the library loads, exports every symbol
that include/galnode.h declares, and its defaults match the Python mirror."""

import ctypes
import os
import re

import numpy as np
import pytest

from galacticus_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(gal_[a-z0-9_]+)\s*\(", text, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("libgalnode.so not built")
    return _abi.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "gal_gpu_evolve_batch" in names and "gal_gpu_init" in names
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_defaults_match_python_mirror(lib):
    a = _abi.Params()
    lib.gal_params_default(ctypes.byref(a))
    b = _abi.default_params()
    assert bytes(a) == bytes(b)


def test_struct_sizes_match_header():
    # gal_params: 14 doubles + 4 ints ... computed by the C compiler in the oracle build
    assert ctypes.sizeof(_abi.StarFormation) == 40
    assert ctypes.sizeof(_abi.Outflow) == 40
    assert ctypes.sizeof(_abi.CieTable) == 40


def test_init_without_gpu_fails_loudly(lib, table):
    """No CPU fallback: on a machine without a GPU, init returns an error."""
    import shutil
    import subprocess
    if shutil.which("nvidia-smi") and subprocess.run(["nvidia-smi", "-L"], capture_output=True).returncode == 0:
        pytest.skip("a GPU is present")
    p = _abi.default_params()
    ctx = ctypes.c_void_p()
    rc = lib.gal_gpu_init(ctypes.byref(p), ctypes.byref(table.struct), ctypes.byref(ctx))
    assert rc == _abi.ERR_NO_DEVICE
    buf = ctypes.create_string_buffer(256)
    assert lib.gal_gpu_last_error(None, buf, 256) == _abi.ERR_NO_DEVICE
    assert b"device" in buf.value


def test_bad_arguments_are_rejected(lib, table):
    p = _abi.default_params()
    p.ode_tolerance_absolute = 0.0
    p.ode_tolerance_relative = 0.0
    ctx = ctypes.c_void_p()
    assert lib.gal_gpu_init(ctypes.byref(p), ctypes.byref(table.struct), ctypes.byref(ctx)) == _abi.ERR_ARGUMENT
    p = _abi.default_params()
    bad = np.array(table.cooling_rate)
    bad[0, 0] = -1.0
    from galacticus_gb300.cie_tables import CieTable
    t2 = CieTable(table.temperature, table.metallicity, bad, table.electron_density)
    assert lib.gal_gpu_init(ctypes.byref(p), ctypes.byref(t2.struct), ctypes.byref(ctx)) == _abi.ERR_TABLE
