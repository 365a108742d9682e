"""ctypes loader of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py for the timed CPU baseline.  The product never
imports this module.
"""

import ctypes
import os
import subprocess

import numpy as np

from galacticus_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build():
    """Compile the oracle with its Makefile (a second or two)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        l = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        up = ctypes.POINTER(ctypes.c_uint32)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        pp = ctypes.POINTER(_abi.Params)
        tp = ctypes.POINTER(_abi.CieTable)
        l.oracle_evolve_batch.argtypes = [pp, tp, ctypes.c_int64, dp, dp, dp, dp, dp, ip, up, ctypes.c_int, ctypes.c_int]
        l.oracle_evolve_batch.restype = ctypes.c_int
        l.oracle_cooling_function.argtypes = [tp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        l.oracle_cooling_function.restype = ctypes.c_double
        l.oracle_electron_density.argtypes = [tp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        l.oracle_electron_density.restype = ctypes.c_double
        l.oracle_cooling_radius.argtypes = [pp, tp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        l.oracle_cooling_radius.restype = ctypes.c_double
        l.oracle_rhs.argtypes = [pp, tp, dp, dp, dp]
        l.oracle_rhs.restype = ctypes.c_int
        l.oracle_ode_test.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, dp, ctypes.c_double, ctypes.c_double]
        l.oracle_ode_test.restype = ctypes.c_int
        l.oracle_count_flops.argtypes = [pp, tp, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, u64p, up]
        l.oracle_count_flops.restype = ctypes.c_int
        _lib = l
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def evolve_batch(params, table, state, param, t_start, t_end, step, threads=0, brent=True):
    """Evolve copies of the given SoA arrays on the CPU.  Returns
    (state, step, status, counters)."""
    n = state.shape[1]
    state = np.ascontiguousarray(state, dtype=np.float64).copy()
    param = np.ascontiguousarray(param, dtype=np.float64)
    t_start = np.ascontiguousarray(t_start, dtype=np.float64)
    t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    step = np.ascontiguousarray(step, dtype=np.float64).copy()
    status = np.zeros(n, dtype=np.int32)
    counters = np.zeros((3, n), dtype=np.uint32)
    rc = lib().oracle_evolve_batch(
        ctypes.byref(params), ctypes.byref(table.struct), n, _dp(state), _dp(param), _dp(t_start), _dp(t_end),
        _dp(step), status.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
        counters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), int(threads), 1 if brent else 0)
    if rc != 0:
        raise RuntimeError(f"oracle_evolve_batch failed with code {rc}")
    return state, step, status, counters


def evolve_batch_interrupt(params, table, state, param, t_start, t_end, step, components, threads=0, brent=True):
    """Evolve copies of the given SoA arrays on the CPU with interrupts
    (gal_gpu_evolve_batch_interrupt's semantics).  Returns (state, step,
    status, counters, t_reached, task)."""
    n = state.shape[1]
    state = np.ascontiguousarray(state, dtype=np.float64).copy()
    param = np.ascontiguousarray(param, dtype=np.float64)
    t_start = np.ascontiguousarray(t_start, dtype=np.float64)
    t_end = np.ascontiguousarray(t_end, dtype=np.float64)
    step = np.ascontiguousarray(step, dtype=np.float64).copy()
    components = np.ascontiguousarray(components, dtype=np.int32)
    status = np.zeros(n, dtype=np.int32)
    counters = np.zeros((3, n), dtype=np.uint32)
    t_reached = np.zeros(n)
    task = np.zeros(n, dtype=np.int32)
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    rc = lib().oracle_evolve_batch_interrupt(
        ctypes.byref(params), ctypes.byref(table.struct), n, _dp(state), _dp(param), _dp(t_start), _dp(t_end),
        _dp(step), ip(components), ip(status), counters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
        _dp(t_reached), ip(task), int(threads), 1 if brent else 0)
    if rc != 0:
        raise RuntimeError(f"oracle_evolve_batch_interrupt failed with code {rc}")
    return state, step, status, counters, t_reached, task


def ode_test(problem, x0, x1, y, tol_abs, tol_rel):
    y = np.ascontiguousarray(y, dtype=np.float64).copy()
    rc = lib().oracle_ode_test(problem, x0, x1, _dp(y), tol_abs, tol_rel)
    return rc, y


def rhs(params, table, param_node, y):
    param_node = np.ascontiguousarray(param_node, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    d = np.zeros(_abi.NY)
    rc = lib().oracle_rhs(ctypes.byref(params), ctypes.byref(table.struct), _dp(param_node), _dp(y), _dp(d))
    if rc:
        raise RuntimeError(f"oracle_rhs failed with code {rc}")
    return d


def cooling_radius(params, table, param_node, mass_hot, metals_hot, brent=True):
    param_node = np.ascontiguousarray(param_node, dtype=np.float64)
    return lib().oracle_cooling_radius(ctypes.byref(params), ctypes.byref(table.struct), _dp(param_node),
                                       mass_hot, metals_hot, 1 if brent else 0)


def count_flops(params, table, param_node, y, t0, t1, step=-1.0):
    """Operation counts (add, mul, div, sqrt, log, exp, pow, atan, cbrt) and
    the (accepted, rejected, rhs) counters of one node evolution."""
    param_node = np.ascontiguousarray(param_node, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64).copy()
    ops = np.zeros(9, dtype=np.uint64)
    counters = np.zeros(3, dtype=np.uint32)
    lib().oracle_count_flops(ctypes.byref(params), ctypes.byref(table.struct), _dp(param_node), _dp(y), t0, t1, step,
                             ops.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                             counters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return ops, counters


def forest_snapshots(forest, output_times):
    """Snapshot slot layout of a forest: (first slot per node, total)."""
    n = forest.n
    first = np.zeros(n, dtype=np.int64)
    t_out = np.ascontiguousarray(output_times, dtype=np.float64)
    l = lib()
    l.oracle_forest_snapshots.restype = ctypes.c_int64
    total = l.oracle_forest_snapshots(ctypes.c_int64(n), forest.parent.ctypes.data_as(ctypes.c_void_p),
                                      forest.time.ctypes.data_as(ctypes.c_void_p), ctypes.c_int32(len(t_out)),
                                      t_out.ctypes.data_as(ctypes.c_void_p), first.ctypes.data_as(ctypes.c_void_p))
    return first, int(total)


def evolve_forest(params, table, forest, state0, output_times, threads=0, brent=True):
    """Evolve a forest (galacticus_gb300.forest.Forest) on the CPU.  Returns
    (state [NY][n] on reaching each parent, status, counters [3][n],
    snapshots [NY][m] at the output times)."""
    n = forest.n
    t_out = np.ascontiguousarray(output_times, dtype=np.float64)
    _, m = forest_snapshots(forest, t_out)
    state0 = np.ascontiguousarray(state0, dtype=np.float64)
    state = np.zeros((_abi.NY, n))
    status = np.zeros(n, dtype=np.int32)
    counters = np.zeros((3, n), dtype=np.uint32)
    snap = np.zeros((_abi.NY, max(m, 1)))
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    l = lib()
    l.oracle_evolve_forest.restype = ctypes.c_int
    host = getattr(forest, "satellite_host", None)
    host = None if host is None else np.ascontiguousarray(host, dtype=np.int32)
    rc = l.oracle_evolve_forest(ctypes.byref(params), ctypes.byref(table.struct), ctypes.c_int64(n), vp(forest.parent),
                                vp(forest.child_first), vp(forest.child_count), vp(forest.time), vp(forest.mass),
                                vp(forest.spin), None if host is None else vp(host), vp(state0),
                                ctypes.c_int32(len(t_out)), vp(t_out), vp(state), vp(status), vp(counters), vp(snap),
                                ctypes.c_int(threads), ctypes.c_int(1 if brent else 0))
    if rc != 0:
        raise RuntimeError(f"oracle_evolve_forest failed with code {rc}")
    return state, status, counters, snap[:, :m]


def grow_trees(tables, seed, root_masses, tree0=0):
    """Grow trees tree0, tree0+1, ... of seed from their root masses with
    the oracle's restatement of the GPU branching's walk, on the builder's
    tables (forest.branch_tables).  Returns (mass, w, parent, child_first,
    child_count, tree_first): the trees one after another, each in the
    builder's order."""
    l = lib()
    vp = ctypes.c_void_p
    l.oracle_grow_trees.argtypes = [vp] * 7 + [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, vp, ctypes.c_int64] + \
        [vp] * 6
    l.oracle_grow_trees.restype = ctypes.c_int64
    roots = np.ascontiguousarray(root_masses, dtype=np.float64)
    n = len(roots)
    tree_first = np.zeros(n, np.int64)
    cap = max(1024, 64 * n)
    while True:
        out = [np.zeros(cap), np.zeros(cap)] + [np.zeros(cap, np.int32) for _ in range(3)]
        ptr = lambda a: a.ctypes.data_as(vp)
        total = l.oracle_grow_trees(ptr(tables["meta"]), ptr(tables["sizes"]), ptr(tables["ln_sigma"]),
                                    ptr(tables["rate"]), ptr(tables["accretion"]), ptr(tables["ln_q"]),
                                    ptr(tables["cdf"]), seed, tree0, n, ptr(roots), cap, *[ptr(a) for a in out],
                                    ptr(tree_first))
        if total >= 0:
            return tuple(a[:total] for a in out) + (tree_first,)
        cap = -total


def branch_math(x, y):
    """The branching walk's FP32 ln (of positive doubles x) and exp (of floats y)."""
    l = lib()
    vp = ctypes.c_void_p
    l.oracle_branch_math.argtypes = [ctypes.c_int64, vp, vp, vp, vp]
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float32)
    lx, ey = np.zeros(len(x), np.float32), np.zeros(len(y), np.float32)
    l.oracle_branch_math(len(x), x.ctypes.data_as(vp), lx.ctypes.data_as(vp), y.ctypes.data_as(vp),
                         ey.ctypes.data_as(vp))
    return lx, ey
