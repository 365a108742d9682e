"""Host-side mirror of Galacticus's ``mergerTreeNodeEvolver`` interface.

``MergerTreeNodeEvolverStandard`` takes the parameters of the reference's
``mergerTreeNodeEvolverStandard`` constructor (merger_trees/node_evolver/
standard.F90:141-311: odeToleranceAbsolute, odeToleranceRelative,
reuseODEStepSize, ...) plus the physics-class choices of the P-std profile,
and its ``evolve`` method advances a batch of nodes with the semantics of
``mergerTreeNodeEvolver%evolve`` (node_evolver/_class.F90:41-57): each node
goes from its current time to ``time_end``; ``step`` carries
``node%timeStep()`` in and out; without ``return_status`` a failed node
raises, as ``Error_Report`` aborts the reference; with it the per-node
status codes are returned, as the optional ``status`` argument does there.

All work happens in the CUDA library through the C ABI of
``include/galnode.h``; this module only marshals numpy arrays.  There is no
CPU fallback: without a GPU or without the built library it raises.
"""

import ctypes

import numpy as np

from . import _abi
from .cie_tables import CieTable


class GalnodeError(RuntimeError):
    pass


def _check(lib, ctx, rc):
    if rc != 0:
        buf = ctypes.create_string_buffer(512)
        lib.gal_gpu_last_error(ctx, buf, 512)
        raise GalnodeError(f"galnode error {rc}: {buf.value.decode(errors='replace')}")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class MergerTreeNodeEvolverStandard:
    """GB300 evolver of node property vectors (batched)."""

    def __init__(self, odeToleranceAbsolute=0.01, odeToleranceRelative=0.01, reuseODEStepSize=True,
                 params=None, table=None, stepBudget=None, ratePrecision="fp64"):
        self.lib = _abi.load_library()
        self.params = params if params is not None else _abi.default_params()
        if params is None:
            self.lib.gal_params_default(ctypes.byref(self.params))
            self.params.ode_tolerance_absolute = odeToleranceAbsolute
            self.params.ode_tolerance_relative = odeToleranceRelative
            self.params.reuse_step_size = 1 if reuseODEStepSize else 0
        if stepBudget is not None:
            self.params.step_budget = int(stepBudget)
        self.table = table if table is not None else CieTable()
        ctx = ctypes.c_void_p()
        rc = self.lib.gal_gpu_init(ctypes.byref(self.params), ctypes.byref(self.table.struct), ctypes.byref(ctx))
        _check(self.lib, None, rc)
        self.ctx = ctx
        self.set_rate_precision(ratePrecision)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.gal_gpu_free(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch(self, threads_per_block=0, blocks_per_sm=0):
        _check(self.lib, self.ctx, self.lib.gal_gpu_set_launch(self.ctx, threads_per_block, blocks_per_sm))

    def set_rate_precision(self, precision):
        """"fp64" (the reference's arithmetic) or "fp32" (FP32 rates; FP64
        state, error norm and step control)."""
        code = {"fp64": _abi.RATES_FP64, "fp32": _abi.RATES_FP32}[precision]
        _check(self.lib, self.ctx, self.lib.gal_gpu_set_rate_precision(self.ctx, code))

    def get_launch(self):
        t, b = ctypes.c_int32(), ctypes.c_int32()
        self.lib.gal_gpu_get_launch(self.ctx, ctypes.byref(t), ctypes.byref(b))
        return t.value, b.value

    def evolve(self, state, param, time_start, time_end, step=None, return_status=False, counters=False):
        """Evolve a batch in place.  ``state`` is the [GAL_NY][n] FP64 SoA
        of evolved properties, ``param`` the [GAL_NP][n] node inputs."""
        state = np.asarray(state)
        if state.dtype != np.float64 or not state.flags.c_contiguous:
            raise ValueError("state must be a C-contiguous float64 array")
        n = state.shape[1]
        param = np.ascontiguousarray(param, dtype=np.float64)
        t0 = np.ascontiguousarray(time_start, dtype=np.float64)
        t1 = np.ascontiguousarray(time_end, dtype=np.float64)
        if param.shape != (_abi.NP, n) or t0.shape != (n,) or t1.shape != (n,) or state.shape != (_abi.NY, n):
            raise ValueError("array shapes do not match the node count")
        if step is None:
            step = np.full(n, -1.0)
        if step.dtype != np.float64 or step.shape != (n,):
            raise ValueError("step must be a float64 array of length n")
        status = np.zeros(n, dtype=np.int32)
        cnt = np.zeros((3, n), dtype=np.uint32) if counters else None
        rc = self.lib.gal_gpu_evolve_batch(
            self.ctx, n, _dp(state), _dp(param), _dp(t0), _dp(t1), _dp(step),
            status.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if counters else None)
        _check(self.lib, self.ctx, rc)
        if not return_status and np.any(status != _abi.STATUS_SUCCESS):
            bad = int(np.flatnonzero(status != _abi.STATUS_SUCCESS)[0])
            raise GalnodeError(f"ODE integration failed for node {bad} with status {int(status[bad])}")
        out = [status] if return_status else []
        if counters:
            out.append(cnt)
        return tuple(out) if len(out) > 1 else (out[0] if out else None)

    def evolve_interruptible(self, state, param, time_start, time_end, step, components, counters=False):
        """Evolve a batch in place with interrupts: the reference's
        ``evolve(..., interrupted, functionInterrupt, ...)``.  ``components``
        holds each node's GAL_COMPONENT_* mask; a node that gives a rate to a
        component it does not have stops at that time.  Returns (status,
        t_reached, task[, counters]): status GAL_STATUS_INTERRUPTED (9) with
        the time reached and the GAL_INTERRUPT_* task of the components to
        create, GAL_STATUS_SUCCESS at time_end, or a failure code."""
        state = np.asarray(state)
        if state.dtype != np.float64 or not state.flags.c_contiguous:
            raise ValueError("state must be a C-contiguous float64 array")
        n = state.shape[1]
        param = np.ascontiguousarray(param, dtype=np.float64)
        t0 = np.ascontiguousarray(time_start, dtype=np.float64)
        t1 = np.ascontiguousarray(time_end, dtype=np.float64)
        comps = np.ascontiguousarray(components, dtype=np.int32)
        if (param.shape != (_abi.NP, n) or t0.shape != (n,) or t1.shape != (n,) or comps.shape != (n,)
                or step.dtype != np.float64 or step.shape != (n,)):
            raise ValueError("array shapes do not match the node count")
        status = np.zeros(n, dtype=np.int32)
        reached = np.zeros(n)
        task = np.zeros(n, dtype=np.int32)
        cnt = np.zeros((3, n), dtype=np.uint32) if counters else None
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        rc = self.lib.gal_gpu_evolve_batch_interrupt(
            self.ctx, n, _dp(state), _dp(param), _dp(t0), _dp(t1), _dp(step), ip(comps), ip(status),
            cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)) if counters else None, _dp(reached), ip(task))
        _check(self.lib, self.ctx, rc)
        return (status, reached, task, cnt) if counters else (status, reached, task)
