"""Parity criterion between a GPU result and the oracle (test infrastructure).

A final value matches when it lies within ten times the ODE tolerance of the
oracle's value, in the solver's own mixed norm:
    |gpu - ref| <= 10 (eps_rel |ref| + eps_abs scale_i),
where scale_i is the absolute-tolerance scale of property i set from the
initial state (the scaleSetTask rules of the standard components).
"""

import numpy as np

from galacticus_gb300 import _abi


def scales(state0, param):
    """[NY][n] absolute-tolerance scales of the initial state."""
    y = np.asarray(state0)
    s = np.empty_like(y)
    hot = 1.0e-3 * param[_abi.P_MASS]
    for i in (_abi.Y_HOT_MASS, _abi.Y_HOT_METALS, _abi.Y_OUTFLOWED_MASS, _abi.Y_OUTFLOWED_METALS):
        s[i] = hot
    mass = np.maximum(np.abs(y[_abi.Y_DISK_GAS]) + np.abs(y[_abi.Y_SPHEROID_GAS]) + np.abs(y[_abi.Y_DISK_STARS])
                      + np.abs(y[_abi.Y_SPHEROID_STARS]), 1.0)
    metals = np.maximum(np.abs(y[_abi.Y_DISK_GAS_METALS]) + np.abs(y[_abi.Y_DISK_STARS_METALS])
                        + np.abs(y[_abi.Y_SPHEROID_GAS_METALS]), np.maximum(mass * 1.0e-4, 1.0))
    for i in (_abi.Y_DISK_GAS, _abi.Y_DISK_STARS, _abi.Y_SPHEROID_GAS, _abi.Y_SPHEROID_STARS):
        s[i] = mass
    for i in (_abi.Y_DISK_GAS_METALS, _abi.Y_DISK_STARS_METALS, _abi.Y_SPHEROID_GAS_METALS):
        s[i] = metals
    stars = np.maximum(y[_abi.Y_SPHEROID_STARS], 0.0)
    s[_abi.Y_BLACK_HOLE] = np.maximum(np.maximum(1.0, 1.0e-4 * stars), y[_abi.Y_BLACK_HOLE])
    return s


def parity_ratio(gpu, ref, state0, param, params, factor=10.0):
    """|gpu-ref| / (factor * tolerance) per property and node; <= 1 passes."""
    tol = factor * (params.ode_tolerance_relative * np.abs(ref) + params.ode_tolerance_absolute * scales(state0, param))
    return np.abs(gpu - ref) / tol


def parity_bound(ref, state0, param, params, factor=10.0):
    """The allowed |gpu - ref| of parity_ratio: factor times the tolerance."""
    return factor * (params.ode_tolerance_relative * np.abs(ref) + params.ode_tolerance_absolute * scales(state0, param))
