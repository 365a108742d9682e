"""ctypes mirror of ``include/galnode.h`` and the loader of the CUDA library.

The structures here are byte-for-byte the C structures of the header; the
constants are the header's enumerations.  Nothing in this module touches a
GPU: loading the library only resolves symbols.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgalnode.so")

# Evolved properties (GAL_Y_*).
Y_NAMES = [
    "hot_mass", "hot_metals", "outflowed_mass", "outflowed_metals",
    "disk_gas", "disk_gas_metals", "disk_stars", "disk_stars_metals",
    "spheroid_gas", "spheroid_gas_metals", "spheroid_stars", "black_hole",
]
NY = 12
(Y_HOT_MASS, Y_HOT_METALS, Y_OUTFLOWED_MASS, Y_OUTFLOWED_METALS, Y_DISK_GAS, Y_DISK_GAS_METALS,
 Y_DISK_STARS, Y_DISK_STARS_METALS, Y_SPHEROID_GAS, Y_SPHEROID_GAS_METALS, Y_SPHEROID_STARS,
 Y_BLACK_HOLE) = range(NY)

# Per-node inputs (GAL_P_*).
NP = 5
P_MASS, P_MASS_RATE, P_RADIUS_VIRIAL, P_VELOCITY_VIRIAL, P_SPIN = range(NP)

STATUS_SUCCESS = 0
STATUS_UNDERFLOW = 15
STATUS_XCPU = 1025
STATUS_NOT_FINITE = 2001
STATUS_INTERRUPTED = 9

COMPONENT_DISK, COMPONENT_SPHEROID, COMPONENT_BLACK_HOLE, COMPONENT_ALL = 1, 2, 4, 7
INTERRUPT_CREATE_DISK, INTERRUPT_CREATE_SPHEROID, INTERRUPT_CREATE_BLACK_HOLE = 1, 2, 4
RATES_FP64 = 0
RATES_FP32 = 1

OK, ERR_ARGUMENT, ERR_CUDA, ERR_TABLE, ERR_NO_DEVICE, ERR_TOO_LARGE = range(6)

PHYS_STAR_FORMATION_DISK = 1 << 0
PHYS_STAR_FORMATION_SPHEROID = 1 << 1
PHYS_FEEDBACK_DISK = 1 << 2
PHYS_FEEDBACK_SPHEROID = 1 << 3
PHYS_BLACK_HOLE_ACCRETION = 1 << 4
PHYS_CGM_ACCRETION = 1 << 5
PHYS_REINCORPORATION = 1 << 6
PHYS_COOLING = 1 << 7
PHYS_ALL = 0xFF

SF_TIMESCALE_DYNAMICAL, SF_TIMESCALE_FIXED = 0, 1
SF_RATE_TIMESCALE, SF_RATE_KRUMHOLZ2009 = 0, 1
OUTFLOW_POWER_LAW, OUTFLOW_FIXED = 0, 1


class StarFormation(ctypes.Structure):
    _fields_ = [
        ("timescale_type", ctypes.c_int32), ("pad", ctypes.c_int32),
        ("efficiency", ctypes.c_double), ("exponent_velocity", ctypes.c_double),
        ("timescale_minimum", ctypes.c_double), ("timescale_fixed", ctypes.c_double),
    ]


class Outflow(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32), ("pad", ctypes.c_int32),
        ("velocity_characteristic", ctypes.c_double), ("exponent", ctypes.c_double),
        ("fraction", ctypes.c_double), ("timescale_fractional_minimum", ctypes.c_double),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("ode_tolerance_absolute", ctypes.c_double),
        ("ode_tolerance_relative", ctypes.c_double),
        ("reuse_step_size", ctypes.c_int32),
        ("trial_count_maximum", ctypes.c_int32),
        ("step_budget", ctypes.c_int32),
        ("physics", ctypes.c_uint32),
        ("omega_matter", ctypes.c_double), ("omega_baryon", ctypes.c_double),
        ("omega_dark_energy", ctypes.c_double), ("hubble_constant", ctypes.c_double),
        ("core_radius_fraction", ctypes.c_double),
        ("cooling_velocity_cutoff", ctypes.c_double),
        ("cooling_degrees_of_freedom", ctypes.c_double),
        ("reincorporation_multiplier", ctypes.c_double),
        ("radius_factor_disk", ctypes.c_double), ("radius_factor_spheroid", ctypes.c_double),
        ("sf_disk", StarFormation), ("sf_spheroid", StarFormation),
        ("recycled_fraction", ctypes.c_double), ("metal_yield", ctypes.c_double),
        ("outflow_disk", Outflow), ("outflow_spheroid", Outflow),
        ("bh_enhancement_spheroid", ctypes.c_double),
        ("bh_enhancement_hot_halo", ctypes.c_double),
        ("bh_temperature_spheroid", ctypes.c_double),
        ("bh_hot_mode_only", ctypes.c_int32), ("pad", ctypes.c_int32),
        ("bh_efficiency_radiative", ctypes.c_double),
        ("bh_efficiency_jet", ctypes.c_double),
        ("timestep_relative", ctypes.c_double), ("timestep_absolute", ctypes.c_double),
        ("sf_disk_rate", ctypes.c_int32), ("krumholz_fast", ctypes.c_int32),
        ("krumholz_frequency", ctypes.c_double), ("krumholz_clumping", ctypes.c_double),
        ("merger_mass_ratio_major", ctypes.c_double),
    ]


class CieTable(ctypes.Structure):
    _fields_ = [
        ("n_temperature", ctypes.c_int32), ("n_metallicity", ctypes.c_int32),
        ("temperature", ctypes.POINTER(ctypes.c_double)),
        ("metallicity", ctypes.POINTER(ctypes.c_double)),
        ("cooling_rate", ctypes.POINTER(ctypes.c_double)),
        ("electron_density", ctypes.POINTER(ctypes.c_double)),
    ]


def default_params():
    """The P-std parameter set, built in Python with the values that
    ``gal_params_default`` writes (tests check the two agree)."""
    p = Params()
    p.ode_tolerance_absolute = 0.01
    p.ode_tolerance_relative = 0.01
    p.reuse_step_size = 1
    p.trial_count_maximum = 8
    p.step_budget = 1_000_000
    p.physics = PHYS_ALL
    p.omega_matter, p.omega_baryon, p.omega_dark_energy, p.hubble_constant = 0.3, 0.045, 0.7, 70.0
    p.core_radius_fraction = 0.3
    p.cooling_velocity_cutoff = 1.0e4
    p.cooling_degrees_of_freedom = 3.0
    p.reincorporation_multiplier = 5.0
    p.radius_factor_disk = p.radius_factor_spheroid = 0.5 ** 0.5
    for sf in (p.sf_disk, p.sf_spheroid):
        sf.timescale_type = SF_TIMESCALE_DYNAMICAL
        sf.efficiency, sf.exponent_velocity, sf.timescale_minimum = 0.01, -1.5, 1.0e-3
        sf.timescale_fixed = 1.0
    p.recycled_fraction, p.metal_yield = 0.46, 0.035
    for o, v in ((p.outflow_disk, 250.0), (p.outflow_spheroid, 100.0)):
        o.type = OUTFLOW_POWER_LAW
        o.velocity_characteristic, o.exponent = v, 3.5
        o.fraction = 1.0
        o.timescale_fractional_minimum = 1.0e-3
    p.bh_enhancement_spheroid, p.bh_enhancement_hot_halo = 5.0, 6.0
    p.bh_temperature_spheroid = 100.0
    p.bh_hot_mode_only = 1
    p.bh_efficiency_radiative = 1.0 - (8.0 / 9.0) ** 0.5
    p.bh_efficiency_jet = 0.0
    p.timestep_relative, p.timestep_absolute = 0.1, 1.0
    p.sf_disk_rate, p.krumholz_fast = SF_RATE_TIMESCALE, 0
    p.krumholz_frequency, p.krumholz_clumping = 0.385, 5.0
    p.merger_mass_ratio_major = 0.25
    return p


_lib = None


def load_library(path=LIB_PATH):
    """Load ``libgalnode.so`` and declare its C signatures.  Raises
    ``OSError`` with a clear message when the library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)
    up = ctypes.POINTER(ctypes.c_uint32)
    vp = ctypes.c_void_p
    ctx_pp = ctypes.POINTER(ctypes.c_void_p)
    lib.gal_params_default.argtypes = [ctypes.POINTER(Params)]
    lib.gal_params_default.restype = None
    lib.gal_version.restype = ctypes.c_char_p
    lib.gal_gpu_init.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(CieTable), ctx_pp]
    lib.gal_gpu_init.restype = ctypes.c_int
    lib.gal_gpu_free.argtypes = [vp]
    lib.gal_gpu_free.restype = None
    lib.gal_gpu_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
    lib.gal_gpu_last_error.restype = ctypes.c_int
    lib.gal_gpu_evolve_batch.argtypes = [vp, ctypes.c_int64, dp, dp, dp, dp, dp, ip, up]
    lib.gal_gpu_evolve_batch.restype = ctypes.c_int
    lib.gal_gpu_evolve_batch_device.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gal_gpu_evolve_batch_device.restype = ctypes.c_int
    lib.gal_gpu_evolve_batch_interrupt.argtypes = [vp, ctypes.c_int64, dp, dp, dp, dp, dp, ip, ip, up, dp, ip]
    lib.gal_gpu_evolve_batch_interrupt.restype = ctypes.c_int
    lib.gal_gpu_evolve_batch_interrupt_device.argtypes = [vp, ctypes.c_int64] + [vp] * 11
    lib.gal_gpu_evolve_batch_interrupt_device.restype = ctypes.c_int
    lib.gal_gpu_set_launch.argtypes = [vp, ctypes.c_int32, ctypes.c_int32]
    lib.gal_gpu_set_launch.restype = ctypes.c_int
    lib.gal_gpu_get_launch.argtypes = [vp, ip, ip]
    lib.gal_gpu_get_launch.restype = ctypes.c_int
    lib.gal_gpu_launch_count.argtypes = [vp]
    lib.gal_gpu_launch_count.restype = ctypes.c_int64
    lib.gal_gpu_set_rate_precision.argtypes = [vp, ctypes.c_int32]
    lib.gal_gpu_set_rate_precision.restype = ctypes.c_int
    lib.gal_gpu_get_rate_precision.argtypes = [vp]
    lib.gal_gpu_get_rate_precision.restype = ctypes.c_int
    lib.gal_gpu_evolve_batch_noalloc.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(CieTable), ctypes.c_int64,
                                                 vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gal_gpu_evolve_batch_noalloc.restype = ctypes.c_int
    lib.gal_calibrate_fp64.argtypes = [dp, dp]
    lib.gal_calibrate_fp64.restype = ctypes.c_int
    lib.gal_selftest_fastmath.argtypes = [dp]
    lib.gal_selftest_fastmath.restype = ctypes.c_int
    _lib = lib
    return lib
