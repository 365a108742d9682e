"""Synthetic collisional-ionisation-equilibrium (CIE) tables.

Galacticus reads its atomic CIE cooling function and electron densities from
``cooling_function_Atomic_CIE_Cloudy.hdf5`` / ``chemical_state_Atomic_CIE_
Cloudy.hdf5``, which it downloads from a separate dataset repository or
computes with Cloudy (source/interface/Cloudy/collisional_ionization_
equilibrium.F90).  Neither the files nor Cloudy are available here, so this
module builds stand-in tables with exactly the reference grid:

* temperature: log10 T = 2.5 ... 9.0 in steps of 0.025 (261 points,
  collisional_ionization_equilibrium.F90:67-68, 151-161);
* metallicity: a Z = 0 row followed by 23 values of log10(Z/Zsun) spaced
  evenly from -4 to log10(30) (:69-70, 152-160; 30 Zsun is the default
  maximum of coolingFunctionAtomicCIECloudy);
* extrapolation attributes "extrapolate" in T and "fix" in Z (:279-286).

The cooling curve is an analytic stand-in of the usual CIE shape: a cut-off
below 10^4 K, hydrogen and helium line peaks near 2x10^4 K and 10^5 K, metal
line peaks near 2.5x10^5 K and 2.5x10^6 K scaling linearly with Z, and a
bremsstrahlung continuum proportional to sqrt(T).  It is normalised so that
the interpolated value at T = 10^6 K, Z = Zsun and n_H = 1e-4 cm^-3 equals
1.4198e-30 erg cm^-3 s^-1, the reference's own known answer for its Cloudy
table (source/tests/cooling_functions.F90:186).  The electron density n_e/n_H
follows smooth ionisation fronts of H, He I and He II plus a small metal
contribution.
"""

import ctypes

import numpy as np

from . import _abi

LOG_T_MIN, LOG_T_MAX, LOG_T_STEP = 2.5, 9.0, 0.025
LOG_Z_MIN, Z_MAX_SOLAR, LOG_Z_STEP = -4.0, 30.0, 0.25
GOLDEN_LAMBDA = 1.4198e-30          # erg cm^-3 s^-1 at (n_H=1e-4, T=1e6 K, Zsun)
GOLDEN_POINT = (1.0e-4, 1.0e6, 1.0)  # n_H, T, Z/Zsun


def grids():
    """Temperature (K) and metallicity (Z/Zsun, first row zero) grids."""
    n_t = int((LOG_T_MAX - LOG_T_MIN) / LOG_T_STEP + 1.5)
    log_z_max = np.log10(Z_MAX_SOLAR)
    n_z = int((log_z_max - LOG_Z_MIN) / LOG_Z_STEP + 1.5)
    log_t = np.linspace(LOG_T_MIN, LOG_T_MAX, n_t)
    log_z = np.linspace(LOG_Z_MIN, log_z_max, n_z)
    temperature = 10.0 ** log_t
    metallicity = np.concatenate([[0.0], 10.0 ** log_z])
    return temperature, metallicity


def _logistic(x):
    return 1.0 / (1.0 + np.exp(-x))


def _bump(log_t, centre, width):
    return np.exp(-(((log_t - centre) / width) ** 2))


def _raw_cooling(log_t, z_solar):
    ionised = _logistic((log_t - 4.12) / 0.045)
    primordial = 7.0e-23 * _bump(log_t, 4.28, 0.14) + 2.2e-23 * _bump(log_t, 5.05, 0.22)
    metals = 6.0e-22 * _bump(log_t, 5.40, 0.33) + 1.2e-22 * _bump(log_t, 6.40, 0.45)
    brems = 2.3e-27 * np.sqrt(10.0 ** log_t)
    return ionised * (primordial + z_solar * metals + brems) + 1.0e-32


def _electron_fraction(log_t, z_solar):
    y_he = 0.0833  # primordial He/H by number
    f_h = _logistic((log_t - 4.10) / 0.05)
    f_he1 = _logistic((log_t - 4.40) / 0.06)
    f_he2 = _logistic((log_t - 4.85) / 0.07)
    metals = 1.0e-3 * z_solar * _logistic((log_t - 5.0) / 0.3)
    return f_h + y_he * (f_he1 + f_he2) + metals + 1.0e-6


def _interp_ln(table_ln, log_t_grid_ln, z_grid, ln_t, z):
    """Bilinear interpolation of a log table at one (ln T, Z/Zsun) point,
    following the reference scheme (CIE_file.F90:665-735)."""
    it = int(np.clip(np.searchsorted(log_t_grid_ln, ln_t, side="right") - 1, 0, len(log_t_grid_ln) - 2))
    ht = (ln_t - log_t_grid_ln[it]) / (log_t_grid_ln[it + 1] - log_t_grid_ln[it])
    if z < z_grid[1]:
        iz, hz = 0, z / z_grid[1]
    else:
        ln_z = np.log(z_grid[1:])
        iz = int(np.clip(np.searchsorted(ln_z, np.log(z), side="right") - 1, 0, len(ln_z) - 2)) + 1
        hz = (np.log(z) - np.log(z_grid[iz])) / (np.log(z_grid[iz + 1]) - np.log(z_grid[iz]))
    f = (table_ln[iz, it] * (1 - ht) * (1 - hz) + table_ln[iz + 1, it] * (1 - ht) * hz
         + table_ln[iz, it + 1] * ht * (1 - hz) + table_ln[iz + 1, it + 1] * ht * hz)
    return np.exp(f)


def build_tables():
    """Return (temperature, metallicity, cooling_rate, electron_density) as
    FP64 arrays; the two tables are row-major [iZ][iT]."""
    temperature, metallicity = grids()
    log_t = np.log10(temperature)
    cooling = np.empty((len(metallicity), len(temperature)))
    electrons = np.empty_like(cooling)
    for j, z in enumerate(metallicity):
        cooling[j] = _raw_cooling(log_t, z)
        electrons[j] = _electron_fraction(log_t, z)
    n_h, t_golden, z_golden = GOLDEN_POINT
    value = _interp_ln(np.log(cooling), np.log(temperature), metallicity, np.log(t_golden), z_golden) * n_h ** 2
    cooling *= GOLDEN_LAMBDA / value
    return temperature, metallicity, cooling, electrons


class CieTable:
    """Owns the table arrays and exposes them as a ``gal_cie_table``."""

    def __init__(self, temperature=None, metallicity=None, cooling_rate=None, electron_density=None):
        if temperature is None:
            temperature, metallicity, cooling_rate, electron_density = build_tables()
        self.temperature = np.ascontiguousarray(temperature, dtype=np.float64)
        self.metallicity = np.ascontiguousarray(metallicity, dtype=np.float64)
        self.cooling_rate = np.ascontiguousarray(cooling_rate, dtype=np.float64)
        self.electron_density = np.ascontiguousarray(electron_density, dtype=np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        self.struct = _abi.CieTable(
            len(self.temperature), len(self.metallicity),
            self.temperature.ctypes.data_as(dp), self.metallicity.ctypes.data_as(dp),
            self.cooling_rate.ctypes.data_as(dp), self.electron_density.ctypes.data_as(dp),
        )

    def interpolate_cooling(self, n_h, temperature, z_solar):
        """Cooling function (erg cm^-3 s^-1) by the reference interpolation."""
        t = min(max(temperature, self.temperature[0]), self.temperature[-1])
        z = min(max(z_solar, self.metallicity[0]), self.metallicity[-1])
        return _interp_ln(np.log(self.cooling_rate), np.log(self.temperature), self.metallicity,
                          np.log(t), z) * n_h ** 2
