"""Synthetic node batches with the shapes of the benchmark configurations.

There are no merger-tree or halo catalogues to read, so the inputs are drawn
from seeded counter-based streams (numpy's Philox4x32 bit generator keyed by
the configuration seed) with the documented distributions.  Host-side only;
nothing here is timed.

Cosmology is the flat matter + cosmological-constant model of
``cosmologyFunctionsMatterLambda`` with the configuration's parameters;
virial quantities use the Bryan & Norman (1998) density contrast
(source/structure_formation/virial_density_contrast/Bryan_Norman.F90:172-196)
relative to the mean matter density.
"""

from dataclasses import dataclass

import numpy as np

from . import _abi

G_INTERNAL = 6.673e-11 * 1.98892e30 / 1.0e6 / (1.0e6 * 3.08567758135e16)  # km^2 s^-2 Mpc / Msun
MPC_PER_KM_PER_S_TO_GYR = 1.0e6 * 3.08567758135e16 / 1.0e3 / (1.0e9 * 3.15581497635456e7)


@dataclass
class Cosmology:
    omega_matter: float = 0.3
    omega_lambda: float = 0.7
    omega_baryon: float = 0.045
    hubble: float = 70.0  # km/s/Mpc
    sigma8: float = 0.8
    n_s: float = 0.96

    @property
    def hubble_gyr(self):
        return self.hubble / MPC_PER_KM_PER_S_TO_GYR

    def time(self, z):
        """Cosmic time (Gyr) at redshift z for a flat matter+Lambda model."""
        a = 1.0 / (1.0 + np.asarray(z, dtype=np.float64))
        return (2.0 / (3.0 * self.hubble_gyr * np.sqrt(self.omega_lambda))
                * np.arcsinh(np.sqrt(self.omega_lambda / self.omega_matter) * a ** 1.5))

    def redshift(self, t):
        """Inverse of time()."""
        x = np.sinh(1.5 * self.hubble_gyr * np.sqrt(self.omega_lambda) * np.asarray(t, dtype=np.float64))
        a = (x / np.sqrt(self.omega_lambda / self.omega_matter)) ** (2.0 / 3.0)
        return 1.0 / a - 1.0

    def density_mean(self, z):
        rho_crit0 = 3.0 * self.hubble ** 2 / (8.0 * np.pi * G_INTERNAL)  # Msun/Mpc^3
        return self.omega_matter * rho_crit0 * (1.0 + np.asarray(z)) ** 3

    def virial_contrast_mean(self, z):
        z = np.asarray(z, dtype=np.float64)
        om = self.omega_matter * (1 + z) ** 3 / (self.omega_matter * (1 + z) ** 3 + self.omega_lambda)
        x = om - 1.0
        return (18.0 * np.pi ** 2 + 82.0 * x - 39.0 * x ** 2) / (x + 1.0)

    def virial(self, mass, z):
        """Virial radius (Mpc) and velocity (km/s) of halos of the given mass."""
        rho = self.virial_contrast_mean(z) * self.density_mean(z)
        r = np.cbrt(3.0 * mass / (4.0 * np.pi * rho))
        v = np.sqrt(G_INTERNAL * mass / r)
        return r, v


SPIN_DEFAULT = 0.04326  # peak of the Bett et al. (2007) spin distribution (parameters/quickTest.xml)


@dataclass
class Batch:
    state: np.ndarray   # [NY][n]
    param: np.ndarray   # [NP][n]
    t_start: np.ndarray
    t_end: np.ndarray
    step: np.ndarray

    @property
    def n(self):
        return self.state.shape[1]

    def copy(self):
        return Batch(self.state.copy(), self.param.copy(), self.t_start.copy(), self.t_end.copy(), self.step.copy())

    def subset(self, idx):
        return Batch(self.state[:, idx].copy(), self.param[:, idx].copy(), self.t_start[idx].copy(),
                     self.t_end[idx].copy(), self.step[idx].copy())


def isolated_halos(n=65536, seed=2, cosmology=None, spin=SPIN_DEFAULT):
    """Batched isolated step: n independent halos, each advanced over one
    timestep.  Halo mass log-uniform in 1e10-1e14 Msun; hot gas
    (Omega_b/Omega_m) M U(0.5,1); metallicity log-uniform 1e-4-0.02 (mass
    fraction); disk and spheroid empty; black hole 1e5 Msun; redshift
    uniform in 0-4; timestep log-uniform in 0.01-1 Gyr."""
    cosmo = cosmology or Cosmology()
    rng = np.random.Generator(np.random.Philox(key=seed))
    u = rng.random((6, n))
    mass = 10.0 ** (10.0 + 4.0 * u[0])
    z = 4.0 * u[1]
    hot = cosmo.omega_baryon / cosmo.omega_matter * mass * (0.5 + 0.5 * u[2])
    metallicity = 10.0 ** (-4.0 + np.log10(200.0) * u[3])
    dt = 10.0 ** (-2.0 + 2.0 * u[4])
    r, v = cosmo.virial(mass, z)
    state = np.zeros((_abi.NY, n))
    state[_abi.Y_HOT_MASS] = hot
    state[_abi.Y_HOT_METALS] = metallicity * hot
    state[_abi.Y_BLACK_HOLE] = 1.0e5
    param = np.zeros((_abi.NP, n))
    param[_abi.P_MASS] = mass
    param[_abi.P_MASS_RATE] = 0.0
    param[_abi.P_RADIUS_VIRIAL] = r
    param[_abi.P_VELOCITY_VIRIAL] = v
    param[_abi.P_SPIN] = spin
    t0 = cosmo.time(z)
    return Batch(state, param, t0, t0 + dt, np.full(n, -1.0))


def galaxy_halos(n=8192, seed=12, cosmology=None, spin=SPIN_DEFAULT):
    """Isolated halos that already hold a galaxy: the halos, hot gas, times
    and timesteps of isolated_halos(), plus a gaseous and stellar disk and
    spheroid with metals, and a central black hole of 1e4-1e9 Msun.  Masses
    (as fractions f of the halo's baryons (Omega_b/Omega_m) M):
    disk gas and stars log-uniform f in 1e-3-0.1, spheroid gas log-uniform f
    in 1e-4-0.1, spheroid stars log-uniform f in 1e-3-0.3, gas metallicities
    log-uniform 1e-3-0.03 (mass fraction), stellar disk metallicity 0.01; the
    black-hole mass log-uniform.  This batch runs every operator of the node
    (spheroid star formation, feedback and Bondi-Hoyle accretion from the
    spheroid gas on both sides of the Jeans-length condition) from the
    first step."""
    batch = isolated_halos(n=n, seed=seed, cosmology=cosmology, spin=spin)
    cosmo = cosmology or Cosmology()
    rng = np.random.Generator(np.random.Philox(key=seed + 1000))
    u = rng.random((8, n))
    baryons = cosmo.omega_baryon / cosmo.omega_matter * batch.param[_abi.P_MASS]
    s = batch.state
    s[_abi.Y_DISK_GAS] = baryons * 10.0 ** (-3.0 + 2.0 * u[0])
    s[_abi.Y_DISK_GAS_METALS] = s[_abi.Y_DISK_GAS] * 10.0 ** (-3.0 + np.log10(30.0) * u[1])
    s[_abi.Y_DISK_STARS] = baryons * 10.0 ** (-3.0 + 2.0 * u[2])
    s[_abi.Y_DISK_STARS_METALS] = 0.01 * s[_abi.Y_DISK_STARS]
    s[_abi.Y_SPHEROID_GAS] = baryons * 10.0 ** (-4.0 + 3.0 * u[3])
    s[_abi.Y_SPHEROID_GAS_METALS] = s[_abi.Y_SPHEROID_GAS] * 10.0 ** (-3.0 + np.log10(30.0) * u[4])
    s[_abi.Y_SPHEROID_STARS] = baryons * 10.0 ** (-3.0 + np.log10(300.0) * u[5])
    s[_abi.Y_BLACK_HOLE] = 10.0 ** (4.0 + 5.0 * u[6])
    return batch


def disk_creation_halos(n=8192, seed=21, cosmology=None, spin=SPIN_DEFAULT):
    """Halos without a disk whose hot gas starts to cool during the step:
    the halos, times and timesteps of isolated_halos(), hot gas log-uniform
    in 1e-3-0.3 of the halo's baryons (Omega_b/Omega_m) M with metallicity
    log-uniform 1e-4-0.02, and halo growth at 0.05-0.5 M per Gyr, whose
    accreted gas raises the cooling rate.  Returns (batch, components): the
    GAL_COMPONENT_* masks say every halo has a spheroid and a black hole and
    no disk, so that cooling into the disk interrupts the integration (at
    the start, part way through the step, or never)."""
    batch = isolated_halos(n=n, seed=seed, cosmology=cosmology, spin=spin)
    cosmo = cosmology or Cosmology()
    rng = np.random.Generator(np.random.Philox(key=seed + 2000))
    u = rng.random((3, n))
    mass = batch.param[_abi.P_MASS]
    hot = cosmo.omega_baryon / cosmo.omega_matter * mass * 10.0 ** (-3.0 + 2.5 * u[0])
    batch.state[_abi.Y_HOT_MASS] = hot
    batch.state[_abi.Y_HOT_METALS] = hot * 10.0 ** (-4.0 + np.log10(200.0) * u[1])
    batch.param[_abi.P_MASS_RATE] = mass * (0.05 + 0.45 * u[2])
    components = np.full(n, _abi.COMPONENT_SPHEROID | _abi.COMPONENT_BLACK_HOLE, dtype=np.int32)
    return batch, components


def isolated_params(tolerance_relative=1.0e-3):
    """P-std parameters with the batched-isolated-step tolerances."""
    p = _abi.default_params()
    p.ode_tolerance_relative = tolerance_relative
    return p
