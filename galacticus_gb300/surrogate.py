"""The learned cooling-function surrogate: data, training, error map, install.

The reference evaluates the cooling function by log-log bilinear
interpolation in a CIE table (cooling/cooling_function/CIE_file.F90:238-317,
665-735).  A 3-64-64-64-1 SiLU network learns
log10 Lambda(log10 T, log10 Z/Zsun, log10 n_H) from samples of exactly that
interpolation (``cooling_samples``), is trained on the GPU by the project's
own FP32 forward/backward and Adam kernels (``gal_surrogate_train``), and is
installed in an evolution context, where the integrator evaluates it on the
tensor cores (BF16 products, FP32 accumulation) instead of the table.  The
table remains the fallback outside the training domain and in the cells of
an error map where the deployed network misses it by more than ``tolerance``
dex.

The cooling function scales exactly as n_H^2 (CIE_file.F90:514-533), so the
network output is log10 Lambda - 2 log10 n_H (normalised): that dependence
is a fixed term and the network learns the temperature and metallicity
dependence, with n_H still an input.
"""

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _abi

N_PARAMS = 64 * 3 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1
DOMAIN_LO = np.array([4.0, -4.0, -6.0], dtype=np.float32)  # log10 T, log10 Z/Zsun, log10 n_H
DOMAIN_HI = np.array([8.5, 0.5, 0.0], dtype=np.float32)


class TrainConfig(ctypes.Structure):
    _fields_ = [("batch_size", ctypes.c_int64), ("epochs", ctypes.c_int32), ("seed", ctypes.c_int32),
                ("learning_rate", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("epsilon", ctypes.c_float), ("learning_rate_final", ctypes.c_float)]


class SurrogateStruct(ctypes.Structure):
    _fields_ = [("params", ctypes.POINTER(ctypes.c_float)),
                ("in_mean", ctypes.c_float * 3), ("in_scale", ctypes.c_float * 3),
                ("y_mean", ctypes.c_float), ("y_scale", ctypes.c_float),
                ("lo", ctypes.c_float * 3), ("hi", ctypes.c_float * 3),
                ("map_t", ctypes.c_int32), ("map_z", ctypes.c_int32),
                ("map_lo_t", ctypes.c_float), ("map_lo_z", ctypes.c_float),
                ("map_dt", ctypes.c_float), ("map_dz", ctypes.c_float),
                ("use_table", ctypes.POINTER(ctypes.c_uint8))]


def _declare(lib):
    if getattr(lib, "_surrogate_declared", False):
        return lib
    fp = ctypes.POINTER(ctypes.c_float)
    lib.gal_surrogate_param_count.restype = ctypes.c_int
    lib.gal_surrogate_train.argtypes = [ctypes.POINTER(TrainConfig), fp, fp, ctypes.c_int64, fp, fp, ctypes.c_int64, fp, fp]
    lib.gal_surrogate_train.restype = ctypes.c_int
    lib.gal_surrogate_gradient.argtypes = [fp, fp, fp, ctypes.c_int64, fp, fp]
    lib.gal_surrogate_gradient.restype = ctypes.c_int
    lib.gal_surrogate_predict.argtypes = [fp, fp, ctypes.c_int64, fp, ctypes.c_int32]
    lib.gal_surrogate_predict.restype = ctypes.c_int
    lib.gal_gpu_set_surrogate.argtypes = [ctypes.c_void_p, ctypes.POINTER(SurrogateStruct)]
    lib.gal_gpu_set_surrogate.restype = ctypes.c_int
    lib.gal_gpu_set_surrogate_split.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.gal_gpu_set_surrogate_split.restype = ctypes.c_int
    lib.gal_gpu_surrogate_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    lib.gal_gpu_surrogate_stats.restype = ctypes.c_int
    lib._surrogate_declared = True
    return lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def cie_log10_lambda(table, log10_t, log10_z, log10_nh):
    """log10 of the cooling function (erg cm^-3 s^-1) by the reference's CIE
    interpolation (CIE_file.F90:238-317, 665-735), vectorised: T clamped to
    the table ("extrapolate" as implemented), Z fixed at the table limits, a
    Z = 0 row interpolated linearly in Z, bilinear in (ln T, ln Z) of ln
    Lambda, times n_H^2."""
    t = np.clip(10.0 ** np.asarray(log10_t, dtype=np.float64), table.temperature[0], table.temperature[-1])
    z = np.clip(10.0 ** np.asarray(log10_z, dtype=np.float64), table.metallicity[0], table.metallicity[-1])
    ln_t_grid = np.log(table.temperature)
    ln_l = np.log(table.cooling_rate)
    ln_t = np.log(t)
    it = np.clip(np.searchsorted(ln_t_grid, ln_t, side="right") - 1, 0, len(ln_t_grid) - 2)
    ht = (ln_t - ln_t_grid[it]) / (ln_t_grid[it + 1] - ln_t_grid[it])
    zg = table.metallicity
    first_zero = zg[0] == 0.0
    iz = np.zeros_like(it)
    hz = np.zeros_like(ht)
    low = first_zero & (z < zg[1]) if first_zero else np.zeros(z.shape, dtype=bool)
    if first_zero:
        iz[low] = 0
        hz[low] = z[low] / zg[1]
    ln_zg = np.where(zg > 0, np.log(np.where(zg > 0, zg, 1.0)), -999.0)
    hi = ~low
    ln_z = np.log(np.where(z > 0, z, 1e-300))
    j = np.clip(np.searchsorted(ln_zg, ln_z, side="right") - 1, 0, len(zg) - 2)
    iz[hi] = j[hi]
    hz[hi] = ((ln_z - ln_zg[j]) / (ln_zg[j + 1] - ln_zg[j]))[hi]
    f = (ln_l[iz, it] * (1 - ht) * (1 - hz) + ln_l[iz + 1, it] * (1 - ht) * hz
         + ln_l[iz, it + 1] * ht * (1 - hz) + ln_l[iz + 1, it + 1] * ht * hz)
    return f / np.log(10.0) + 2.0 * np.asarray(log10_nh, dtype=np.float64)


def cooling_samples(table, n, seed=4):
    """n samples uniform in the training domain and their log10 Lambda."""
    rng = np.random.Generator(np.random.Philox(key=seed))
    x = DOMAIN_LO + (DOMAIN_HI - DOMAIN_LO) * rng.random((n, 3))
    y = cie_log10_lambda(table, x[:, 0], x[:, 1], x[:, 2])
    return x.astype(np.float64), y


def init_params(seed=4):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases."""
    rng = np.random.Generator(np.random.Philox(key=seed + 1000))
    p = np.zeros(N_PARAMS, dtype=np.float32)
    o = 0
    for fan_in, fan_out in ((3, 64), (64, 64), (64, 64), (64, 1)):
        b = 1.0 / np.sqrt(fan_in)
        p[o:o + fan_in * fan_out] = rng.uniform(-b, b, fan_in * fan_out)
        o += fan_in * fan_out + fan_out
    return p


@dataclass
class CoolingSurrogate:
    params: np.ndarray
    in_mean: np.ndarray
    in_scale: np.ndarray
    y_mean: float
    y_scale: float
    tolerance: float = 0.01
    map_lo: tuple = (4.0, -4.0)
    map_step: tuple = (0.05, 0.125)
    use_table: np.ndarray = field(default=None)
    history: np.ndarray = field(default=None)
    rms_dex: float = float("nan")

    def normalise(self, x):
        return ((np.asarray(x, dtype=np.float64) - self.in_mean) / self.in_scale).astype(np.float32)

    def predict(self, x, tensor_cores=True):
        """log10 Lambda of the network (tensor-core BF16 path by default)."""
        lib = _declare(_abi.load_library())
        x = np.asarray(x, dtype=np.float64)
        xn = np.ascontiguousarray(self.normalise(x))
        out = np.zeros(len(xn), dtype=np.float32)
        p = np.ascontiguousarray(self.params, dtype=np.float32)
        rc = lib.gal_surrogate_predict(_fp(p), _fp(xn), len(xn), _fp(out), 1 if tensor_cores else 0)
        if rc:
            raise RuntimeError(f"gal_surrogate_predict failed ({rc})")
        return out.astype(np.float64) * self.y_scale + self.y_mean + 2.0 * x[:, 2]

    def struct(self):
        lib = _declare(_abi.load_library())
        assert self.use_table is not None, "build the error map first"
        self._p = np.ascontiguousarray(self.params, dtype=np.float32)
        self._map = np.ascontiguousarray(self.use_table, dtype=np.uint8)
        s = SurrogateStruct()
        s.params = _fp(self._p)
        for i in range(3):
            s.in_mean[i] = self.in_mean[i]
            s.in_scale[i] = self.in_scale[i]
            s.lo[i] = DOMAIN_LO[i]
            s.hi[i] = DOMAIN_HI[i]
        s.y_mean, s.y_scale = self.y_mean, self.y_scale
        s.map_t, s.map_z = self._map.shape
        s.map_lo_t, s.map_lo_z = self.map_lo
        s.map_dt, s.map_dz = self.map_step
        s.use_table = self._map.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        return s

    def install(self, evolver):
        lib = _declare(evolver.lib)
        s = self.struct()
        self._struct = s
        rc = lib.gal_gpu_set_surrogate(evolver.ctx, ctypes.byref(s))
        if rc:
            buf = ctypes.create_string_buffer(512)
            lib.gal_gpu_last_error(evolver.ctx, buf, 512)
            raise RuntimeError(f"gal_gpu_set_surrogate failed: {buf.value.decode()}")

    def uninstall(self, evolver):
        """Remove the surrogate from the context: the table alone again."""
        lib = _declare(evolver.lib)
        rc = lib.gal_gpu_set_surrogate(evolver.ctx, None)
        if rc:
            raise RuntimeError(f"gal_gpu_set_surrogate(NULL) failed ({rc})")

    def build_error_map(self, table, tolerance=None, per_cell=64, seed=7):
        """Mark the (log10 T, log10 Z) cells where the deployed network misses
        the table by more than `tolerance` dex at any of `per_cell` random
        points (n_H enters exactly as 2 log10 n_H, so it is sampled freely)."""
        if tolerance is not None:
            self.tolerance = tolerance
        nt = int(round((DOMAIN_HI[0] - DOMAIN_LO[0]) / self.map_step[0]))
        nz = int(round((DOMAIN_HI[1] - DOMAIN_LO[1]) / self.map_step[1]))
        rng = np.random.Generator(np.random.Philox(key=seed))
        it = np.repeat(np.arange(nt), nz * per_cell)
        iz = np.tile(np.repeat(np.arange(nz), per_cell), nt)
        u = rng.random((len(it), 3))
        x = np.empty((len(it), 3))
        x[:, 0] = self.map_lo[0] + (it + u[:, 0]) * self.map_step[0]
        x[:, 1] = self.map_lo[1] + (iz + u[:, 1]) * self.map_step[1]
        x[:, 2] = DOMAIN_LO[2] + (DOMAIN_HI[2] - DOMAIN_LO[2]) * u[:, 2]
        err = np.abs(self.predict(x) - cie_log10_lambda(table, x[:, 0], x[:, 1], x[:, 2]))
        worst = err.reshape(nt, nz, per_cell).max(axis=2)
        self.use_table = (worst > self.tolerance).astype(np.uint8)
        self.cell_error = worst
        return self.use_table


def train(table, n_samples=2_000_000, epochs=20, batch_size=256, learning_rate=1e-3, seed=4, validation=0.1,
          tolerance=0.01, learning_rate_final=1e-5):
    """Train the surrogate on the GPU on samples of the table interpolation
    (90/10 train/validation split) and build its error map.  Adam starts at
    ``learning_rate`` and decays on a cosine to ``learning_rate_final``
    (pass ``learning_rate_final=learning_rate`` for a constant rate)."""
    lib = _declare(_abi.load_library())
    x, y_total = cooling_samples(table, n_samples, seed)
    y = y_total - 2.0 * x[:, 2]  # the exact n_H^2 scaling is a fixed term
    n_val = int(round(validation * n_samples))
    n_train = n_samples - n_val
    in_mean = (DOMAIN_LO + DOMAIN_HI).astype(np.float64) / 2.0
    in_scale = (DOMAIN_HI - DOMAIN_LO).astype(np.float64) / 2.0
    y_mean = float(y[:n_train].mean())
    y_scale = float(y[:n_train].std())
    xn = ((x - in_mean) / in_scale).astype(np.float32)
    yn = ((y - y_mean) / y_scale).astype(np.float32)
    x_tr, y_tr = np.ascontiguousarray(xn[:n_train]), np.ascontiguousarray(yn[:n_train])
    x_va, y_va = np.ascontiguousarray(xn[n_train:]), np.ascontiguousarray(yn[n_train:])
    params = init_params(seed)
    history = np.zeros(2 * epochs, dtype=np.float32)
    cfg = TrainConfig(batch_size, epochs, seed, learning_rate, 0.9, 0.999, 1e-8, learning_rate_final)
    rc = lib.gal_surrogate_train(ctypes.byref(cfg), _fp(x_tr), _fp(y_tr), n_train, _fp(x_va), _fp(y_va), n_val,
                                 _fp(params), _fp(history))
    if rc:
        raise RuntimeError(f"gal_surrogate_train failed ({rc})")
    s = CoolingSurrogate(params, in_mean, in_scale, y_mean, y_scale, tolerance=tolerance,
                         history=history.reshape(epochs, 2))
    s.rms_dex = float(np.sqrt(history[-1]) * y_scale)
    s.build_error_map(table)
    return s


def gradient(params, x_norm, y_norm):
    """Loss and gradient from the training kernels (for gradient checks)."""
    lib = _declare(_abi.load_library())
    p = np.ascontiguousarray(params, dtype=np.float32)
    xn = np.ascontiguousarray(x_norm, dtype=np.float32)
    yn = np.ascontiguousarray(y_norm, dtype=np.float32)
    g = np.zeros(N_PARAMS, dtype=np.float32)
    loss = ctypes.c_float()
    rc = lib.gal_surrogate_gradient(_fp(p), _fp(xn), _fp(yn), len(yn), _fp(g), ctypes.byref(loss))
    if rc:
        raise RuntimeError(f"gal_surrogate_gradient failed ({rc})")
    return loss.value, g


def set_split(evolver, split):
    """The batch launch with a surrogate: split (default) or one kernel."""
    lib = _declare(evolver.lib)
    rc = lib.gal_gpu_set_surrogate_split(evolver.ctx, 1 if split else 0)
    if rc:
        raise RuntimeError(f"gal_gpu_set_surrogate_split failed ({rc})")


def stats(evolver):
    lib = _declare(evolver.lib)
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    lib.gal_gpu_surrogate_stats(evolver.ctx, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value
