"""Merger forests: the host tree builder and whole-forest evolution on the GPU.

Mirrors the reference's tree layer around the node evolver: trees from the
Cole et al. (2000) builder with Parkinson, Cole & Helly (2008) branching
(merger_trees/construct/builder/Cole2000/_class.F90:360-913), evolved node by
node to their parents' times with promotion and merging at each parent
(merger_trees/evolver/standard.F90:762-1035).  The arrays and their meaning
are those of include/galnode_forest.h.
"""

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi


TRANSFER_EISENSTEIN_HU_1999 = 0  # the reference's default transfer function
TRANSFER_EISENSTEIN_HU_1998 = 1


class PchParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("g0", "gamma1", "gamma2", "accuracy_first", "accuracy_second",
                                                "sigma8", "n_s", "temperature_cmb")] + \
               [("transfer_function", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("neutrino_number_effective", ctypes.c_double), ("neutrino_mass_summed", ctypes.c_double)]


SATELLITES_NONE = 0       # secondary progenitors merge at their parent's time
SATELLITES_JIANG2008 = 1  # satellites merge after the Jiang et al. (2008) time on a Benson (2005) orbit


class ForestSpec(ctypes.Structure):
    _fields_ = [("n_trees", ctypes.c_int64), ("seed", ctypes.c_uint64), ("root_mass_min", ctypes.c_double),
                ("root_mass_max", ctypes.c_double), ("root_mass_slope", ctypes.c_double),
                ("root_redshift", ctypes.c_double), ("redshift_max", ctypes.c_double),
                ("mass_resolution", ctypes.c_double), ("satellites", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("satellite_timescale_multiplier", ctypes.c_double)]


def _declare(lib):
    if getattr(lib, "_forest_declared", False):
        return lib
    vp = ctypes.c_void_p
    pp = ctypes.POINTER(_abi.Params)
    lib.gal_pch_params_default.argtypes = [ctypes.POINTER(PchParams)]
    lib.gal_pch_params_default.restype = None
    lib.gal_forest_build.argtypes = [pp, ctypes.POINTER(PchParams), ctypes.POINTER(ForestSpec), ctypes.POINTER(vp)]
    lib.gal_forest_build.restype = ctypes.c_int
    lib.gal_forest_node_count.argtypes = [vp]
    lib.gal_forest_node_count.restype = ctypes.c_int64
    lib.gal_forest_get.argtypes = [vp] * 8
    lib.gal_forest_get.restype = ctypes.c_int
    lib.gal_forest_free.argtypes = [vp]
    lib.gal_forest_free.restype = None
    lib.gal_forest_get_satellite_host.argtypes = [vp, vp]
    lib.gal_forest_get_satellite_host.restype = ctypes.c_int
    lib.gal_satellite_merging_time.argtypes = [pp] + [ctypes.c_double] * 6
    lib.gal_satellite_merging_time.restype = ctypes.c_double
    lib.gal_satellite_orbits.argtypes = [ctypes.c_uint64, ctypes.c_double, ctypes.c_int64, vp, vp]
    lib.gal_satellite_orbits.restype = ctypes.c_int
    lib.gal_cosmic_time.argtypes = [pp, ctypes.c_double]
    lib.gal_cosmic_time.restype = ctypes.c_double
    lib.gal_redshift.argtypes = [pp, ctypes.c_double]
    lib.gal_redshift.restype = ctypes.c_double
    lib.gal_pch_sigma.argtypes = [pp, ctypes.POINTER(PchParams), ctypes.c_double]
    lib.gal_pch_sigma.restype = ctypes.c_double
    lib.gal_pch_transfer.argtypes = [pp, ctypes.POINTER(PchParams), ctypes.c_double]
    lib.gal_pch_transfer.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    lib.gal_pch_branching_rates.argtypes = [ctypes.POINTER(PchParams)] + [ctypes.c_double] * 5 + [dp, dp]
    lib.gal_pch_branching_rates.restype = ctypes.c_int
    lib.gal_gpu_forest_build.argtypes = [vp, pp, ctypes.POINTER(PchParams), ctypes.POINTER(ForestSpec),
                                         ctypes.POINTER(vp)]
    lib.gal_gpu_forest_build.restype = ctypes.c_int
    lib.gal_pch_branch_tables.argtypes = [pp, ctypes.POINTER(PchParams), ctypes.POINTER(ForestSpec)] + [vp] * 7
    lib.gal_pch_branch_tables.restype = ctypes.c_int
    lib.gal_forest_build_stats.argtypes = [vp, vp]
    lib.gal_forest_build_stats.restype = ctypes.c_int
    lib.gal_gpu_forest_create.argtypes = [vp, ctypes.c_int64] + [vp] * 8 + [ctypes.c_int32, vp, ctypes.POINTER(vp)]
    lib.gal_gpu_forest_create.restype = ctypes.c_int
    for name in ("gal_gpu_forest_evolve", "gal_gpu_forest_sync"):
        getattr(lib, name).argtypes = [vp, vp]
        getattr(lib, name).restype = ctypes.c_int
    lib.gal_gpu_forest_snapshot_count.argtypes = [vp]
    lib.gal_gpu_forest_snapshot_count.restype = ctypes.c_int64
    lib.gal_gpu_forest_results.argtypes = [vp, vp] + [vp] * 6
    lib.gal_gpu_forest_results.restype = ctypes.c_int
    lib.gal_gpu_forest_accepted_steps.argtypes = [vp, vp]
    lib.gal_gpu_forest_accepted_steps.restype = ctypes.c_int64
    lib.gal_gpu_forest_autotune.argtypes = [vp, vp, ctypes.c_int32, vp]
    lib.gal_gpu_forest_autotune.restype = ctypes.c_int
    lib.gal_gpu_forest_free.argtypes = [vp]
    lib.gal_gpu_forest_free.restype = None
    lib._forest_declared = True
    return lib


def _vp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Forest:
    tree: np.ndarray
    parent: np.ndarray
    child_first: np.ndarray
    child_count: np.ndarray
    time: np.ndarray
    mass: np.ndarray
    spin: np.ndarray
    # For a satellite's phase (from its infall to its merger), the node it
    # fell into; -1 for every other node.  None: no satellites.
    satellite_host: np.ndarray = None
    # Where the build's time went (gal_forest_build_stats); None for forests
    # not made by build().
    build_stats: dict = None

    @property
    def n(self):
        return len(self.parent)

    @property
    def n_trees(self):
        return int(self.tree.max()) + 1 if self.n else 0

    def subset(self, trees):
        """The forest made of the given trees (ids of `tree`), node order
        kept, indices remapped and the trees renumbered 0.. in increasing
        order of their ids.  Returns (forest, [n_sub] original node index)."""
        keep = np.isin(self.tree, np.asarray(trees))
        idx = np.flatnonzero(keep)
        new = np.full(self.n, -1, np.int64)
        new[idx] = np.arange(len(idx))
        parent = self.parent[idx]
        parent = np.where(parent >= 0, new[np.maximum(parent, 0)], -1).astype(np.int32)
        count = self.child_count[idx].copy()
        first = np.where(count > 0, new[self.child_first[idx]], 0).astype(np.int32)
        _, renum = np.unique(self.tree[idx], return_inverse=True)
        host = None
        if self.satellite_host is not None:
            host = self.satellite_host[idx]
            host = np.where(host >= 0, new[np.maximum(host, 0)], -1).astype(np.int32)
        return Forest(renum.astype(np.int32), parent, first, count, self.time[idx].copy(), self.mass[idx].copy(),
                      self.spin[idx].copy(), host), idx


def lpt_assignment(forest, n_ranks):
    """Trees to ranks by longest processing time first, node count as the
    cost (the reference's work sharing hands out forests largest first,
    tasks/evolve_forests/work_share/_class.F90:37): trees in decreasing
    node count (ties by tree id) each go to the rank with the fewest nodes
    so far (ties to the lowest rank).  Returns one sorted array of tree ids
    per rank."""
    counts = np.bincount(forest.tree, minlength=forest.n_trees)
    order = np.lexsort((np.arange(len(counts)), -counts))
    load = np.zeros(n_ranks, dtype=np.int64)
    owner = np.empty(len(counts), dtype=np.int64)
    for t in order:
        r = int(np.argmin(load))
        owner[t] = r
        load[r] += counts[t]
    return [np.flatnonzero(owner == r) for r in range(n_ranks)]


def partition(forest, rank, n_ranks):
    """This rank's share of one forest (lpt_assignment): (sub-forest, [n]
    original node indices)."""
    return forest.subset(lpt_assignment(forest, n_ranks)[rank])


def pch_params():
    lib = _declare(_abi.load_library())
    p = PchParams()
    lib.gal_pch_params_default(ctypes.byref(p))
    return p


def _spec(n_trees, seed, root_mass_min, root_mass_max, root_mass_slope, redshift_max, mass_resolution, satellites,
          satellite_timescale_multiplier, root_redshift=0.0):
    return ForestSpec(n_trees, seed, root_mass_min, root_mass_max, root_mass_slope, root_redshift, redshift_max,
                      mass_resolution, satellites, 0, satellite_timescale_multiplier)


def build(params, n_trees, seed=3, root_mass_min=1e10, root_mass_max=1e14, root_mass_slope=-0.9, redshift_max=8.0,
          mass_resolution=1e8, pch=None, satellites=SATELLITES_NONE, satellite_timescale_multiplier=0.75, gpu=None,
          root_redshift=0.0):
    """Build a forest on the host (OpenMP over trees), or with its branches
    grown on the GPU of ``gpu`` (an evolver; gal_gpu_forest_build: the same
    builder with keyed per-branch streams, so other trees for the same
    seed).  With satellites=SATELLITES_JIANG2008 secondary progenitors
    orbit as satellites until their merging time (timescaleMultiplier as in
    the reference's quickTest, 0.75)."""
    lib = _declare(_abi.load_library())
    spec = _spec(n_trees, seed, root_mass_min, root_mass_max, root_mass_slope, redshift_max, mass_resolution,
                 satellites, satellite_timescale_multiplier, root_redshift)
    pch = pch or pch_params()
    handle = ctypes.c_void_p()
    if gpu is None:
        rc = lib.gal_forest_build(ctypes.byref(params), ctypes.byref(pch), ctypes.byref(spec), ctypes.byref(handle))
        if rc:
            raise RuntimeError(f"gal_forest_build failed ({rc})")
    else:
        from .evolver import _check
        _check(gpu.lib, gpu.ctx, lib.gal_gpu_forest_build(gpu.ctx, ctypes.byref(params), ctypes.byref(pch),
                                                          ctypes.byref(spec), ctypes.byref(handle)))
    n = lib.gal_forest_node_count(handle)
    # (every element is written by gal_forest_get)
    arrays = [np.empty(n, np.int32) for _ in range(4)] + [np.empty(n) for _ in range(3)]
    lib.gal_forest_get(handle, *[_vp(a) for a in arrays])
    host = None
    if satellites != SATELLITES_NONE:
        host = np.empty(n, np.int32)
        lib.gal_forest_get_satellite_host(handle, _vp(host))
    stats = np.zeros(7)
    lib.gal_forest_build_stats(handle, _vp(stats))
    lib.gal_forest_free(handle)
    return Forest(*arrays, host, build_stats=dict(tables_s=stats[0], gpu_growth_s=stats[1], download_renumber_s=stats[2],
                                                  per_tree_s=stats[3], assembly_s=stats[4], generations=int(stats[5]),
                                                  total_s=stats[6]))


def branch_tables(params, seed=3, root_mass_min=1e10, root_mass_max=1e14, redshift_max=8.0, mass_resolution=1e8,
                  pch=None, root_redshift=0.0):
    """The GPU branching's inputs for a forest (gal_pch_branch_tables): a
    dict with ``sizes``, ``meta`` and the tables ``ln_sigma``, ``rate``,
    ``accretion``, ``ln_q``, ``cdf``."""
    lib = _declare(_abi.load_library())
    spec = _spec(1, seed, root_mass_min, root_mass_max, -0.9, redshift_max, mass_resolution, SATELLITES_NONE, 0.75,
                 root_redshift)
    pch = pch or pch_params()
    sizes, meta = np.zeros(2, np.int32), np.zeros(10)
    args = (ctypes.byref(params), ctypes.byref(pch), ctypes.byref(spec))
    rc = lib.gal_pch_branch_tables(*args, _vp(sizes), _vp(meta), None, None, None, None, None)
    if rc:
        raise RuntimeError(f"gal_pch_branch_tables failed ({rc})")
    t = dict(sizes=sizes, meta=meta, ln_sigma=np.zeros(sizes[0]), rate=np.zeros(sizes[1]),
             accretion=np.zeros(sizes[1]), ln_q=np.zeros(sizes[1] * 96), cdf=np.zeros(sizes[1] * 96))
    lib.gal_pch_branch_tables(*args, _vp(sizes), _vp(meta), *[_vp(t[k]) for k in ("ln_sigma", "rate", "accretion",
                                                                                    "ln_q", "cdf")])
    return t


def satellite_orbits(n, mu=1.0, seed=1):
    """n orbits (radial, tangential velocity at the virial radius, units of
    the host's virial velocity) from the builder's Benson (2005) sampler."""
    lib = _declare(_abi.load_library())
    ur, ut = np.zeros(n), np.zeros(n)
    rc = lib.gal_satellite_orbits(seed, mu, n, _vp(ur), _vp(ut))
    if rc:
        raise RuntimeError(f"gal_satellite_orbits failed ({rc})")
    return ur, ut


def satellite_merging_time(params, mass_host, mass_satellite, t, velocity_radial, velocity_tangential,
                           multiplier=0.75):
    """The builder's Jiang et al. (2008) merging time (Gyr) for one orbit
    (velocities in units of the host's virial velocity); negative when the
    orbit is unbound."""
    lib = _declare(_abi.load_library())
    return lib.gal_satellite_merging_time(ctypes.byref(params), mass_host, mass_satellite, t, velocity_radial,
                                          velocity_tangential, multiplier)


def branching_rates(pch, alpha, sigma_parent, mass_parent, mass_resolution, w=1.686):
    """(split rate, sub-resolution accretion rate) per unit w of the
    builder, for sigma(M) = sigma_parent (M/mass_parent)^alpha."""
    lib = _declare(_abi.load_library())
    r, a = ctypes.c_double(), ctypes.c_double()
    rc = lib.gal_pch_branching_rates(ctypes.byref(pch), alpha, sigma_parent, mass_parent, mass_resolution, w,
                                     ctypes.byref(r), ctypes.byref(a))
    if rc:
        raise RuntimeError(f"gal_pch_branching_rates failed ({rc})")
    return r.value, a.value


def redshift(params, t):
    """Redshift at cosmic time t (Gyr) in the cosmology of params."""
    lib = _declare(_abi.load_library())
    return lib.gal_redshift(ctypes.byref(params), float(t))


def output_times(params, n=20, redshift_max=8.0):
    """n output times from redshift_max to 0, evenly spaced in ln(1+z)."""
    lib = _declare(_abi.load_library())
    z = (1.0 + redshift_max) ** (1.0 - np.arange(n) / (n - 1)) - 1.0
    z[-1] = 0.0
    return np.array([lib.gal_cosmic_time(ctypes.byref(params), float(zz)) for zz in z])


def initial_state(params, forest, black_hole_seed=100.0):
    """Initial states of the progenitor-less nodes: hot gas at the universal
    baryon fraction of the halo mass, primordial (metal-free), and a seed
    black hole; everything else empty."""
    state = np.zeros((_abi.NY, forest.n))
    state[_abi.Y_HOT_MASS] = params.omega_baryon / params.omega_matter * forest.mass
    state[_abi.Y_BLACK_HOLE] = black_hole_seed
    return state


class ForestEvolver:
    """A forest resident on the GPU of an evolver context (one CUDA graph per
    evolution)."""

    def __init__(self, evolver, forest, state0, times):
        self.lib = _declare(evolver.lib)
        self.ev = evolver
        self.forest = forest
        self.n = forest.n
        self._keep = [np.ascontiguousarray(a) for a in (forest.parent, forest.child_first, forest.child_count,
                                                         forest.time, forest.mass, forest.spin)]
        self.state0 = np.ascontiguousarray(state0, dtype=np.float64)
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        handle = ctypes.c_void_p()
        self._host = None if forest.satellite_host is None else np.ascontiguousarray(forest.satellite_host,
                                                                                    dtype=np.int32)
        rc = self.lib.gal_gpu_forest_create(evolver.ctx, self.n, *[_vp(a) for a in self._keep],
                                            None if self._host is None else _vp(self._host), _vp(self.state0),
                                            len(self.times), _vp(self.times), ctypes.byref(handle))
        if rc:
            raise RuntimeError(f"gal_gpu_forest_create failed ({rc}): {self._message()}")
        self.handle = handle

    def _message(self):
        buf = ctypes.create_string_buffer(512)
        self.lib.gal_gpu_last_error(self.ev.ctx, buf, 512)
        return buf.value.decode()

    def evolve(self, sync=True):
        rc = self.lib.gal_gpu_forest_evolve(self.ev.ctx, self.handle)
        if rc:
            raise RuntimeError(f"gal_gpu_forest_evolve failed ({rc}): {self._message()}")
        if sync:
            self.sync()

    def sync(self):
        rc = self.lib.gal_gpu_forest_sync(self.ev.ctx, self.handle)
        if rc:
            raise RuntimeError(f"forest evolution failed ({rc}): {self._message()}")

    def results(self, snapshots=True):
        """(state, status, counters, snapshots, snapshot node, snapshot output);
        the last three are None with snapshots=False."""
        m = self.lib.gal_gpu_forest_snapshot_count(self.handle) if snapshots else 0
        state = np.zeros((_abi.NY, self.n))
        status = np.zeros(self.n, np.int32)
        counters = np.zeros((3, self.n), np.uint32)
        snap = np.zeros((_abi.NY, max(m, 1))) if snapshots else None
        snap_node = np.zeros(max(m, 1), np.int32) if snapshots else None
        snap_out = np.zeros(max(m, 1), np.int32) if snapshots else None
        vp = lambda a: None if a is None else _vp(a)
        rc = self.lib.gal_gpu_forest_results(self.ev.ctx, self.handle, _vp(state), _vp(status), _vp(counters), vp(snap),
                                             vp(snap_node), vp(snap_out))
        if rc:
            raise RuntimeError(f"gal_gpu_forest_results failed ({rc}): {self._message()}")
        if not snapshots:
            return state, status, counters, None, None, None
        return state, status, counters, snap[:, :m], snap_node[:m], snap_out[:m]

    def snapshot_count(self):
        return int(self.lib.gal_gpu_forest_snapshot_count(self.handle))

    def accepted_steps(self):
        return int(self.lib.gal_gpu_forest_accepted_steps(self.ev.ctx, self.handle))

    def autotune(self, repeats=3):
        times = np.full(8, -1.0)
        rc = self.lib.gal_gpu_forest_autotune(self.ev.ctx, self.handle, repeats, _vp(times))
        if rc:
            raise RuntimeError(f"gal_gpu_forest_autotune failed ({rc}): {self._message()}")
        return times[:6]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gal_gpu_forest_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
