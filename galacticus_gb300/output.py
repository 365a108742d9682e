"""Forest snapshots in the reference's output layout.

The reference's standard outputter (merger_trees/outputter/standard.F90)
writes, for output number i (output times in increasing order, counted from
1), a group Outputs/Output{i} with the attributes outputTime (Gyr),
outputExpansionFactor, timeUnitInSI, distanceUnitInSI and outputType
(:1290-1340), a subgroup nodeData holding one dataset per node property with
one entry per node that exists at that time (:280-290: nodes whose time is
the output time once the tree has been evolved to it), trees one after
another, and the per-tree datasets mergerTreeIndex, mergerTreeStartIndex and
mergerTreeCount locating each tree's block (:333-336).  The node properties
carry the component names of its output (diskMassStellar,
diskAbundancesGasMetals, hotHaloMass, basicMass, nodeIndex, ... as read by
testSuite/test-reproducibility.py:50-67).

HDF5 is absent on both machines this library runs on (no libhdf5, no h5py),
so write() puts the same tree of names into an uncompressed NumPy archive:
each dataset under its HDF5 path ("Outputs/Output1/nodeData/diskMassStellar")
and each attribute under "path@name".  read() gives back nested dictionaries
that are indexed like h5py groups (out["Outputs"]["Output1"]["nodeData"]...).
"""

import numpy as np

from . import _abi

# Reference property name of each evolved quantity (GAL_Y_*).  The standard
# spheroid's stellar metals are not among the evolved quantities here, so
# spheroidAbundancesStellarMetals is not written.
PROPERTY_NAMES = {
    _abi.Y_HOT_MASS: "hotHaloMass",
    _abi.Y_HOT_METALS: "hotHaloAbundancesMetals",
    _abi.Y_OUTFLOWED_MASS: "hotHaloOutflowedMass",
    _abi.Y_OUTFLOWED_METALS: "hotHaloOutflowedAbundancesMetals",
    _abi.Y_DISK_GAS: "diskMassGas",
    _abi.Y_DISK_GAS_METALS: "diskAbundancesGasMetals",
    _abi.Y_DISK_STARS: "diskMassStellar",
    _abi.Y_DISK_STARS_METALS: "diskAbundancesStellarMetals",
    _abi.Y_SPHEROID_GAS: "spheroidMassGas",
    _abi.Y_SPHEROID_GAS_METALS: "spheroidAbundancesGasMetals",
    _abi.Y_SPHEROID_STARS: "spheroidMassStellar",
    _abi.Y_BLACK_HOLE: "blackHoleMass",
}

GIGA_YEAR_SI = 3.15581497635456e16  # s
MEGA_PARSEC_SI = 3.08567758135e22  # m


def _satellite(forest):
    host = forest.satellite_host
    return np.zeros(forest.n, bool) if host is None else np.asarray(host) >= 0


def halo_mass(forest, node, t):
    """Basic (halo) mass of each node at time t, as the forest evolver's
    segments have it (dmoInterpolateNodeInitialize, nodes/operators/physics/
    dark_matter_only_mass/interpolate.F90:84-168, 217-239): a primary
    progenitor grows linearly by its parent's unresolved mass (the parent's
    mass beyond its other progenitors' and the satellites falling into it),
    every other node -- satellites included -- keeps its mass."""
    node = np.asarray(node)
    n = forest.n
    sat = _satellite(forest)
    host = np.full(n, -1) if forest.satellite_host is None else np.asarray(forest.satellite_host)
    par_all = forest.parent
    has_all = par_all >= 0
    brought = np.bincount(host[sat], weights=forest.mass[sat], minlength=n) + \
        np.bincount(par_all[has_all], weights=np.where(sat, 0.0, forest.mass)[has_all], minlength=n)
    par = forest.parent[node]
    t0 = forest.time[node]
    m0 = forest.mass[node]
    has = par >= 0
    p0 = np.where(has, par, 0)
    t1 = np.where(has, forest.time[p0], t0)
    primary = has & (forest.child_first[p0] == node) & (t1 > t0) & ~sat[node]
    dt = np.where(primary, t1 - t0, 1.0)
    rate = np.maximum(forest.mass[p0] - brought[p0], 0.0) / dt
    m1 = np.where(primary, m0 + rate * dt, m0)
    frac = np.where(primary, (t - t0) / dt, 0.0)
    return m0 + (m1 - m0) * frac


def layout(params, forest, output_times, snapshots, snapshot_node, snapshot_output):
    """The output tree as a flat dictionary {HDF5 path: array}, attributes
    under "path@name"."""
    from . import forest as forest_mod
    t_out = np.asarray(output_times, dtype=np.float64)
    if np.any(np.diff(t_out) <= 0.0):
        raise ValueError("output times must increase")
    snapshots = np.asarray(snapshots)
    snapshot_node = np.asarray(snapshot_node, dtype=np.int64)
    snapshot_output = np.asarray(snapshot_output, dtype=np.int64)
    if snapshots.shape != (_abi.NY, snapshot_node.size) or snapshot_output.shape != snapshot_node.shape:
        raise ValueError("snapshots must be [NY][m] with m node and output indices")
    if snapshot_node.size and (snapshot_node.min() < 0 or snapshot_node.max() >= forest.n or
                               snapshot_output.min() < 0 or snapshot_output.max() >= t_out.size):
        raise ValueError("snapshot node or output index out of range")
    out = {"Outputs@outputCount": np.int64(t_out.size)}
    for k, t in enumerate(t_out):
        g = f"Outputs/Output{k + 1}"
        sel = np.flatnonzero(snapshot_output == k)
        nodes = snapshot_node[sel]
        order = np.lexsort((nodes, forest.tree[nodes]))  # trees one after another, nodes in index order
        sel, nodes = sel[order], nodes[order]
        if np.unique(nodes).size != nodes.size:
            raise ValueError(f"node recorded twice at output {k + 1}")
        z = forest_mod.redshift(params, t)
        out[f"{g}@outputTime"] = np.float64(t)
        out[f"{g}@outputExpansionFactor"] = np.float64(1.0 / (1.0 + z))
        out[f"{g}@timeUnitInSI"] = np.float64(GIGA_YEAR_SI)
        out[f"{g}@distanceUnitInSI"] = np.float64(MEGA_PARSEC_SI)
        out[f"{g}@outputType"] = np.str_("standard")
        d = f"{g}/nodeData"
        out[f"{d}/nodeIndex"] = nodes.astype(np.int64)
        out[f"{d}/parentIndex"] = forest.parent[nodes].astype(np.int64)
        sat = _satellite(forest)[nodes]
        out[f"{d}/nodeIsIsolated"] = np.where(sat, 0, 1).astype(np.int64)
        out[f"{d}/basicMass"] = halo_mass(forest, nodes, t)
        # A satellite was last isolated at its infall (its phase's start).
        out[f"{d}/basicTimeLastIsolated"] = np.where(sat, forest.time[nodes], t)
        for y, name in PROPERTY_NAMES.items():
            out[f"{d}/{name}"] = snapshots[y, sel].astype(np.float64)
        trees, start, count = np.unique(forest.tree[nodes], return_index=True, return_counts=True)
        out[f"{g}/mergerTreeIndex"] = trees.astype(np.int64)
        out[f"{g}/mergerTreeStartIndex"] = start.astype(np.int64)
        out[f"{g}/mergerTreeCount"] = count.astype(np.int64)
    return out


def write(path, params, forest, output_times, snapshots, snapshot_node, snapshot_output):
    """Write the snapshots of an evolved forest (ForestEvolver.results) to
    path (a .npz archive) in the reference's output layout."""
    np.savez(path, **layout(params, forest, output_times, snapshots, snapshot_node, snapshot_output))


def read(path):
    """Nested dictionaries of a written file: groups are dicts, datasets
    arrays, a group's attributes in its "attrs" dict."""
    root = {"attrs": {}}
    with np.load(path, allow_pickle=False) as f:
        for key in f.files:
            path_part, _, attr = key.partition("@")
            node = root
            for part in path_part.split("/"):
                if attr or part != path_part.split("/")[-1]:
                    node = node.setdefault(part, {"attrs": {}})
                else:
                    node[part] = f[key]
            if attr:
                node["attrs"][attr] = f[key][()]
    return root
