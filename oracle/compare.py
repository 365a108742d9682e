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


# ---- per-halo final-mass criterion ----------------------------------------
# The target of the surrogate form: final stellar (disk + spheroid stars)
# and cold-gas (disk + spheroid gas) masses within 1e-3 relative of the FP64
# oracle, halo by halo, over halos whose oracle mass is above 1e6 Msun.

MASS_MINIMUM = 1.0e6
MASS_BAR = 1.0e-3
SUMS = (("stellar", (_abi.Y_DISK_STARS, _abi.Y_SPHEROID_STARS)),
        ("cold_gas", (_abi.Y_DISK_GAS, _abi.Y_SPHEROID_GAS)))


def mass_sums(state):
    """{name: [n] stellar / cold-gas mass} of a [NY][n] state."""
    return {name: state[a] + state[b] for name, (a, b) in SUMS}


def relative_mass_errors(gpu, ref):
    """{name: ([n] |gpu/ref - 1|, [n] mask ref > 1e6 Msun)}."""
    g, r = mass_sums(gpu), mass_sums(ref)
    out = {}
    for name in g:
        big = r[name] > MASS_MINIMUM
        rel = np.zeros_like(r[name])
        rel[big] = np.abs(g[name][big] / r[name][big] - 1.0)
        out[name] = (rel, big)
    return out


def mass_movement(ref, moved):
    """[n] largest relative change of the stellar or cold-gas mass between
    the oracle's answer and each of the `moved` answers (halos below 1e6 Msun
    count as not moving)."""
    r = mass_sums(ref)
    worst = np.zeros(ref.shape[1])
    for m in moved:
        s = mass_sums(m)
        for name in r:
            big = r[name] > MASS_MINIMUM
            d = np.zeros_like(worst)
            d[big] = np.abs(s[name][big] / r[name][big] - 1.0)
            worst = np.maximum(worst, d)
    return worst


def perturbed_table(table, dex):
    """The CIE table with every cooling rate multiplied by 10^dex."""
    from galacticus_gb300.cie_tables import CieTable
    return CieTable(table.temperature, table.metallicity, table.cooling_rate * 10.0 ** dex, table.electron_density)


def conditioning(oracle_mod, params, table, batch, ref, lambda_dex=1.0e-4, threads=0):
    """How well the oracle's own stellar and cold-gas masses are determined,
    per halo: the largest relative change under (a) the relative tolerance
    x0.9 and x1.1 (the integration) and (b) the cooling function scaled by
    10^(+-lambda_dex) (Lambda known to 1e-4 dex, a tenth of the tightest
    error gate).  Returns ([n] movement, [NY][n] worst absolute change of
    every property under (a) and (b))."""
    from galacticus_gb300 import workloads
    moved = []
    for factor in (0.9, 1.1):
        q = workloads.isolated_params(tolerance_relative=params.ode_tolerance_relative * factor)
        moved.append(oracle_mod.evolve_batch(q, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                             batch.step, threads=threads)[0])
    for dex in (lambda_dex, -lambda_dex):
        moved.append(oracle_mod.evolve_batch(params, perturbed_table(table, dex), batch.state, batch.param,
                                             batch.t_start, batch.t_end, batch.step, threads=threads)[0])
    sensitivity = np.max([np.abs(m - ref) for m in moved], axis=0)
    return mass_movement(ref, moved), sensitivity


def bar_shares(gpu, ref, movement):
    """Per-halo shares within the 1e-3 bar: over all halos above 1e6 Msun
    ("all"), and over those whose oracle masses move by less than the bar
    under conditioning() ("conditioned").  {name: {...}} plus the worst
    errors."""
    errs = relative_mass_errors(gpu, ref)
    good = movement <= MASS_BAR
    out = {}
    for name, (rel, big) in errs.items():
        out[name] = {"all": float(np.mean(rel[big] <= MASS_BAR)),
                     "conditioned": float(np.mean(rel[big & good] <= MASS_BAR)),
                     "p99": float(np.percentile(rel[big], 99)), "max": float(rel[big].max()),
                     "max_conditioned": float(rel[big & good].max())}
    out["ill_conditioned"] = float(np.mean(~good))
    out["min_conditioned"] = min(out[n]["conditioned"] for n, _ in SUMS)
    out["min_all"] = min(out[n]["all"] for n, _ in SUMS)
    return out


def select_gate(run, ref, movement, gates, share=0.995):
    """Pick the loosest error-map gate of the cooling surrogate whose final
    stellar and cold-gas masses meet the 1e-3 bar halo by halo: at least
    `share` of the well-conditioned halos above 1e6 Msun within 1e-3 of the
    oracle, for both masses.  `gates` run from loose to tight; a gate of
    None is the table alone (the network never used).  run(gate) returns
    (final state, network share of the cooling evaluations).  Every gate is
    run (the records show the trade-off).  Returns (chosen gate, {gate:
    record}); None when only the table meets the bar."""
    results = {}
    chosen = None
    for gate in gates:
        state, net_share = run(gate)
        rec = bar_shares(state, ref, movement)
        rec["network_share"] = net_share
        rec["meets_bar"] = rec["min_conditioned"] >= share
        results[gate] = rec
        if rec["meets_bar"] and chosen is None:
            chosen = gate
    return chosen, results
