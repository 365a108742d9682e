#!/usr/bin/env python3
"""Benchmark of the node-evolution hot path on GB300.

Metric: node-timesteps/s (accepted adaptive Cash-Karp steps of one node per
second) of the batched isolated-halo step: 65,536 halos per GPU, each
advanced over one timestep at relative tolerance 1e-3 (P-std physics).  A
"step" of this benchmark is one evolve pass over the whole batch.

The headline form is the batched surrogate form: FP64 state, error norm and
step control, FP32 rates, and the cooling function from the learned MLP
surrogate (trained here on the GPU, 2M samples, 20 epochs) with the table as
fallback, at the loosest error-map gate (0.01 dex, then tighter) whose
final stellar and cold-gas masses stay within 1e-3 of the FP64 oracle in
total.  The plain FP64 form, the FP32-rate form without the network and the
surrogate form at the 0.01-dex gate are timed beside it in the same run, with
their final-mass errors.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs one process per GPU under torch.distributed.run with no
collective on the data path (weak scaling): every rank evolves its own batch
of independent halos, and the uneven-trees forest (4,096 trees per rank) is
one forest split over the ranks by longest processing time first on node
counts; rank 0 prints the JSON line with the max-over-ranks time.

`--impl reference` times the reference algorithm on the host CPU.  The
Fortran reference cannot be built in this environment (no gfortran, GSL,
HDF5 or FoX), so that arm runs the C++ restatement in oracle/ with every
host thread.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "node-timesteps/s on 1 GB300: batched+surrogate vs plain GPU at <=1e-3 mass error"
UNIT = "node-timesteps/s"
N_NODES = 65536
WORKLOAD = "isolated-halo step: 65,536 halos/GPU, M 1e10-1e14 Msun, dt 0.01-1 Gyr, rel tol 1e-3, P-std physics"
TREES_WORKLOAD = ("uneven trees: {} PCH trees (seed 3), roots dN/dlnM ~ M^-0.9 on 1e10-1e14 Msun, resolution "
                  "1e8 Msun, z=8->0 with 20 outputs, rel tol 1e-3{}")
SATELLITES = {"jiang2008": 1, "none": 0}


def satellite_note(args):
    return ("; satellites merge after the Jiang et al. (2008) time (x0.75) on Benson (2005) orbits"
            if args.satellites == "jiang2008" else "; secondary progenitors merge at their parent's time")
# Error-map gates tried for the surrogate form (dex), loose to tight; the
# table alone comes after them.
GATES = (0.01, 0.003, 0.001, 0.0003, 0.0001)
MLP_FLOPS = 2 * (3 * 64 + 64 * 64 + 64 * 64 + 64)  # per network evaluation
# dram__bytes_read.sum + dram__bytes_write.sum of the headline launch (the
# surrogate form's two kernels on this workload) from one ncu --set full
# capture, per pass, and the same capture's FP64 pipe utilisation
# (sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active) of each
# kernel, each timed alone.
HEADLINE_DRAM_BYTES = 8.952064e6 + 10.888192e6
HEADLINE_FP64_PIPE_PCT = {"network kernel": 3.17, "table kernel": 27.19}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nodes", type=int, default=N_NODES)
    ap.add_argument("--form", choices=["compare", "plain", "fast", "surrogate", "trees-plain", "trees-fast",
                                       "trees-surrogate"], default="compare",
                    help="compare: the headline run; otherwise time one form alone (for profiling)")
    ap.add_argument("--gate", type=float, default=0.003,
                    help="error-map tolerance of --form surrogate and --workload scale (dex; 0: the table alone)")
    ap.add_argument("--trees", type=int, default=4096, help="trees of the uneven-trees workload (0: skip it)")
    ap.add_argument("--tree-steps", type=int, default=2, help="timed evolutions of the whole forest per form")
    ap.add_argument("--workload", choices=["isolated", "scale"], default="isolated",
                    help="scale: the full chosen form on a forest at scale (one JSON line of its own)")
    ap.add_argument("--trees-scale", type=int, default=65536, help="trees of the scale workload (0: skip it)")
    ap.add_argument("--satellites", choices=sorted(SATELLITES), default="jiang2008",
                    help="forests: satellites as the reference's default classes have them, or none")
    ap.add_argument("--halo", type=int, default=-1,
                    help="with a single --form: evolve only this halo of the batch (profiling the batch's tail)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_flops_per_step(params, table, batch, weights_path, sample=512):
    """Weighted FP64 flops per accepted node-timestep, counted by the oracle's
    counting scalar on a sample of the batch (closed-form cooling radius, as
    the kernel computes it)."""
    from oracle import oracle
    with open(weights_path) as f:
        w = json.load(f)
    weights = np.array([w[k] for k in w["order"]], dtype=np.float64)
    total, steps = 0.0, 0
    idx = np.linspace(0, batch.n - 1, min(sample, batch.n)).astype(int)
    for i in idx:
        ops, counters = oracle.count_flops(params, table, batch.param[:, i], batch.state[:, i], batch.t_start[i],
                                           batch.t_end[i], batch.step[i])
        total += float(np.dot(ops.astype(np.float64), weights))
        steps += int(counters[0])
    return total / max(steps, 1)


def reduce_over_ranks(dist, device, elapsed, work=None):
    """Weak scaling over the ranks of one node: every rank evolves its own
    halos or trees (no collective on the data path), so the job's time is the
    slowest rank's (max) and its work the sum over ranks.  Returns
    (elapsed, work) unchanged without a process group."""
    if not dist:
        return elapsed, work
    import torch
    t = torch.tensor([float(elapsed)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if work is not None:
        w = torch.tensor([int(work)], device=device, dtype=torch.int64)
        dist.all_reduce(w, op=dist.ReduceOp.SUM)
        work = int(w.item())
    return float(t.item()), work


def gather_ranks(dist, device, values):
    """Every rank's list of numbers, in rank order (rank 0 reports them);
    [values] without a process group."""
    if not dist:
        return [list(values)]
    import torch
    mine = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    every = [torch.zeros_like(mine) for _ in range(dist.get_world_size())]
    dist.all_gather(every, mine)
    return [e.tolist() for e in every]


def cpu_baseline(params, table, batch, seconds=10.0):
    """The oracle on every host core over repeats of the full batch; returns
    the baseline record and the final state of the first pass."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    t_start = time.perf_counter()
    steps = reps = 0
    first = None
    while True:
        out, _, status, counters = oracle.evolve_batch(params, table, batch.state, batch.param, batch.t_start,
                                                       batch.t_end, batch.step, threads=cores, brent=True)
        if first is None:
            first = out
        steps += int(counters[0].sum())
        reps += 1
        elapsed = time.perf_counter() - t_start
        if elapsed >= seconds:
            break
    return ({"value": steps / elapsed, "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"{reps} passes over the {batch.n}-halo batch ({elapsed:.1f} s, Brent cooling radius as in the reference)"},
            first)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from galacticus_gb300 import workloads
    from galacticus_gb300.cie_tables import CieTable
    from oracle import oracle
    params = workloads.isolated_params()
    table = CieTable()
    batch = workloads.isolated_halos(n=args.nodes, seed=2)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step, threads=cores)
    times, steps = [], 0
    # Each step is a bounded sample: the full batch (about 0.1 s of CPU work per pass).
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, _, counters = oracle.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                batch.step, threads=cores, brent=True)
        times.append(time.perf_counter() - t0)
        steps += int(counters[0].sum())
    value = steps / sum(times)
    # The same passes with the closed-form cooling radius the GPU kernels use
    # (exact for this cooling model; the reference finds it by Brent's
    # method): the share of the GPU's speed-up that is the algorithm's.
    tc, steps_c = 0.0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, _, counters = oracle.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end,
                                                batch.step, threads=cores, brent=False)
        tc += time.perf_counter() - t0
        steps_c += int(counters[0].sum())
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox halos)",
        "config": {"workload": WORKLOAD, "nodes": args.nodes, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} passes over the {args.nodes}-halo batch; C++ restatement of the "
                                   "reference algorithm (the Fortran reference is not buildable here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "closed_form_cooling_radius": {"value": steps_c / tc, "unit": UNIT,
                                       "note": "the same passes with the GPU kernels' closed-form cooling radius "
                                               "instead of the reference's Brent root (informative; value is the "
                                               "reference's algorithm)"},
    }
    print(json.dumps(line), flush=True)


def oracle_mod():
    from oracle import oracle
    return oracle


def lambda_sensitivity(params, table, batch, ref, dexes=(1e-4, 3e-4, 1e-3, 3e-3, 1e-2)):
    """What a systematic error in Lambda does to the per-halo bar: the
    oracle rerun with every cooling rate scaled by 10^dex, and the share of
    halos above 1e6 Msun whose stellar and cold-gas masses stay within 1e-3
    (a network used in a halo's cells shifts its Lambda by about its
    deployed error there)."""
    from oracle import compare, oracle
    out = {}
    for dex in dexes:
        m = oracle.evolve_batch(params, compare.perturbed_table(table, dex), batch.state, batch.param, batch.t_start,
                                batch.t_end, batch.step, threads=os.cpu_count() or 1)[0]
        errs = compare.relative_mass_errors(m, ref)
        out[str(dex)] = {name: {"share_within_1e-3": float(np.mean(rel[big] <= 1e-3)),
                                "p99": float(np.percentile(rel[big], 99))} for name, (rel, big) in errs.items()}
    return out


def mass_errors(gpu, ref):
    """Final stellar (disk + spheroid stars) and cold-gas (disk + spheroid
    gas) masses against the FP64 oracle: relative error of the population
    total, and per-halo quantiles over halos above 1e6 Msun."""
    from galacticus_gb300 import _abi
    out = {}
    for name, idx in (("stellar", (_abi.Y_DISK_STARS, _abi.Y_SPHEROID_STARS)),
                      ("cold_gas", (_abi.Y_DISK_GAS, _abi.Y_SPHEROID_GAS))):
        g = gpu[idx[0]] + gpu[idx[1]]
        r = ref[idx[0]] + ref[idx[1]]
        big = r > 1e6
        rel = np.abs(g[big] / r[big] - 1.0)
        out[name] = {"total": float(abs(g.sum() / r.sum() - 1.0)), "median": float(np.median(rel)),
                     "p99": float(np.percentile(rel, 99)), "max": float(rel.max()),
                     "share_within_1e-3": float(np.mean(rel <= 1e-3))}
    out["max_total"] = max(out["stellar"]["total"], out["cold_gas"]["total"])
    return out


def forest_mass_errors(state, ref, forest_):
    """Root-level final stellar and cold-gas masses of a forest against the
    FP64 oracle: relative error of the totals and per-root quantiles."""
    from galacticus_gb300 import _abi
    roots = forest_.parent < 0
    out = {}
    for name, idx in (("stellar", (_abi.Y_DISK_STARS, _abi.Y_SPHEROID_STARS)),
                      ("cold_gas", (_abi.Y_DISK_GAS, _abi.Y_SPHEROID_GAS))):
        g = state[idx[0]][roots] + state[idx[1]][roots]
        r = ref[idx[0]][roots] + ref[idx[1]][roots]
        big = r > 1e6
        rel = np.abs(g[big] / r[big] - 1.0)
        out[name] = {"total": float(abs(g.sum() / r.sum() - 1.0)), "median": float(np.median(rel)),
                     "p99": float(np.percentile(rel, 99)), "max": float(rel.max())}
    out["max_total"] = max(out["stellar"]["total"], out["cold_gas"]["total"])
    return out


def run_trees(args, params, table, net, gate, rank, dist, device):
    """The uneven-trees workload: 4,096 PCH trees evolved z=8->0 with 20
    outputs, one CUDA graph (one persistent kernel) per evolution, in the
    plain, FP32-rate and surrogate forms; the launch shape of the surrogate
    form picked by the autotuner."""
    import torch
    from galacticus_gb300 import forest, surrogate
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    world = dist.get_world_size() if dist else 1
    t0 = time.perf_counter()
    # One forest of `trees` per rank (seed 3), split over the ranks by
    # longest processing time first on node counts (weak scaling).
    f_all = forest.build(params, n_trees=args.trees * world, seed=3, satellites=SATELLITES[args.satellites])
    f, _ = forest.partition(f_all, rank, world)
    build_s = time.perf_counter() - t0
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params)
    out = {"workload": TREES_WORKLOAD.format(args.trees * world, satellite_note(args)), "nodes": f.n, "leaves": int((f.child_count == 0).sum()),
           "max_tree_nodes": int(np.bincount(f.tree).max()), "build_s": build_s,
           "split": f"{world} rank(s), trees assigned longest processing time first by node count",
           "graph": "one CUDA graph per evolution: counter reset, leaf-queue reset, one persistent kernel",
           "timing": "host clock around the graph launch and its completion event, after 1 warm-up evolution", "forms": {}}
    results = {}
    for name, rates in (("plain", "fp64"), ("fast_no_network", "fp32"), ("surrogate", "fp32")):
        ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
        if name == "surrogate" and gate is not None:
            net.build_error_map(table, tolerance=gate)
            net.install(ev)
        fe = forest.ForestEvolver(ev, f, state0, times)
        if name == "surrogate":
            tuned = fe.autotune(repeats=2)
            out["autotune"] = {"shapes": ["64x1", "128x1", "128x2", "256x1", "256x2", "512x1"],
                               "ms": [None if x < 0 else float(x) for x in tuned], "chosen": list(ev.get_launch()),
                               "note": "one lane per node: the warps-per-node axis is 1 by construction"}
        elif name == "fast_no_network":
            ev.set_launch(128, 2)
        fe.evolve()
        s0 = surrogate.stats(ev) if name == "surrogate" and gate is not None else (0, 0)
        reps = max(1, args.tree_steps)
        if dist:
            dist.barrier()
        torch.cuda.synchronize(device)
        tb = time.perf_counter()
        for _ in range(reps):
            fe.evolve(sync=False)
        fe.sync()
        dt = (time.perf_counter() - tb) / reps
        acc = fe.accepted_steps()
        per_rank = gather_ranks(dist, device, [dt, acc, f.n])
        dt, accepted_all = reduce_over_ranks(dist, device, dt, acc)
        state, status = fe.results(snapshots=False)[:2]
        entry = {"value": accepted_all / dt, "s_per_evolution": dt, "accepted_steps": acc, "launch": list(ev.get_launch()),
                 "failed_nodes": int((status != 0).sum())}
        if world > 1:
            entry["per_rank"] = [{"s_per_evolution": r[0], "accepted_steps": int(r[1]), "nodes": int(r[2])}
                                 for r in per_rank]
        if name == "surrogate":
            s1 = surrogate.stats(ev) if gate is not None else (0, 0)
            entry["network_share"] = (s1[0] - s0[0]) / max(1, (s1[0] - s0[0]) + (s1[1] - s0[1]))
            entry["gate_dex"] = gate
        results[name] = state
        out["forms"][name] = entry
        fe.close()
        ev.close()
    if rank == 0:
        from oracle import oracle
        tb = time.perf_counter()
        ref = oracle.evolve_forest(params, table, f, state0, times, threads=os.cpu_count() or 1, brent=True)[0]
        cpu_s = time.perf_counter() - tb
        acc = out["forms"]["plain"]["accepted_steps"]
        out["cpu_baseline"] = {"value": acc / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"one evolution of the whole forest ({cpu_s:.1f} s)"}
        for name, state in results.items():
            out["forms"][name]["mass_error"] = forest_mass_errors(state, ref, f)
        out["speedup_surrogate_vs_plain"] = out["forms"]["surrogate"]["value"] / out["forms"]["plain"]["value"]
    return out


def scale_record(args, params, table, net, gate):
    """The full chosen form at scale (65,536 PCH trees, seed 5, roots
    dN/dlnM ~ M^-0.9 on 1e10-1e14 Msun, resolution 1e8 Msun, z=10->0 with
    50 outputs, rel tol 1e-3): one warm-up and one timed evolution of the
    plain GPU form and of the surrogate form at `gate` (None: the table
    alone), the surrogate's fallback rate, final-mass errors of the roots
    against the plain GPU form, and against the CPU oracle on a sample of
    the trees (every 128th tree, evolved on all host cores; its time is the
    CPU baseline)."""
    from galacticus_gb300 import _abi, forest, surrogate, workloads
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard
    from oracle import oracle
    t0 = time.perf_counter()
    f = forest.build(params, n_trees=args.trees_scale, seed=5, redshift_max=10.0, satellites=SATELLITES[args.satellites])
    build_s = time.perf_counter() - t0
    state0 = forest.initial_state(params, f)
    times = forest.output_times(params, n=50, redshift_max=10.0)
    out = {"workload": f"scale: {args.trees_scale} PCH trees (seed 5), roots dN/dlnM ~ M^-0.9 on 1e10-1e14 Msun, "
                       f"resolution 1e8 Msun, z=10->0 with 50 outputs, rel tol 1e-3{satellite_note(args)}",
           "metric": METRIC, "unit": UNIT,
           "nodes": f.n, "leaves": int((f.child_count == 0).sum()), "max_tree_nodes": int(np.bincount(f.tree).max()),
           "build_s": build_s, "timing": "host clock around one graph launch and its completion, after one warm-up",
           "forms": {}}
    # The same builder with its branches grown on the GPU (keyed per-branch
    # streams: other trees of the same distribution), host clock around the
    # whole build (tables, roots, branching, spins, satellites, layout), and
    # both builders without satellites (the branches alone).
    ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32")
    builds = {}
    for sat in sorted({args.satellites, "none"}):
        for where in ("host", "gpu"):
            if where == "host" and sat == args.satellites:
                builds[f"{where}_{sat}"] = {"s": build_s, "nodes": f.n, **f.build_stats}
                continue
            tb = time.perf_counter()
            fb = forest.build(params, n_trees=args.trees_scale, seed=5, redshift_max=10.0, satellites=SATELLITES[sat],
                              gpu=ev if where == "gpu" else None)
            builds[f"{where}_{sat}"] = {"s": time.perf_counter() - tb, "nodes": fb.n, **fb.build_stats}
            del fb
    ev.close()
    out["tree_builds"] = builds
    states, counts = {}, {}
    for name, rates in (("plain", "fp64"), ("surrogate", "fp32")):
        ev = MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision=rates)
        ev.set_launch(128, 1 if rates == "fp64" else 2)
        if name == "surrogate" and gate is not None:
            net.build_error_map(table, tolerance=gate)
            net.install(ev)
        tc = time.perf_counter()
        fe = forest.ForestEvolver(ev, f, state0, times)
        create_s = time.perf_counter() - tc
        out["snapshots"] = fe.snapshot_count()
        fe.evolve()
        s0 = surrogate.stats(ev) if name == "surrogate" and gate is not None else (0, 0)
        tb = time.perf_counter()
        fe.evolve()
        dt = time.perf_counter() - tb
        tr = time.perf_counter()
        state, status, counters = fe.results(snapshots=False)[:3]
        results_s = time.perf_counter() - tr
        entry = {"value": float(counters[0].sum()) / dt, "s_per_evolution": dt, "accepted_steps": int(counters[0].sum()),
                 "rhs_evaluations": int(counters[2].sum()), "failed_nodes": int((status != 0).sum()),
                 "create_s": create_s, "results_s": results_s}
        if name == "surrogate":
            s1 = surrogate.stats(ev) if gate is not None else (0, 0)
            served = s1[0] - s0[0]
            entry["gate_dex"] = gate
            entry["fallback_rate"] = 1.0 - served / max(1, served + (s1[1] - s0[1]))
        states[name] = state
        counts[name] = counters
        out["forms"][name] = entry
        fe.close()
        ev.close()
    # The CPU oracle on every 128th tree (trees are independent: each one's
    # GPU result is its result alone).
    sample = np.arange(0, f.n_trees, 128)
    sub, idx = f.subset(sample)
    tb = time.perf_counter()
    ref = oracle.evolve_forest(params, table, sub, forest.initial_state(params, sub), times,
                               threads=os.cpu_count() or 1, brent=True)[0]
    cpu_s = time.perf_counter() - tb
    acc_sample = int(counts["plain"][0][idx].sum())
    out["cpu_baseline"] = {"value": acc_sample / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                           "sample": f"{len(sample)} of the trees ({sub.n} nodes), one evolution ({cpu_s:.1f} s)"}
    for name in states:
        out["forms"][name]["mass_error_vs_cpu_sample"] = forest_mass_errors(states[name][:, idx], ref, sub)
    out["forms"]["surrogate"]["mass_error_vs_plain_gpu"] = forest_mass_errors(states["surrogate"], states["plain"], f)
    out["speedup_surrogate_vs_plain"] = out["forms"]["surrogate"]["value"] / out["forms"]["plain"]["value"]
    # Rooflines: the reference's FP64 work per RHS evaluation (counted by the
    # oracle on the isolated-halo workload) times the RHS evaluations, and the
    # forest arrays each evolution reads and writes.
    flops_peak, calib_ms = ctypes.c_double(), ctypes.c_double()
    lib = _abi.load_library()
    lib.gal_calibrate_fp64(ctypes.byref(flops_peak), ctypes.byref(calib_ms))
    batch = workloads.isolated_halos(n=4096, seed=2)
    f_step = algorithmic_flops_per_step(params, table, batch, os.path.join(ROOT, "oracle", "flop_weights.json"))
    _, _, _, cb = oracle.evolve_batch(params, table, batch.state, batch.param, batch.t_start, batch.t_end, batch.step)
    f_rhs = f_step * cb[0].sum() / cb[2].sum()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    nbytes = f.n * (2 * _abi.NY * 8 + 6 * 4 + 8) + out["snapshots"] * _abi.NY * 8
    for name, entry in out["forms"].items():
        achieved = f_rhs * entry["rhs_evaluations"] / entry["s_per_evolution"]
        # In the FP32-rate forms most of the reference's FP64 work runs on the
        # FP32 pipe: the same ratio is then an FP64-equivalent rate and may
        # exceed the FP64 peak.
        key = "fp64" if name == "plain" else "fp64_equivalent"
        entry["roofline"] = {key: {"achieved_tflops": achieved / 1e12, "peak_tflops": flops_peak.value / 1e12,
                                   "frac": achieved / flops_peak.value,
                                   "basis": "the reference's FP64 flops per RHS evaluation (counted by the oracle) "
                                            "times the RHS evaluations, over the evolution time"},
                             "hbm": {"achieved_gbs": nbytes / entry["s_per_evolution"] / 1e9, "peak_gbs": peaks.get("hbm_gbs"),
                                     "frac": (nbytes / entry["s_per_evolution"] / 1e9 / peaks["hbm_gbs"]) if peaks.get("hbm_gbs") else None}}
    out["flops_per_rhs"] = f_rhs
    return out


def run_scale(args):
    """--workload scale: the scale record alone (the surrogate at --gate)."""
    import torch
    from galacticus_gb300 import surrogate, workloads
    from galacticus_gb300.cie_tables import CieTable
    torch.cuda.set_device(0)
    params = workloads.isolated_params()
    table = CieTable()
    net = surrogate.train(table)
    print(json.dumps(scale_record(args, params, table, net, args.gate if args.gate > 0 else None)), flush=True)


def run_ours(args):
    import torch
    from galacticus_gb300 import _abi, workloads, surrogate
    from galacticus_gb300.cie_tables import CieTable
    from galacticus_gb300.evolver import MergerTreeNodeEvolverStandard

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)

    params = workloads.isolated_params()
    table = CieTable()
    forms = {
        "plain": MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp64"),
        "fast": MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32"),
        "surrogate": MergerTreeNodeEvolverStandard(params=params, table=table, ratePrecision="fp32"),
    }
    for ev in forms.values():
        ev.set_launch(128, 2 if ev is not forms["plain"] else 1)
    lib = forms["plain"].lib
    batch = workloads.isolated_halos(n=args.nodes, seed=2 + rank)
    if args.halo >= 0:
        if args.form == "compare" or args.form.startswith("trees-"):
            raise SystemExit("--halo needs one batch form (--form plain, fast or surrogate)")
        batch = batch.subset(np.array([args.halo]))
    n = batch.n

    # The learned cooling surrogate: trained on this GPU by the library's own
    # kernels (not needed when one form without it is profiled alone).
    tt0 = time.perf_counter()
    net = surrogate.train(table) if args.form in ("compare", "surrogate", "trees-surrogate") else None
    train_s = time.perf_counter() - tt0

    def dev_tensor(a, dtype=torch.float64):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dtype)

    pristine_state = dev_tensor(batch.state)
    pristine_step = dev_tensor(batch.step)
    state = pristine_state.clone()
    step = pristine_step.clone()
    param = dev_tensor(batch.param)
    t0 = dev_tensor(batch.t_start)
    t1 = dev_tensor(batch.t_end)
    status = torch.zeros(n, dtype=torch.int32, device=dev)
    counters = torch.zeros((3, n), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)
    stream = torch.cuda.Stream(dev)  # one non-default stream orders copies, flush, events and our kernel
    torch.cuda.set_stream(stream)

    def one_step(ev, ev0=None, ev1=None, evk0=None, evk1=None):
        flush.zero_()  # evict the previous step's data from L2 (between timed iterations)
        if ev0 is not None:
            ev0.record(stream)
        state.copy_(pristine_state)  # every step evolves the same halos from the same initial state
        step.copy_(pristine_step)
        if evk0 is not None:
            evk0.record(stream)
        rc = ev.lib.gal_gpu_evolve_batch_device(ev.ctx, n, state.data_ptr(), param.data_ptr(), t0.data_ptr(),
                                                t1.data_ptr(), step.data_ptr(), status.data_ptr(), counters.data_ptr(),
                                                stream.cuda_stream)
        if rc:
            raise RuntimeError(f"gal_gpu_evolve_batch_device failed: {rc}")
        if evk1 is not None:
            evk1.record(stream)
        if ev1 is not None:
            ev1.record(stream)

    def final_state(ev):
        one_step(ev)
        torch.cuda.synchronize()
        if int((status != 0).sum()) != 0:
            raise RuntimeError("node evolution failed")
        return state.cpu().numpy()

    def timed(ev, clocks=None, passes=None):
        """W warm-up passes, then K passes (or `passes`) bracketed by barrier + synchronize."""
        steps = passes or args.steps
        for _ in range(max(args.warmup, 3)):
            one_step(ev)
        torch.cuda.synchronize()
        assert int((status != 0).sum()) == 0, "node evolution failed during warm-up"
        accepted = int(counters[0].sum())
        evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(4)) for _ in range(steps)]
        launches0 = lib.gal_gpu_launch_count(ev.ctx)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if clocks else None
        if sampler:
            sampler.__enter__()
        wall0 = time.perf_counter()
        for e in evs:
            one_step(ev, *e)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        if sampler:
            sampler.__exit__(None, None, None)
        if dist:
            dist.barrier()
        total_ms = sum(a.elapsed_time(b) for a, b, _, _ in evs)
        kernel_ms = statistics.mean(a.elapsed_time(b) for _, _, a, b in evs)
        if passes is None:
            total_ms, accepted_all = reduce_over_ranks(dist, dev, total_ms, accepted)
        else:
            accepted_all = accepted  # a rank-0 side measurement
        return {"value": accepted_all * steps / (total_ms * 1e-3), "ms_per_step": total_ms / steps,
                "kernel_ms": kernel_ms, "accepted_per_pass": accepted, "launches": lib.gal_gpu_launch_count(ev.ctx) - launches0,
                "wall_ms": wall * 1e3, "clocks": sampler.summary() if sampler else None}

    if args.form.startswith("trees-"):
        # One forest form alone (profiling runs): W + K evolutions of the forest.
        from galacticus_gb300 import forest as forest_mod
        name = args.form[len("trees-"):]
        ev = forms[name]
        if name == "surrogate":
            net.build_error_map(table, tolerance=args.gate)
            net.install(ev)
        f, _ = forest_mod.partition(forest_mod.build(params, n_trees=args.trees * world, seed=3,
                                                     satellites=SATELLITES[args.satellites]), rank, world)
        fe = forest_mod.ForestEvolver(ev, f, forest_mod.initial_state(params, f), forest_mod.output_times(params))
        for _ in range(args.warmup):
            fe.evolve()
        tb = time.perf_counter()
        for _ in range(args.steps):
            fe.evolve()
        dt = (time.perf_counter() - tb) / max(1, args.steps)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "form": args.form, "value": fe.accepted_steps() / dt, "unit": UNIT,
                              "s_per_evolution": dt, "nodes": f.n, "steps": args.steps, "warmup": args.warmup,
                              "launch": list(ev.get_launch())}), flush=True)
        fe.close()
        for e in forms.values():
            e.close()
        if dist:
            dist.destroy_process_group()
        return
    if args.form != "compare":
        # One form alone (profiling runs): no oracle, no comparison.
        ev = forms[args.form]
        if args.form == "surrogate":
            net.build_error_map(table, tolerance=args.gate)
            net.install(ev)
        r = timed(ev)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "form": args.form, "value": r["value"], "unit": UNIT,
                              "ms_per_step": r["ms_per_step"], "kernel_ms": r["kernel_ms"], "steps": args.steps,
                              "warmup": args.warmup, "launch": list(ev.get_launch())}), flush=True)
        for e in forms.values():
            e.close()
        if dist:
            dist.destroy_process_group()
        return

    # The FP64 oracle's final state of this rank's batch (rank 0 reports errors)
    # and the CPU baseline, timed on the host cores.
    cpu = None
    ref = None
    if rank == 0:
        cpu, ref = cpu_baseline(params, table, batch)

    # Error-map gate of the surrogate form, chosen by the per-halo bar: the
    # loosest of GATES at which 99.5% of the well-conditioned halos keep their
    # final stellar and cold-gas masses within 1e-3 of the FP64 oracle (halos
    # whose oracle masses themselves move by more than 1e-3 when the
    # tolerance changes by 10% or Lambda by 1e-4 dex are exempt).  None: no
    # gate with the network meets the bar and the form runs on the table.
    # Decided on rank 0.
    from oracle import compare
    movement = sensitivity_lambda = None
    if rank == 0:
        movement, _ = compare.conditioning(oracle_mod(), params, table, batch, ref, threads=os.cpu_count() or 1)
        sensitivity_lambda = lambda_sensitivity(params, table, batch, ref)

    totals = {}

    def run_gate(gate):
        ev = forms["surrogate"]
        if gate is None:
            net.uninstall(ev)
            out = final_state(ev)
            totals[gate] = mass_errors(out, ref)
            return out, 0.0
        net.build_error_map(table, tolerance=gate)
        net.install(ev)
        a = surrogate.stats(ev)
        out = final_state(ev)
        b = surrogate.stats(ev)
        totals[gate] = mass_errors(out, ref)
        return out, (b[0] - a[0]) / max(1, (b[0] - a[0]) + (b[1] - a[1]))

    gate_results = {}
    chosen = None
    if rank == 0:
        chosen, gate_results = compare.select_gate(run_gate, ref, movement, GATES + (None,))
        for gate, rec in gate_results.items():
            if gate is not None:
                net.build_error_map(table, tolerance=gate)
                net.install(forms["surrogate"])
                rec["table_cells"] = float(net.use_table.mean())
            else:
                net.uninstall(forms["surrogate"])
                rec["table_cells"] = 1.0
            rec["value"] = timed(forms["surrogate"], passes=10)["value"]
    if dist:
        g = torch.tensor([-1.0 if chosen is None else chosen], device=dev, dtype=torch.float64)
        dist.broadcast(g, 0)
        chosen = None if float(g.item()) < 0 else float(g.item())
    if chosen is None:
        net.uninstall(forms["surrogate"])
    else:
        net.build_error_map(table, tolerance=chosen)
        net.install(forms["surrogate"])
    s0 = surrogate.stats(forms["surrogate"]) if chosen is not None else (0, 0)
    headline = timed(forms["surrogate"], clocks=True)
    s1 = surrogate.stats(forms["surrogate"]) if chosen is not None else (0, 0)
    network_share = (s1[0] - s0[0]) / max(1, (s1[0] - s0[0]) + (s1[1] - s0[1]))
    # The same form in one network kernel over all nodes (no split launch).
    one_kernel = None
    if chosen is not None:
        surrogate.set_split(forms["surrogate"], False)
        one_kernel = timed(forms["surrogate"], passes=20)["value"]
        surrogate.set_split(forms["surrogate"], True)
    others = {name: timed(forms[name]) for name in ("plain", "fast")}
    if rank == 0:
        for name in ("plain", "fast"):
            st = final_state(forms[name])
            others[name]["mass_error"] = mass_errors(st, ref)
            others[name]["bar"] = compare.bar_shares(st, ref, movement)

    trees = run_trees(args, params, table, net, chosen, rank, dist, dev) if args.trees > 0 else None
    scale = scale_record(args, params, table, net, chosen) if rank == 0 and args.trees_scale > 0 else None

    # End-to-end through the public host API (pinned host buffers, copies in the timed region).
    ev = forms["surrogate"]
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h_state, h_param, h_t0, h_t1, h_step = pin(batch.state), pin(batch.param), pin(batch.t_start), pin(batch.t_end), pin(batch.step)
    h_status = pin(np.zeros(n, dtype=np.int32))
    h_counters = pin(np.zeros((3, n), dtype=np.uint32))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    e2e_times = []
    for i in range(args.warmup + args.steps):
        np.copyto(h_state, batch.state)
        np.copyto(h_step, batch.step)
        tb = time.perf_counter()
        rc = lib.gal_gpu_evolve_batch(ev.ctx, n, dp(h_state), dp(h_param), dp(h_t0), dp(h_t1), dp(h_step),
                                      h_status.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                      h_counters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        te = time.perf_counter() - tb
        if rc:
            raise RuntimeError("gal_gpu_evolve_batch failed")
        if i >= args.warmup:
            e2e_times.append(te)
    e2e_total, _ = reduce_over_ranks(dist, dev, sum(e2e_times))
    e2e_value = headline["value"] * headline["ms_per_step"] * args.steps * 1e-3 / e2e_total
    h2d = n * (_abi.NY + _abi.NP + 3) * 8
    d2h = n * (_abi.NY + 1) * 8 + n * 4 + n * 12

    if rank == 0:
        flops_peak, calib_ms = ctypes.c_double(), ctypes.c_double()
        lib.gal_calibrate_fp64(ctypes.byref(flops_peak), ctypes.byref(calib_ms))
        f_step = algorithmic_flops_per_step(params, table, batch, os.path.join(ROOT, "oracle", "flop_weights.json"))
        peaks = {}
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except OSError:
            pass
        k_ms = headline["kernel_ms"]
        acc = headline["accepted_per_pass"]
        achieved = f_step * acc / (k_ms * 1e-3)
        bytes_launch = n * ((_abi.NY + _abi.NP + 3) * 8 + (_abi.NY + 1) * 8 + 4 + 12)
        net_evals = (s1[0] - s0[0]) / max(1, args.steps)  # network evaluations (one per node and RHS) per pass
        mlp_tflops = net_evals * MLP_FLOPS / (k_ms * 1e-3) / 1e12
        err = totals[chosen]
        bar = gate_results[chosen]
        form = ("batched surrogate (fp32 rates + MLP cooling, table fallback)" if chosen is not None else
                "batched fp32-rate form with the surrogate gated off: no error-map gate with the network meets the "
                "per-halo bar, so every cooling evaluation uses the table")
        line = {
            "metric": METRIC, "value": headline["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": headline["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 state, error norm and step control; f32 rates" +
                     ("; MLP on bf16 tensor cores (split hi/lo operands, f32 accumulate)" if chosen is not None else ""),
            "data": "synthetic (seeded Philox halos; reference datasets absent)",
            "config": {"workload": WORKLOAD, "nodes_per_gpu": n, "form": form,
                       "gate_dex": chosen, "l2": "flushed between timed iterations (256 MB memset outside the kernel event pair)",
                       "launch": list(forms["surrogate"].get_launch()), "accepted_steps_per_pass": acc},
            "speedup_vs_plain": headline["value"] / others["plain"]["value"],
            "mass_error": err,
            "per_halo_bar": {"criterion": "stellar and cold-gas mass within 1e-3 of the FP64 oracle for >= 99.5% of "
                                          "the well-conditioned halos above 1e6 Msun (exempt: oracle masses that move "
                                          "by > 1e-3 under rel tol x0.9/x1.1 or Lambda x10^(+-1e-4))",
                             "headline": bar, "network_meets_bar": chosen is not None,
                             "lambda_sensitivity": sensitivity_lambda},
            "forms": {
                "surrogate": {"value": headline["value"], "ms_per_step": headline["ms_per_step"], "gate_dex": chosen,
                              "table_cells": bar["table_cells"], "network_share": network_share,
                              "mass_error": err, "bar": bar,
                              "launch": "split: nodes the network may serve on the network kernel, the others on the "
                                        "FP32-rate kernel without it, at once on two streams",
                              "one_kernel_value": one_kernel},
                "plain": {k: others["plain"][k] for k in ("value", "ms_per_step", "mass_error", "bar")},
                "fast_no_network": {k: others["fast"][k] for k in ("value", "ms_per_step", "mass_error", "bar")},
            },
            "surrogate": {"train_s": train_s, "val_rms_dex": net.rms_dex, "samples": 2_000_000, "epochs": 20,
                          "map_cells_dex": list(net.map_step),
                          "gates_tried": {str(k): dict(v, totals=totals[k]) for k, v in gate_results.items()}},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(headline["launches"]),
            "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": flops_peak.value / 1e12, "unit": "TFLOP/s",
                         "frac": achieved / flops_peak.value, "traffic": HEADLINE_DRAM_BYTES,
                         "traffic_unit": "bytes per pass: the split launch's two kernels (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                         "basis": "the reference's FP64 work per node-timestep (counted by the oracle) over the headline "
                                  "launch's time (both kernels of the split launch, CUDA events on the launching stream, "
                                  "which waits for the second stream): an FP64-equivalent rate, since this form runs the "
                                  "rates on the FP32 pipe and keeps FP64 for the state, error norm and step control",
                         "peak_source": "measured by gal_calibrate_fp64 (DFMA loop on all SMs); MEASURED_PEAKS.json has no FP64 figure",
                         "flops_per_node_timestep": f_step, "kernel_ms": k_ms,
                         "tensor": {"achieved": mlp_tflops, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                                    "frac": mlp_tflops / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                                    "basis": "the MLP's flops (16,896 per evaluation) times the network evaluations "
                                             "per pass (one per node and RHS that used it), over the kernel time"},
                         "hbm": {"achieved": bytes_launch / (k_ms * 1e-3) / 1e9, "peak": peaks.get("hbm_gbs"),
                                 "unit": "GB/s", "bytes_per_launch": bytes_launch},
                         "fp64_pipe": {"active_pct_of_peak": HEADLINE_FP64_PIPE_PCT,
                                       "metric": "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active",
                                       "source": "ncu --set full capture of the headline split launch, each kernel "
                                                 "timed alone, one GB300"}},
            "wall_ms_timed_region": headline["wall_ms"],
            "clocks": headline["clocks"],
            "cpu_baseline": cpu,
        }
        if trees:
            line["trees"] = trees
        if scale:
            line["scale"] = scale
        print(json.dumps(line), flush=True)
    for ev in forms.values():
        ev.close()
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.workload == "scale":
        run_scale(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
