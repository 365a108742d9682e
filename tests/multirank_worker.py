"""One rank of the multi-rank host-logic check (launched by
tests/test_multirank_cpu.py under torch.distributed.run with the gloo
backend, on CPU).

Each rank builds its own isolated halos as bench.py does (seed 2 + rank),
reduces a timing and a work count with bench.reduce_over_ranks, and takes
its longest-processing-time share of one forest (forest.partition, as
bench.py's uneven-trees workload does).  It evolves its share with the CPU
oracle -- the stand-in for its GPU here -- and gathers every rank's final
node states with their node indices; rank 0 writes the union next to the
same forest evolved whole by one process, in <out_dir>."""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main(out_dir):
    import torch
    import torch.distributed as dist

    import bench
    from galacticus_gb300 import forest, workloads
    from galacticus_gb300.cie_tables import CieTable
    from oracle import oracle

    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    cpu = torch.device("cpu")
    elapsed, work = bench.reduce_over_ranks(dist, cpu, 1.5 + rank, 10 * (rank + 1))

    params = workloads.isolated_params()
    halos = workloads.isolated_halos(n=64, seed=2 + rank)
    mine = torch.tensor([float(halos.state.sum()), float(halos.param.sum())], dtype=torch.float64)
    every = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(every, mine)

    # One forest, split over the ranks (with satellites, as the bench's: a
    # satellite's phase and its host stay in their tree, so a share's
    # satellite hosts are remapped into the share).
    table = CieTable()
    whole = forest.build(params, n_trees=7, seed=3, root_mass_min=1e10, root_mass_max=3e11,
                         satellites=forest.SATELLITES_JIANG2008)
    assert (whole.satellite_host >= 0).sum() > 0
    times = forest.output_times(params, n=5)
    part, idx = forest.partition(whole, rank, world)
    state = oracle.evolve_forest(params, table, part, forest.initial_state(params, part), times, brent=False)[0]
    shares = [None] * world
    dist.all_gather_object(shares, {"idx": idx.tolist(), "state": state.tolist(), "nodes": int(part.n),
                                    "trees": forest.lpt_assignment(whole, world)[rank].tolist()})
    per_rank = bench.gather_ranks(dist, cpu, [float(rank), float(part.n)])
    if rank == 0:
        union = np.full((len(state), whole.n), np.nan)
        for sh in shares:
            union[:, sh["idx"]] = np.array(sh["state"])
        single = oracle.evolve_forest(params, table, whole, forest.initial_state(params, whole), times, brent=False)[0]
        np.save(os.path.join(out_dir, "union.npy"), union)
        np.save(os.path.join(out_dir, "single.npy"), single)
        with open(os.path.join(out_dir, "split.json"), "w") as f:
            json.dump({"trees": [sh["trees"] for sh in shares], "nodes": [sh["nodes"] for sh in shares],
                       "tree_nodes": np.bincount(whole.tree).tolist(), "per_rank": per_rank}, f)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "elapsed": elapsed, "work": work,
                   "checksums": [e.tolist() for e in every]}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
