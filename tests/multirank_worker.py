"""One rank of the multi-rank host-logic check (launched by
tests/test_multirank_cpu.py under torch.distributed.run with the gloo
backend, on CPU).

Each rank builds its own share of the work exactly as bench.py does -- the
halos of seed 2 + rank and the trees of seed 3 + rank -- reduces a timing and
a work count with bench.reduce_over_ranks, gathers checksums of its inputs,
and writes what it saw to <out_dir>/rank<r>.json."""

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main(out_dir):
    import torch
    import torch.distributed as dist

    import bench
    from galacticus_gb300 import forest, workloads

    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    cpu = torch.device("cpu")
    elapsed, work = bench.reduce_over_ranks(dist, cpu, 1.5 + rank, 10 * (rank + 1))

    params = workloads.isolated_params()
    halos = workloads.isolated_halos(n=64, seed=2 + rank)
    trees = forest.build(params, n_trees=2, seed=3 + rank, root_mass_min=1e10, root_mass_max=1e11)
    mine = torch.tensor([float(halos.state.sum()), float(halos.param.sum()), float(trees.mass.sum()), float(trees.n)],
                        dtype=torch.float64)
    every = [torch.zeros(4, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(every, mine)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": rank, "world": world, "elapsed": elapsed, "work": work,
                   "checksums": [e.tolist() for e in every]}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
