"""The N>1 bench path on CPU: two gloo ranks, each with its own seeded batch
(weak scaling), whole-job numbers from a max-over-ranks time and a sum of
levels -- the only cross-rank traffic."""
from __future__ import annotations

import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, outdir):
    import json

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      OMP_NUM_THREADS="1")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    b = bench.workload(rank, B=12, n_min=2048, n_max=4096)
    ms, levels = bench.aggregate(10.0 + rank, 100 * (rank + 1), dist, "cpu")
    with open(os.path.join(outdir, f"r{rank}.json"), "w") as f:
        json.dump([float(b.mu.sum()), ms, levels], f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import json

    world = 2
    port = _free_port()
    mp.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    (mu0, ms0, l0), (mu1, ms1, l1) = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    assert mu0 != mu1  # independent batches per rank
    assert ms0 == ms1 == 11.0  # max over ranks
    assert l0 == l1 == 300  # sum over ranks
    rank_seeds = {3 + 100 * r for r in range(world)}
    assert len(rank_seeds) == world
    assert np.isfinite(mu0)
