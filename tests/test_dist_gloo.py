"""Multi-rank host logic on CPU (gloo, world size 2): target sharding with the
final gather, and the max-over-ranks timing reduction. The per-rank compute is
the FP64 oracle, so no GPU is needed."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, result_dir):
    import torch.distributed as dist
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle as O
    from pypo_gb300 import dist as D
    from pypo_gb300 import surfaces as SF
    from pypo_gb300 import engine
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    src = SF.paraboloid(1.0, [9, 8], gmode=1, lims_a=[0.1, 1.5])
    s7 = engine.generate_grid(src)
    t7 = np.zeros((7, 37))
    rng = np.random.default_rng(0)
    t7[0:2] = rng.uniform(-1, 1, (2, 37))
    t7[2] = 2.5
    t7[5] = -1.0
    cur = rng.standard_normal((12, s7.shape[1]))
    compute = lambda *a: O.run(*a, nthreads=1)
    out = D.propagate_sharded("EH", s7, cur, 1, 9, 8, t7, 4.0, compute=compute)
    full = O.run("EH", s7, cur, 1, 9, 8, t7, 4.0, nthreads=1)
    ok = np.array_equal(out, full)
    mx = D.max_over_ranks(10.0 + rank)
    np.save(os.path.join(result_dir, f"rank{rank}.npy"), np.array([ok, mx == 10.0 + world - 1], dtype=bool))
    dist.destroy_process_group()


def test_shard_ranges_cover_targets_once():
    from pypo_gb300.dist import shard_range
    for nt in (0, 1, 5, 37, 90601):
        for world in (1, 2, 3, 8):
            spans = [shard_range(nt, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nt
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1


def test_sharded_propagation_world2_gloo(tmp_path, oracle_mod, lib):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        ok = np.load(tmp_path / f"rank{r}.npy")
        assert ok.all(), f"rank {r}: {ok}"
