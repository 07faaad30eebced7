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


def _oracle_adjoint(O, mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, eps=1.0, t=-1.0):
    """Reference gradients of L = sum(cot * out) from the FP64 oracle: L is
    linear in the currents (unit-current evaluations are exact); central
    differences (h = 1e-6 wavelengths) for the normal displacements."""
    L = lambda s, c, tt: float((cot * O.run(mode, s, c, gmode, ncx, ncy, tt, k, eps, t, nthreads=1)).sum())
    ns, nt = src7.shape[1], tgt7.shape[1]
    gc = np.zeros((12, ns))
    for r in range(12):
        for i in range(ns):
            c = np.zeros_like(cur)
            c[r, i] = 1.0
            gc[r, i] = L(src7, c, tgt7)
    h = 1e-6 * 2 * np.pi / k

    def fd(points, i, f):
        p, m = points.copy(), points.copy()
        p[:3, i] += h * points[3:6, i]
        m[:3, i] -= h * points[3:6, i]
        return (f(p) - f(m)) / (2 * h)
    gs = np.array([fd(src7, i, lambda s: L(s, cur, tgt7)) for i in range(ns)])
    gt = None if mode == "FF" else np.array([fd(tgt7, j, lambda tt: L(src7, cur, tt)) for j in range(nt)])
    return {"cur": gc, "ds": gs, "dt": gt}


def _adjoint_worker(rank, world, port, result_dir):
    import torch.distributed as dist
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle as O
    from pypo_gb300 import dist as D
    from pypo_gb300 import engine, surfaces as SF
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(3)
    ok = []
    for mode in ("EH", "FF"):
        s7 = engine.generate_grid(SF.plane([4, 3], gmode=0, lims_a=[-1.0, 1.0]))   # xy grid: both ends weighted
        if mode == "FF":
            t7 = engine.generate_grid(SF.farfield([3, 3], [-20, 20], [-20, 20]))
        else:
            t7 = np.zeros((7, 7))
            t7[0:2] = rng.uniform(-1, 1, (2, 7))
            t7[2] = 2.5
            t7[5] = -1.0
            t7[6] = 1.0
        cur = rng.standard_normal((12, s7.shape[1]))
        cot = rng.standard_normal((engine.n_out(mode), t7.shape[1]))
        compute = lambda *a: _oracle_adjoint(O, *a)
        got = D.adjoint_sharded(mode, s7, cur, 0, 4, 3, t7, 4.0, cot, compute=compute)
        ref = _oracle_adjoint(O, mode, s7, cur, 0, 4, 3, t7, 4.0, cot)
        rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
        ok.append(rel(got["cur"], ref["cur"]) <= 1e-12)
        ok.append(rel(got["ds"], ref["ds"]) <= 1e-6)
        ok.append((got["dt"] is None) if mode == "FF" else rel(got["dt"], ref["dt"]) <= 1e-6)
    np.save(os.path.join(result_dir, f"adj_rank{rank}.npy"), np.array(ok, dtype=bool))
    dist.destroy_process_group()


def test_trapezoid_weights_and_point_cloud():
    from pypo_gb300.dist import as_point_cloud, trapezoid_weights
    w = trapezoid_weights(12, 0, 4, 3).reshape(4, 3)
    assert np.array_equal(w[0], [0.25, 0.5, 0.25]) and np.array_equal(w[1], [0.5, 1.0, 0.5])
    wuv = trapezoid_weights(12, 1, 4, 3).reshape(4, 3)
    assert np.array_equal(wuv[0], [0.5, 0.5, 0.5]) and np.array_equal(wuv[1], [1.0, 1.0, 1.0])
    assert np.array_equal(trapezoid_weights(5, -1, 0, 0), np.ones(5))
    s7 = np.ones((7, 12))
    assert np.array_equal(as_point_cloud(s7, 0, 4, 3)[6], trapezoid_weights(12, 0, 4, 3))


def test_sharded_adjoint_world2_gloo(tmp_path, oracle_mod, lib):
    """Source-sharded adjoint (gather of the source-side gradients, all_reduce
    of the target-side partial sums) against the unsharded reference."""
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_adjoint_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        ok = np.load(tmp_path / f"adj_rank{r}.npy")
        assert ok.all(), f"rank {r}: {ok}"


def _dev_worker(rank, world, port, result_dir):
    """The device-resident variants on CPU tensors (gloo), with the oracle's
    forward and FP64 adjoint as each rank's compute."""
    import torch
    import torch.distributed as dist
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle as O
    from pypo_gb300 import dist as D
    from pypo_gb300 import engine, surfaces as SF
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    T = torch.from_numpy
    rng = np.random.default_rng(9)
    s7 = engine.generate_grid(SF.plane([5, 4], gmode=0, lims_a=[-1.0, 1.0]))
    t7 = np.zeros((7, 23))
    t7[0:2] = rng.uniform(-1, 1, (2, 23))
    t7[2] = 2.5
    t7[5] = -1.0
    t7[6] = 1.0
    cur = rng.standard_normal((12, s7.shape[1]))
    cot = rng.standard_normal((12, 23))
    ok = []
    fwd = lambda m, a, c, g, x, y, t, k, e, d: T(O.run(m, a.numpy(), c.numpy(), g, x, y, t.numpy(), k, e, d,
                                                        nthreads=1))
    out = D.propagate_sharded_dev("EH", T(s7), T(cur), 0, 5, 4, T(t7), 4.0, compute=fwd)
    ok.append(isinstance(out, torch.Tensor) and np.array_equal(out.numpy(),
                                                                O.run("EH", s7, cur, 0, 5, 4, t7, 4.0, nthreads=1)))

    def adj(m, a, c, g, x, y, t, k, ct, e, d):
        r = O.adjoint(m, a.numpy(), c.numpy(), g, x, y, t.numpy(), k, ct.numpy(), e, d, nthreads=1)
        return {n: T(v) for n, v in r.items()}
    got = D.adjoint_sharded_dev("EH", T(s7), T(cur), 0, 5, 4, T(t7), 4.0, T(cot), compute=adj)
    ref = O.adjoint("EH", s7, cur, 0, 5, 4, t7, 4.0, cot, nthreads=1)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    for name in ("cur", "ds", "dt"):
        ok.append(isinstance(got[name], torch.Tensor) and rel(got[name].numpy(), ref[name]) <= 1e-12)
    pc = D.as_point_cloud_dev(T(s7), 0, 5, 4).numpy()
    ok.append(np.array_equal(pc, D.as_point_cloud(s7, 0, 5, 4)))
    np.save(os.path.join(result_dir, f"dev_rank{rank}.npy"), np.array(ok, dtype=bool))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_device_resident_sharding_gloo(tmp_path, oracle_mod, lib, world):
    """propagate_sharded_dev / adjoint_sharded_dev: tensors in and out, the
    gather and the all_reduce on the tensors' device; uneven shards at world 3."""
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_dev_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        ok = np.load(tmp_path / f"dev_rank{r}.npy")
        assert ok.all(), f"rank {r}: {ok}"
