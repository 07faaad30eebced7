"""Multi-GPU use of the integrator (one process per GPU, torch.distributed).

Target points are independent, so one large propagation splits into
contiguous target shards: every rank holds the (replicated) sources, computes
its shard, and the shards are gathered at the end. No other collective sits
on the data path. `max_over_ranks` is the timing reduction used by bench.py.
"""
import numpy as np


def shard_range(nt, rank, world):
    """[begin, end) of rank's contiguous target shard (sizes differ by at most 1)."""
    base, extra = divmod(nt, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def propagate_sharded(mode, src7, cur, gmode, ncx, ncy, tgt7, k, epsilon=1.0, t_dir=-1.0, compute=None):
    """Propagate with the targets sharded over the default process group.

    src7, cur, tgt7: host float64 arrays, identical on every rank. `compute`
    (default: pypo_gb300.engine.propagate on this rank's GPU) maps the call on
    a target shard to its (n_out, shard) output. Returns the full
    (n_out, nt) output on every rank.
    """
    import torch
    import torch.distributed as dist
    from . import engine
    if compute is None:
        compute = engine.propagate
    rank, world = dist.get_rank(), dist.get_world_size()
    nt = tgt7.shape[1]
    b, e = shard_range(nt, rank, world)
    part = compute(mode, src7, cur, gmode, ncx, ncy, np.ascontiguousarray(tgt7[:, b:e]), k, epsilon, t_dir)
    nout = part.shape[0]
    width = nt // world + (1 if nt % world else 0)
    buf = torch.zeros((nout, width), dtype=torch.float64)
    buf[:, :e - b] = torch.from_numpy(np.ascontiguousarray(part))
    backend = dist.get_backend()
    if backend == "nccl":
        buf = buf.cuda()
    gathered = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(gathered, buf)
    out = np.empty((nout, nt))
    for r in range(world):
        rb, re = shard_range(nt, r, world)
        out[:, rb:re] = gathered[r][:, :re - rb].cpu().numpy()
    return out


def max_over_ranks(value):
    """Largest value over the default process group (timing reduction)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
