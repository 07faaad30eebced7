"""Multi-GPU use of the integrator (one process per GPU, torch.distributed).

Forward: target points are independent, so one large propagation splits into
contiguous target shards. Every rank holds the (replicated) sources, computes
its shard, and the shards are gathered at the end; no other collective sits
on the data path.

Adjoint: the gradients with respect to the currents and the source
displacement are sums over targets per source, the target-displacement
gradient a sum over sources per target. One pass covers both: every rank
takes a contiguous source shard against all targets (the fused adjoint), the
source-side gradients are gathered, and the per-rank partial sums of the
target side are added with one all_reduce (the one real exchange step).
A source shard is not a grid any more, so it goes as a point cloud
(gmode -1) with the trapezoid weights folded into its area row.

The *_dev variants keep everything on each rank's device: torch tensors in,
NCCL collectives on device buffers, torch tensors out (no host round trip).

`max_over_ranks` is the timing reduction used by bench.py.
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


def trapezoid_weights(n, gmode, ncx, ncy):
    """Per-point trapezoid weights of a grid, as the reference's field sums
    apply them (src/CPU/Propagation.h:1109-1126): x/u ends 0.5; y/v ends 0.5
    unless gmode == 1 (uv); 1 everywhere for a point cloud (gmode < 0)."""
    w = np.ones(n)
    if gmode < 0:
        return w
    i = np.arange(n)
    xu, yv = i // ncy, i % ncy
    w[(xu == 0) | (xu == ncx - 1)] *= 0.5
    if gmode != 1:
        w[(yv == 0) | (yv == ncy - 1)] *= 0.5
    return w


def as_point_cloud(src7, gmode, ncx, ncy):
    """src7 as a point cloud (gmode -1): the trapezoid weights move into row 6."""
    out = np.array(src7, dtype=np.float64, copy=True)
    out[6] *= trapezoid_weights(out.shape[1], gmode, ncx, ncy)
    return out


def _gather_rows(local, n, rank, world, dist, backend):
    """All-gather a (rows, shard) float64 array of contiguous shards into (rows, n)."""
    import torch
    rows = local.shape[0]
    width = n // world + (1 if n % world else 0)
    b, e = shard_range(n, rank, world)
    buf = torch.zeros((rows, width), dtype=torch.float64)
    buf[:, :e - b] = torch.from_numpy(np.ascontiguousarray(local))
    if backend == "nccl":
        buf = buf.cuda()
    gathered = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(gathered, buf)
    out = np.empty((rows, n))
    for r in range(world):
        rb, re = shard_range(n, r, world)
        out[:, rb:re] = gathered[r][:, :re - rb].cpu().numpy()
    return out


def adjoint_sharded(mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon=1.0, t_dir=-1.0, compute=None):
    """Adjoint with the sources sharded over the default process group.

    Arguments as pypo_gb300.engine.adjoint (host float64 arrays, identical on
    every rank). `compute` (default engine.adjoint on this rank's GPU) maps
    (mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon, t_dir) to the
    dict {"cur", "ds", "dt"} of that sub-problem. Returns the full gradients on
    every rank ("dt" is None for the far field).
    """
    import torch
    import torch.distributed as dist
    from . import engine
    if compute is None:
        compute = engine.adjoint
    rank, world = dist.get_rank(), dist.get_world_size()
    backend = dist.get_backend()
    ns, nt = src7.shape[1], tgt7.shape[1]
    b, e = shard_range(ns, rank, world)
    pts = as_point_cloud(src7, gmode, ncx, ncy)
    g = compute(mode, np.ascontiguousarray(pts[:, b:e]), np.ascontiguousarray(cur[:, b:e]), -1, 0, 0, tgt7, k, cot,
                epsilon, t_dir)
    out = {"cur": _gather_rows(g["cur"], ns, rank, world, dist, backend),
           "ds": _gather_rows(g["ds"][None, :], ns, rank, world, dist, backend)[0], "dt": None}
    if mode != "FF":
        dt = torch.from_numpy(np.ascontiguousarray(g["dt"], dtype=np.float64))
        if backend == "nccl":
            dt = dt.cuda()
        dist.all_reduce(dt, op=dist.ReduceOp.SUM)
        out["dt"] = dt.cpu().numpy()
    return out


def _gather_cols(local, n, rank, world):
    """All-gather a (rows, shard) tensor of contiguous column shards into
    (rows, n), on local's device (the collective runs on that device)."""
    import torch
    import torch.distributed as dist
    width = n // world + (1 if n % world else 0)
    b, e = shard_range(n, rank, world)
    buf = torch.zeros((local.shape[0], width), dtype=local.dtype, device=local.device)
    buf[:, :e - b] = local
    gathered = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(gathered, buf)
    parts = []
    for r in range(world):
        rb, re = shard_range(n, r, world)
        parts.append(gathered[r][:, :re - rb])
    return torch.cat(parts, dim=1)


def propagate_sharded_dev(mode, src7, cur, gmode, ncx, ncy, tgt7, k, epsilon=1.0, t_dir=-1.0, precision="mixed",
                          m_zero=False, compute=None):
    """Device-resident propagate_sharded: src7, cur, tgt7 are float64 torch
    tensors on this rank's device, identical on every rank. `compute`
    (default: pypo_gb300.engine.propagate_dev) maps the call on a target shard
    (a contiguous 7-row tensor) to its (n_out, shard) tensor. Returns the full
    (n_out, nt) output on every rank's device."""
    import torch.distributed as dist
    from . import engine
    if compute is None:
        def compute(*a):
            return engine.propagate_dev(*a, precision=precision, m_zero=m_zero)
    rank, world = dist.get_rank(), dist.get_world_size()
    nt = tgt7.shape[1]
    b, e = shard_range(nt, rank, world)
    local = compute(mode, src7, cur, gmode, ncx, ncy, tgt7[:, b:e].contiguous(), k, epsilon, t_dir)
    return _gather_cols(local, nt, rank, world)


def as_point_cloud_dev(src7, gmode, ncx, ncy):
    """as_point_cloud for a torch tensor, on its device."""
    import torch
    out = src7.clone()
    n = out.shape[1]
    if gmode >= 0:
        i = torch.arange(n, device=out.device)
        xu, yv = i // ncy, i % ncy
        w = torch.ones(n, dtype=out.dtype, device=out.device)
        w = torch.where((xu == 0) | (xu == ncx - 1), 0.5 * w, w)
        if gmode != 1:
            w = torch.where((yv == 0) | (yv == ncy - 1), 0.5 * w, w)
        out[6] *= w
    return out


def adjoint_sharded_dev(mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon=1.0, t_dir=-1.0,
                        precision="mixed", m_zero=False, compute=None):
    """Device-resident adjoint_sharded: float64 torch tensors on this rank's
    device, identical on every rank. `compute` (default: engine.adjoint_dev
    into fresh device buffers) maps (mode, src7, cur, gmode, ncx, ncy, tgt7,
    k, cot, epsilon, t_dir) on a source shard (a point cloud) to the dict
    {"cur", "ds", "dt"} of device tensors. Returns the full gradients on every
    rank's device ("dt" is None for the far field); the target side is one
    all_reduce of the ranks' partial sums."""
    import torch
    import torch.distributed as dist
    from . import engine
    if compute is None:
        def compute(md, s7, c, gm, nx, ny, t7, kk, ct, eps, t):
            gc = torch.empty_like(c)
            gs = torch.empty(s7.shape[1], dtype=torch.float64, device=s7.device)
            gt = None if md == "FF" else torch.empty(t7.shape[1], dtype=torch.float64, device=t7.device)
            engine.adjoint_dev(md, s7, c, gm, nx, ny, t7, kk, ct, eps, t, precision=precision, m_zero=m_zero,
                               grad_cur=gc, grad_ds=gs, grad_dt=gt)
            return {"cur": gc, "ds": gs, "dt": gt}
    rank, world = dist.get_rank(), dist.get_world_size()
    ns = src7.shape[1]
    b, e = shard_range(ns, rank, world)
    pts = as_point_cloud_dev(src7, gmode, ncx, ncy)
    g = compute(mode, pts[:, b:e].contiguous(), cur[:, b:e].contiguous(), -1, 0, 0, tgt7, k, cot, epsilon, t_dir)
    out = {"cur": _gather_cols(g["cur"], ns, rank, world), "ds": _gather_cols(g["ds"][None, :], ns, rank, world)[0],
           "dt": None}
    if mode != "FF":
        dt = g["dt"].clone()
        dist.all_reduce(dt, op=dist.ReduceOp.SUM)
        out["dt"] = dt
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
