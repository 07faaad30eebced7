"""The device-resident sharded entries on one GPU through NCCL (a one-rank
process group): the default compute (engine.propagate_dev / adjoint_dev) and
the collectives run on device tensors, and the results equal the unsharded
device calls."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_dev_one_rank_nccl(cuda, lib):
    import torch
    import torch.distributed as dist
    from pypo_gb300 import configs, dist as D, engine
    os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{_free_port()}", rank=0, world_size=1)
    try:
        w = configs.dish_eh(scale=0.1)
        s7, cur, t7 = (torch.tensor(w[k], device=cuda) for k in ("s7", "cur", "t7"))
        grid = (w["gmode"], w["ncx"], w["ncy"])
        out = D.propagate_sharded_dev("EH", s7, cur, *grid, t7, w["k"], m_zero=True)
        ref = engine.propagate_dev("EH", s7, cur, *grid, t7, w["k"], m_zero=True)
        assert out.is_cuda and torch.equal(out, ref)
        cot = torch.tensor(np.random.default_rng(1).standard_normal((12, t7.shape[1])), device=cuda)
        got = D.adjoint_sharded_dev("EH", s7, cur, *grid, t7, w["k"], cot, m_zero=True)
        gc, gs, gt = torch.empty_like(cur), torch.empty(s7.shape[1], dtype=torch.float64, device=cuda), \
            torch.empty(t7.shape[1], dtype=torch.float64, device=cuda)
        engine.adjoint_dev("EH", s7, cur, *grid, t7, w["k"], cot, m_zero=True, grad_cur=gc, grad_ds=gs, grad_dt=gt)
        rel = lambda a, b: float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
        # the shard is a point cloud (weights folded into the areas): equal up to rounding
        assert rel(got["cur"], gc) <= 1e-12 and rel(got["ds"], gs) <= 1e-12 and rel(got["dt"], gt) <= 1e-12
    finally:
        dist.destroy_process_group()
