"""The allocation-free entry point po_run_dev_static against po_run_dev.

po_run_dev_static exists for callers that cannot allocate device memory
(frameworks that reserve the GPU's memory for their own pool, latency-critical
loops that cannot take cudaFree's device-wide synchronisation): its scratch is
a fixed array inside the library. This file is collected last so that a run
stopping at the first failure has run every other test already; it also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.common import PHASE_TOL, REL_L2_TOL, errors

pytestmark = pytest.mark.gpu

MODE = {"JM": 0, "EH": 1, "JMEH": 2, "EHP": 3, "FF": 4, "scalar": 5}


def _static(lib, mode, w, s7, cur, t7, out, status, m_zero, stream):
    return lib.po_run_dev_static(MODE[mode], s7.shape[1], s7.data_ptr(), w["gmode"], w["ncx"], w["ncy"],
                                 cur.data_ptr(), t7.shape[1], t7.data_ptr(), float(w["k"]), 1.0, -1.0,
                                 1 if m_zero else 0, out.data_ptr(), status.data_ptr(),
                                 ctypes.c_void_p(stream.cuda_stream))


def test_static_scratch_entry_matches_allocating_entry(cuda, lib):
    import torch
    from pypo_gb300 import configs, engine
    stream = torch.cuda.current_stream()
    status = torch.full((1,), -7, dtype=torch.int32, device=cuda)
    cases = [configs.dish_eh(scale=0.2), configs.dish_ff(scale=0.06)]
    cases[1]["cur"][6:] = np.random.default_rng(3).standard_normal(cases[1]["cur"][6:].shape) * 0.1
    outs = []
    for w in cases:   # two calls in a row, different modes and sizes, on the shared array
        s7 = torch.tensor(w["s7"], device=cuda)
        cur = torch.tensor(w["cur"], device=cuda)
        t7 = torch.tensor(w["t7"], device=cuda)
        m_zero = not np.any(w["cur"][6:])
        ref = engine.propagate_dev(w["mode"], s7, cur, w["gmode"], w["ncx"], w["ncy"], t7, w["k"],
                                   m_zero=m_zero)
        out = torch.full_like(ref, float("nan"))
        rc = _static(lib, w["mode"], w, s7, cur, t7, out, status, m_zero, stream)
        assert rc == 0, lib.po_last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        e, p = errors(got, want, w["mode"])
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (w["name"], e, p)
        outs.append(got)
    # the first case again: the previous call's leftovers must not leak in
    w = cases[0]
    s7, cur, t7 = (torch.tensor(w[k], device=cuda) for k in ("s7", "cur", "t7"))
    out = torch.empty((12, t7.shape[1]), dtype=torch.float64, device=cuda)
    assert _static(lib, w["mode"], w, s7, cur, t7, out, status, True, stream) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), outs[0])


def test_static_scratch_rejects_oversized_problems(cuda, lib):
    import torch
    big_ns = 1_000_000   # 88 MB of packed sources alone
    s7 = torch.zeros((7, 1), dtype=torch.float64, device=cuda)
    out = torch.zeros((12, 1), dtype=torch.float64, device=cuda)
    rc = lib.po_run_dev_static(1, big_ns, s7.data_ptr(), -1, 0, 0, s7.data_ptr(), 1, s7.data_ptr(),
                               1.0, 1.0, -1.0, 0, out.data_ptr(), None,
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 5
    assert b"static array" in lib.po_last_error()
