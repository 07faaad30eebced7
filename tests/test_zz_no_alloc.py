"""The allocation-free entry point po_run_dev_static.

It exists for callers that cannot allocate device memory: frameworks that
reserve the GPU's memory for their own pool, and latency-critical loops that
cannot take cudaFree's device-wide synchronisation. Its scratch is a fixed
array inside the library. Checked here, through the C-ABI:
  * against the allocating entry (po_run_dev) on two calls in a row of
    different modes and sizes, and again on the first case (no leftovers);
  * against the reference's own outputs (golden vectors), every mode;
  * at full dish_eh size, where the array's limit caps the source chunks,
    with no change in device memory in use across the call;
  * a wait timeout set in its internal status word comes back through
    po_device_error, once, and is then cleared;
  * captured in a CUDA graph, it replays to the same bits and reads its
    inputs at replay time;
  * oversized problems are rejected with a message.
This file is collected last so that a run stopping at the first failure has
run every other test already; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.common import PHASE_TOL, REL_L2_TOL, errors, load_case

pytestmark = pytest.mark.gpu

MODE = {"JM": 0, "EH": 1, "JMEH": 2, "EHP": 3, "FF": 4, "scalar": 5}


def _static(lib, mode, w, s7, cur, t7, out, status, m_zero, stream, t_dir=-1.0, eps=1.0):
    return lib.po_run_dev_static(MODE[mode], s7.shape[1], s7.data_ptr(), w["gmode"], w["ncx"], w["ncy"],
                                 cur.data_ptr(), t7.shape[1], t7.data_ptr(), float(w["k"]), float(eps), t_dir,
                                 1 if m_zero else 0, out.data_ptr(),
                                 status.data_ptr() if status is not None else None,
                                 ctypes.c_void_p(stream.cuda_stream))


def _in_use(lib, torch):
    """(free device bytes, the library pool's bytes in use), after a synchronise."""
    torch.cuda.synchronize()
    used = ctypes.c_ulonglong(0)
    assert lib.po_scratch_in_use(ctypes.byref(used)) == 0, lib.po_last_error()
    return torch.cuda.mem_get_info()[0], used.value


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


@pytest.mark.parametrize("t_dir", [-1.0, 1.0])
def test_static_scratch_entry_matches_the_reference(cuda, lib, t_dir):
    """Every mode on the golden case (the reference's own FP64 outputs)."""
    import torch
    c = load_case("paruv_to_plane")
    src = c["src"]
    stream = torch.cuda.current_stream()
    s7 = torch.tensor(c["src_grid"], device=cuda)
    t7 = torch.tensor(c["tgt_grid"], device=cuda)
    w = {"gmode": int(src["gmode"]), "ncx": int(src["gridsize"][0]), "ncy": int(src["gridsize"][1]),
         "k": float(c["k"])}
    tag = "fwd" if t_dir < 0 else "bwd"
    for mode in ("JM", "EH", "JMEH", "EHP", "scalar"):
        cur = torch.tensor(c["cur"][:2] if mode == "scalar" else c["cur"], device=cuda)
        ref = c[f"out_{mode}_{tag}"]
        out = torch.full(ref.shape, float("nan"), dtype=torch.float64, device=cuda)
        rc = _static(lib, mode, w, s7, cur, t7, out, None, False, stream, t_dir, float(c["epsilon"]))
        assert rc == 0, lib.po_last_error()
        torch.cuda.synchronize()
        e, p = errors(out.cpu().numpy(), ref, mode)
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (mode, tag, e, p)


def test_static_scratch_at_full_size_allocates_nothing(cuda, lib):
    """dish_eh at full size (251,001 sources, 90,601 targets): the 64 MiB
    array caps the source chunks (the allocating entry takes more), and the
    result still meets the bar against po_run_dev; neither the free device
    memory nor the library pool's memory in use changes across the call."""
    import torch
    from pypo_gb300 import configs, engine
    w = configs.dish_eh()
    stream = torch.cuda.current_stream()
    s7, cur, t7 = (torch.tensor(w[k], device=cuda) for k in ("s7", "cur", "t7"))
    ref = engine.propagate_dev("EH", s7, cur, 1, w["ncx"], w["ncy"], t7, w["k"], m_zero=True)
    out = torch.empty_like(ref)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    assert _static(lib, "EH", w, s7, cur, t7, out, status, True, stream) == 0, lib.po_last_error()
    before = _in_use(lib, torch)
    out.fill_(float("nan"))
    assert _static(lib, "EH", w, s7, cur, t7, out, status, True, stream) == 0, lib.po_last_error()
    after = _in_use(lib, torch)
    assert after == before, (before, after)
    assert int(status.item()) == 0
    e, p = errors(out.cpu().numpy(), ref.cpu().numpy(), "EH")
    assert e <= REL_L2_TOL and p <= PHASE_TOL, (e, p)


def test_static_timeout_reaches_po_device_error(cuda, lib):
    """A timeout in the internal status word (calls with status NULL) is
    reported by po_device_error once and then cleared; a later call of the
    entry does not hide it."""
    import torch
    from pypo_gb300 import configs
    w = configs.dish_eh(scale=0.05)
    stream = torch.cuda.current_stream()
    s7, cur, t7 = (torch.tensor(w[k], device=cuda) for k in ("s7", "cur", "t7"))
    out = torch.empty((12, t7.shape[1]), dtype=torch.float64, device=cuda)
    code = ctypes.c_int(-1)
    assert _static(lib, "EH", w, s7, cur, t7, out, None, True, stream) == 0
    assert lib.po_device_error(ctypes.c_void_p(stream.cuda_stream), ctypes.byref(code)) == 0
    assert code.value == 0
    # the bounded wait of the kernels, run out on purpose into the internal word
    assert lib.po_wait_selftest(256, None, 1, ctypes.c_void_p(stream.cuda_stream)) == 0, lib.po_last_error()
    assert _static(lib, "EH", w, s7, cur, t7, out, None, True, stream) == 0
    assert lib.po_device_error(ctypes.c_void_p(stream.cuda_stream), ctypes.byref(code)) == 0
    assert code.value == 101
    assert lib.po_device_error(ctypes.c_void_p(stream.cuda_stream), ctypes.byref(code)) == 0
    assert code.value == 0


@pytest.mark.parametrize("name,scale", [("dish_eh", 0.1), ("dish_ff", 0.05)])
def test_static_entry_replays_in_a_cuda_graph(cuda, lib, name, scale):
    """The allocation-free entry inside a captured CUDA graph (near field, and
    the far field with its radix sort): after one call outside capture (the
    set-up), the captured call replays to the same bits, and a replay after
    the currents were scaled in place gives the scaled field (the graph
    reads its inputs at replay time)."""
    import torch
    from pypo_gb300 import configs
    w = getattr(configs, name)(scale=scale)
    s7, cur, t7 = (torch.tensor(w[k], device=cuda) for k in ("s7", "cur", "t7"))
    out = torch.empty((12, t7.shape[1]), dtype=torch.float64, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        assert _static(lib, w["mode"], w, s7, cur, t7, out, status, True, side) == 0, lib.po_last_error()
    torch.cuda.synchronize()
    ref = out.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        stream = torch.cuda.current_stream()
        assert _static(lib, w["mode"], w, s7, cur, t7, out, status, True, stream) == 0, lib.po_last_error()
    out.fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, ref) and int(status.item()) == 0
    cur.mul_(2.0)
    g.replay()
    torch.cuda.synchronize()
    assert torch.allclose(out, 2.0 * ref, rtol=1e-6, atol=1e-6 * float(ref.abs().max()))


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
