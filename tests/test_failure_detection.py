"""Failure detection without a GPU fault.

The kernels bound every wait on a tile copy and, when a wait runs out, set
an error word and leave (no trap, no exit): the reference instead calls
exit() on a CUDA error (src/include/MemUtils.h:27-34). po_wait_selftest runs
that bounded wait, with a small poll limit, on an mbarrier that nothing
arrives on and no copy is issued to, so the CTA leaves with nothing in
flight. The GPU tests check that the timeout comes back through the caller's
status word, through po_device_error (once, then cleared) and as a host
entry's return code; the CPU tests check the host-side mapping of statuses.
"""
import ctypes

import numpy as np
import pytest


def test_host_mapping_of_statuses(lib):
    """No GPU needed: argument errors are rejected before any CUDA call, and
    a non-zero status becomes a POError carrying the library's message."""
    from pypo_gb300._lib import POError, check
    assert lib.po_wait_selftest(16, None, 7, None) == 1
    assert b"word must be 0" in lib.po_last_error()
    assert lib.po_device_error(None, None) == 1
    with pytest.raises(POError, match="status 1: po_device_error: null code"):
        check(1)
    check(0)


@pytest.mark.gpu
def test_selftest_sets_the_callers_status_word(cuda, lib):
    import torch
    st = torch.zeros(1, dtype=torch.int32, device=cuda)
    s = torch.cuda.current_stream()
    assert lib.po_wait_selftest(1000, st.data_ptr(), 0, ctypes.c_void_p(s.cuda_stream)) == 0, lib.po_last_error()
    torch.cuda.synchronize()
    assert int(st.item()) == 101
    # the context is still usable: a plain torch op and a propagation run
    assert float(torch.ones(4, device=cuda).sum().item()) == 4.0


@pytest.mark.gpu
def test_timeout_through_po_device_error_and_a_host_entry(cuda, lib):
    import torch
    from pypo_gb300 import engine, surfaces as SF
    from pypo_gb300._lib import POError
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    code = ctypes.c_int(-1)
    assert lib.po_device_error(s, ctypes.byref(code)) == 0 and code.value == 0
    assert lib.po_wait_selftest(1000, None, 0, s) == 0, lib.po_last_error()
    assert lib.po_device_error(s, ctypes.byref(code)) == 0 and code.value == 101
    assert lib.po_device_error(s, ctypes.byref(code)) == 0 and code.value == 0
    # a host-buffer entry reads the word after its kernels: a timeout left in
    # it turns into the entry's status 4 and a message
    s7 = engine.generate_grid(SF.paraboloid(2.0, [6, 7], gmode=1, lims_a=[0.1, 1.0]))
    t7 = engine.generate_grid(SF.translate(SF.plane([4, 5], gmode=0, lims_a=[-1, 1]), dz=2.0))
    cur = np.random.default_rng(0).standard_normal((12, s7.shape[1]))
    engine.propagate("EH", s7, cur, 1, 6, 7, t7, 5.0)
    assert lib.po_wait_selftest(1000, None, 0, s) == 0
    torch.cuda.synchronize()
    with pytest.raises(POError, match="status 4: a kernel gave up waiting"):
        engine.propagate("EH", s7, cur, 1, 6, 7, t7, 5.0)
    # cleared by that read: the next call succeeds
    out = engine.propagate("EH", s7, cur, 1, 6, 7, t7, 5.0)
    assert np.isfinite(out).all()
