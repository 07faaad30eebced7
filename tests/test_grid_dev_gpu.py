"""FP64 grid generation on the device (po_generate_grid_dev) against the
reference's own grids (golden vectors made by running the reference's grid
generator, tests/golden/make_golden.py) and against the host generator, for
every surface type and grid mode, the 4x4 transform and the rms surface
error (the reference's mt19937 sequence)."""
import numpy as np
import pytest

from tests.common import GOLDEN, from_json

pytestmark = pytest.mark.gpu

CASES = ["par_xy", "par_uv", "hyp_xy", "hyp_uv", "ell_xy", "ell_uv", "pl_xy", "pl_uv", "aoe", "par_rms"]


@pytest.mark.parametrize("name", CASES)
def test_device_grid_matches_reference_and_host(cuda, lib, name):
    from pypo_gb300 import engine
    g = np.load(GOLDEN / "golden_grids.npz")
    d = from_json(str(g[f"{name}_json"]))
    ref = g[f"{name}_grid"]
    got = engine.generate_grid_dev(d, device=cuda).cpu().numpy()
    tol = 1e-13 * max(1.0, np.abs(ref).max())
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol)
    np.testing.assert_allclose(got, engine.generate_grid(d), rtol=0, atol=tol)


def test_device_grid_feeds_propagation(cuda, lib):
    """A grid generated on the device, propagated without leaving it, equals
    the propagation of the host-generated grid."""
    import torch
    from pypo_gb300 import configs, engine
    w = configs.dish_eh(scale=0.05)
    s7d = engine.generate_grid_dev(w["src"], device=cuda)
    t7d = engine.generate_grid_dev(w["tgt"], device=cuda)
    np.testing.assert_allclose(s7d.cpu().numpy(), w["s7"], rtol=0, atol=1e-13 * np.abs(w["s7"]).max())
    cur = torch.tensor(w["cur"], device=cuda)
    a = engine.propagate_dev("EH", s7d, cur, w["gmode"], w["ncx"], w["ncy"], t7d, w["k"], m_zero=True)
    b = engine.propagate_dev("EH", torch.tensor(w["s7"], device=cuda), cur, w["gmode"], w["ncx"], w["ncy"],
                             torch.tensor(w["t7"], device=cuda), w["k"], m_zero=True)
    rel = float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
    assert rel <= 1e-6, rel


def test_device_grid_rejects_bad_arguments(cuda, lib):
    """Invalid grid mode, sizes or output pointer: a status and a message from
    the C-ABI, no launch."""
    import ctypes
    import torch
    from pypo_gb300 import marshal as M
    g = np.load(GOLDEN / "golden_grids.npz")
    d = from_json(str(g["par_xy_json"]))
    out = torch.empty((7, int(np.prod(d["gridsize"]))), dtype=torch.float64, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rp, keep = M.fill_reflparams(d, ctypes.c_double)
    rp.gmode = 7
    assert lib.po_generate_grid_dev(rp, ctypes.c_void_p(out.data_ptr()), 1, 1, stream) != 0
    assert b"gmode" in lib.po_last_error()
    rp, keep = M.fill_reflparams(d, ctypes.c_double)
    assert lib.po_generate_grid_dev(rp, None, 1, 1, stream) != 0
    assert b"null" in lib.po_last_error()
