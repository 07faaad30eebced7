"""Efficiency reductions on the device (po_efficiency_sums_dev) against the
reference's Efficiencies.py outputs (golden vectors)."""
import numpy as np
import pytest

from tests.common import GOLDEN, from_json

pytestmark = pytest.mark.gpu


def test_device_efficiencies_match_reference(cuda, lib):
    import torch
    from pypo_gb300 import efficiencies as E, engine
    g = np.load(GOLDEN / "golden_eff.npz")
    g7 = engine.generate_grid_dev(from_json(str(g["surface_json"])), transform=False, device=cuda)
    n = g7.shape[1]
    block = np.zeros((12, n))
    for c, f in enumerate((g["co"], g["xp"], g["fit"])):   # as Ex, Ey, Ez
        block[c], block[3 + c] = f.real, f.imag
    fields = torch.tensor(block, device=cuda)
    e, r = g["ell"], g["rect"]
    ell = {"shape": "ell", "center": e[0:2], "outer": e[2:4]}
    rect = {"shape": "rect", "center": r[0:2], "outer_x": r[2:4], "outer_y": r[4:6]}
    tol = 1e-12
    assert abs(E.spillover_dev(g7, fields, 0, ell) - g["spill_ell"]) <= tol
    assert abs(E.spillover_dev(g7, fields, 0, rect) - g["spill_rect"]) <= tol
    assert abs(E.taper_dev(g7, fields, 0, ell) - g["taper_ell"]) <= tol
    assert abs(E.taper_dev(g7, fields, 0, rect) - g["taper_rect"]) <= tol
    assert abs(E.taper_dev(g7, fields, 0, None) - g["taper_all"]) <= tol
    assert abs(E.xpol_dev(g7, fields, 0, 1) - g["xpol"]) <= tol
    assert abs(E.main_beam_dev(g7, fields, 0, fields, 2) - g["mainbeam"]) <= tol
    # deterministic: the same sums twice
    assert E.taper_dev(g7, fields, 0, ell) == E.taper_dev(g7, fields, 0, ell)


def test_device_efficiency_rejects_bad_arguments(cuda, lib):
    import ctypes
    import torch
    g7 = torch.zeros((7, 4), dtype=torch.float64, device=cuda)
    sums = torch.zeros(10, dtype=torch.float64, device=cuda)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.po_efficiency_sums_dev(4, p(g7), p(g7), p(g7), None, None, 5, None, p(sums), st) != 0
    assert b"shape" in lib.po_last_error()
    assert lib.po_efficiency_sums_dev(4, p(g7), p(g7), p(g7), None, p(g7), 0, None, p(sums), st) != 0
    assert b"imaginary row without a real row" in lib.po_last_error()
    # a real second field (a fitted Gaussian) needs no imaginary row
    assert lib.po_efficiency_sums_dev(4, p(g7), p(g7), p(g7), p(g7), None, 0, None, p(sums), st) == 0


def test_reference_signatures_match_reference(cuda, lib):
    """calcSpillover / calcTaper / calcXpol / calcMainBeam with the
    reference's own arguments (numpy components shaped like the grid, the
    surface's reflector dict): the grid and the sums made on the device."""
    from pypo_gb300 import efficiencies as E
    g = np.load(GOLDEN / "golden_eff.npz")
    surf = from_json(str(g["surface_json"]))
    shape = tuple(int(v) for v in surf["gridsize"])
    co, xp, fit = (g[k].reshape(shape) for k in ("co", "xp", "fit"))
    e, r = g["ell"], g["rect"]
    ell = {"shape": "ell", "center": e[0:2], "outer": e[2:4]}
    rect = {"shape": "rect", "center": r[0:2], "outer_x": r[2:4], "outer_y": r[4:6]}
    tol = 1e-12
    assert abs(E.calcSpillover(co, surf, ell) - g["spill_ell"]) <= tol
    assert abs(E.calcSpillover(co, surf, rect) - g["spill_rect"]) <= tol
    assert abs(E.calcTaper(co, surf, ell) - g["taper_ell"]) <= tol
    assert abs(E.calcTaper(co, surf, rect) - g["taper_rect"]) <= tol
    assert abs(E.calcTaper(co, surf, None) - g["taper_all"]) <= tol
    assert abs(E.calcTaper(co, surf, {}) - g["taper_all"]) <= tol
    assert abs(E.calcXpol(co, xp) - g["xpol"]) <= tol
    assert abs(E.calcMainBeam(co, surf, fit) - g["mainbeam"]) <= tol
    with pytest.raises(ValueError, match="points"):
        E.calcSpillover(co.ravel()[:-1], surf, ell)
