"""Source producers on the device (po_gauss_beam_dev, po_calc_jm_dev) against
the reference's makeGaussBeam and calcCurrents outputs (golden vectors) and
the host restatements, and a feed generated entirely on the device driving a
propagation."""
import numpy as np
import pytest

from tests.common import GOLDEN, from_json

pytestmark = pytest.mark.gpu


def _close(got, ref, tol=1e-12):
    np.testing.assert_allclose(got, ref, rtol=0, atol=tol * max(1e-300, np.abs(ref).max()))


def test_gauss_beam_dev_matches_reference(cuda, lib):
    import torch
    from pypo_gb300 import beams, engine, surfaces as SF
    g = np.load(GOLDEN / "golden_gauss.npz")
    s7 = engine.generate_grid(from_json(str(g["plane_json"])))
    f, c = beams.gauss_beam_dev(torch.tensor(s7, device=cuda), 3.0, 10.0, 0.0, 4 * np.pi)
    _close(f.cpu().numpy(), g["fields"])
    _close(c.cpu().numpy(), g["currents"])
    s7b = engine.generate_grid(SF.plane([15, 15], gmode=0, lims_a=[-20, 20]))
    f2, c2 = beams.gauss_beam_dev(torch.tensor(s7b, device=cuda), 1.0, 5.0, 50.0, 1.0, mode=2)
    _close(c2.cpu().numpy(), g["currents2"])
    assert torch.all(c2[6:] == 0)
    # behind the waist (z + z0 < 0: conjugated fields) and PMC mode, against the host restatement
    s7c = engine.generate_grid(SF.translate(SF.plane([9, 7], gmode=0, lims_a=[-10, 10]), dz=-3.0))
    fh, ch = beams.gauss_beam(s7c, 2.0, 4.0, 1.0, 2.0, mode=1)
    fd, cd = beams.gauss_beam_dev(torch.tensor(s7c, device=cuda), 2.0, 4.0, 1.0, 2.0, mode=1)
    _close(fd.cpu().numpy(), fh)
    _close(cd.cpu().numpy(), ch)


def test_calc_jm_dev_matches_reference(cuda, lib):
    import torch
    from pypo_gb300 import beams, engine
    g = np.load(GOLDEN / "golden_calcjm.npz")
    s7 = torch.tensor(engine.generate_grid(from_json(str(g["surface_json"]))), device=cuda)
    f = torch.tensor(g["fields"], device=cuda)
    for mode in range(4):
        _close(beams.calc_jm_dev(s7, f, mode).cpu().numpy(), g[f"currents{mode}"], 1e-14)


def test_device_feed_chain_matches_host_chain(cuda, lib):
    """Grid, feed currents and propagation all on the device (the feed -> dish workload,
    reduced) equal the host-built chain."""
    import torch
    from pypo_gb300 import beams, configs, engine
    w = configs.feed_dish_jm(scale=0.3)
    s7d = engine.generate_grid_dev(w["src"], device=cuda)
    _, curd = beams.gauss_beam_dev(s7d, 3.0, 10.0, 0.0, 4 * np.pi)
    t7d = engine.generate_grid_dev(w["tgt"], device=cuda)
    out_d = engine.propagate_dev("JM", s7d, curd, w["gmode"], w["ncx"], w["ncy"], t7d, w["k"])
    out_h = engine.propagate("JM", w["s7"], w["cur"], w["gmode"], w["ncx"], w["ncy"], w["t7"], w["k"])
    rel = float(np.linalg.norm(out_d.cpu().numpy() - out_h) / np.linalg.norm(out_h))
    assert rel <= 1e-6, rel


def test_source_producers_reject_bad_arguments(cuda, lib):
    import ctypes
    import torch
    s7 = torch.zeros((7, 4), dtype=torch.float64, device=cuda)
    out = torch.zeros((12, 4), dtype=torch.float64, device=cuda)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.po_gauss_beam_dev(4, p(s7), -1.0, 1.0, 0.0, 1.0, 0, p(out), p(out), st) != 0
    assert b"wavelength" in lib.po_last_error()
    assert lib.po_gauss_beam_dev(4, p(s7), 1.0, 1.0, 0.0, 1.0, 5, p(out), p(out), st) != 0
    assert lib.po_calc_jm_dev(4, p(s7), p(out), 7, p(out), st) != 0
    assert b"mode" in lib.po_last_error()
    assert lib.po_calc_jm_dev(4, p(s7), None, 0, p(out), st) != 0
