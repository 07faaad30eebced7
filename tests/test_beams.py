"""Source producers (pypo_gb300.beams) against the reference's outputs
(golden vectors): makeGaussBeam in full and PEC modes, calcCurrents in every
mode; and the oracle's restatement of the efficiencies pinned to the
reference's Efficiencies.py."""
import numpy as np

from tests.common import GOLDEN, from_json


def test_gauss_beam_matches_reference(lib):
    from pypo_gb300 import beams, engine, surfaces as SF
    g = np.load(GOLDEN / "golden_gauss.npz")
    s7 = engine.generate_grid(from_json(str(g["plane_json"])))
    f, c = beams.gauss_beam(s7, 3.0, 10.0, 0.0, 4 * np.pi)
    np.testing.assert_allclose(f, g["fields"], rtol=0, atol=1e-13 * np.abs(g["fields"]).max())
    np.testing.assert_allclose(c, g["currents"], rtol=0, atol=1e-13 * np.abs(g["currents"]).max())
    s7b = engine.generate_grid(SF.plane([15, 15], gmode=0, lims_a=[-20, 20]))
    f2, c2 = beams.gauss_beam(s7b, 1.0, 5.0, 50.0, 1.0, mode=2)
    np.testing.assert_allclose(c2, g["currents2"], rtol=0, atol=1e-13 * np.abs(g["currents2"]).max())
    assert np.all(c2[6:] == 0)   # PEC mode: no magnetic current


def test_calc_jm_matches_reference(lib):
    """Equivalent currents of seeded fields on a rotated, shifted uv paraboloid
    against the reference's calcCurrents, every mode."""
    from pypo_gb300 import beams, engine
    g = np.load(GOLDEN / "golden_calcjm.npz")
    s7 = engine.generate_grid(from_json(str(g["surface_json"])))
    for mode in range(4):
        ref = g[f"currents{mode}"]
        got = beams.calc_jm(s7, g["fields"], mode)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14 * np.abs(ref).max(), err_msg=f"mode {mode}")


def test_efficiencies_match_reference():
    """Spillover, taper, cross-polar and main-beam efficiencies against the
    reference's Efficiencies.py run on the same field (golden vectors)."""
    from oracle import efficiencies as E
    from pypo_gb300 import engine
    g = np.load(GOLDEN / "golden_eff.npz")
    b = engine.generate_grid(from_json(str(g["surface_json"])), transform=False)
    x, y, a = b[0], b[1], b[6]
    e, r = g["ell"], g["rect"]
    ell = {"shape": "ell", "center": e[0:2], "outer": e[2:4]}
    rect = {"shape": "rect", "center": r[0:2], "outer_x": r[2:4], "outer_y": r[4:6]}
    assert abs(E.spillover(g["co"], x, y, a, ell) - g["spill_ell"]) <= 1e-13
    assert abs(E.spillover(g["co"], x, y, a, rect) - g["spill_rect"]) <= 1e-13
    assert abs(E.taper(g["co"], x, y, a, ell) - g["taper_ell"]) <= 1e-13
    assert abs(E.taper(g["co"], x, y, a, rect) - g["taper_rect"]) <= 1e-13
    assert abs(E.taper(g["co"], x, y, a, None) - g["taper_all"]) <= 1e-13
    assert abs(E.xpol(g["co"], g["xp"]) - g["xpol"]) <= 1e-13
    assert abs(E.main_beam(g["co"], g["fit"]) - g["mainbeam"]) <= 1e-13
