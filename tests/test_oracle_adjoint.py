"""The oracle's FP64 adjoint (po_oracle_adjoint) against central finite
differences of the oracle's forward, on CPU: current entries, source and
target normal displacement, every mode with an adjoint and both time
directions. The bar is 1e-6 relative (FP64 with h = 1e-3 on currents and
1e-6 wavelengths on displacements)."""
import numpy as np
import pytest

from oracle import grids as OG


def _case(rng, mode):
    s7 = OG.generate(OG.paraboloid(3.0, [7, 8], gmode=1, lims_a=[0.2, 2.0]))
    if mode == "FF":
        t7 = OG.generate(OG.farfield([5, 4], [-20, 20], [-15, 15]))
    else:
        t7 = OG.generate(OG.translate(OG.plane([5, 4], gmode=0, lims_a=[-1, 1]), dz=3.0))
        t7[3:6] *= -1.0
    nc = 2 if mode == "scalar" else 12
    cur = rng.standard_normal((nc, s7.shape[1]))
    nout = {"scalar": 2, "JMEH": 24}.get(mode, 12)
    cot = rng.standard_normal((nout, t7.shape[1]))
    return s7, cur, t7, cot, (1, 7, 8)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("mode", ["EH", "JM", "JMEH", "FF", "scalar"])
@pytest.mark.parametrize("t", [-1.0, 1.0])
def test_oracle_adjoint_matches_finite_differences(oracle_mod, mode, t):
    O = oracle_mod
    rng = np.random.default_rng({"EH": 1, "JM": 2, "JMEH": 3, "FF": 4, "scalar": 5}[mode] * 10 + (t > 0))
    s7, cur, t7, cot, grid = _case(rng, mode)
    k = 2 * np.pi / 0.9
    loss = lambda s, c, tt: float((cot * O.run(mode, s, c, *grid, tt, k, 1.0, t, nthreads=4)).sum())
    g = O.adjoint(mode, s7, cur, *grid, t7, k, cot, 1.0, t, nthreads=4)
    h_c, h_d = 1e-3, 1e-6 * (2 * np.pi / k)
    rows = rng.integers(0, cur.shape[0], 6)
    cols = rng.integers(0, s7.shape[1], 6)
    fc = []
    for r, c in zip(rows, cols):
        cp, cm = cur.copy(), cur.copy()
        cp[r, c] += h_c
        cm[r, c] -= h_c
        fc.append((loss(s7, cp, t7) - loss(s7, cm, t7)) / (2 * h_c))
    assert _rel(g["cur"][rows, cols], np.array(fc)) <= 1e-6

    def moved(p7, i, h):
        q = p7.copy()
        q[:3, i] += h * p7[3:6, i]
        return q

    si = rng.choice(s7.shape[1], 6, replace=False)
    fs = [(loss(moved(s7, i, h_d), cur, t7) - loss(moved(s7, i, -h_d), cur, t7)) / (2 * h_d) for i in si]
    assert _rel(g["ds"][si], np.array(fs)) <= 1e-6
    if mode != "FF":
        ti = rng.choice(t7.shape[1], 6, replace=False)
        ft = [(loss(s7, cur, moved(t7, j, h_d)) - loss(s7, cur, moved(t7, j, -h_d))) / (2 * h_d) for j in ti]
        assert _rel(g["dt"][ti], np.array(ft)) <= 1e-6
    else:
        assert "dt" not in g


def test_oracle_adjoint_rejects_ehp_and_handles_empty(oracle_mod):
    O = oracle_mod
    s7 = OG.generate(OG.plane([3, 3], gmode=0, lims_a=[-1, 1]))
    t7 = s7.copy()
    t7[2] += 1.0
    with pytest.raises(RuntimeError):
        O.adjoint("EHP", s7, np.ones((12, 9)), 0, 3, 3, t7, 3.0, np.ones((15, 9)))
    g = O.adjoint("EH", s7, np.ones((12, 9)), 0, 3, 3, t7[:, :0], 3.0, np.ones((12, 0)))
    assert not g["cur"].any() and not g["ds"].any() and g["dt"].size == 0
