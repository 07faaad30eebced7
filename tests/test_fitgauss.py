"""Gaussian beam fit, CPU side: the oracle against the reference's own fits
(tests/golden/golden_fitgauss.npz, made by make_golden.py from the
reference's FitGauss.py), and the library's native downhill simplex
(po_fmin) against scipy.optimize.fmin, the minimiser the reference calls."""
import pathlib

import numpy as np
import pytest

from oracle import fitgauss as OF

pytestmark = pytest.mark.filterwarnings("ignore::RuntimeWarning")   # log10(0) in dB patterns

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "golden_fitgauss.npz"


def _golden():
    return np.load(GOLDEN)


def fit_keys():
    g = _golden()
    return sorted(k for k in g.files if "__s" in k and "__r" in k and not k.endswith("__loop"))


def _parse(key):
    name, s, t, r = key.split("__")
    return name, int(s[1:]), float(t[1:]), None if r == "rnone" else float(r[1:])


@pytest.mark.parametrize("key", fit_keys())
def test_oracle_matches_reference_fit(key):
    g = _golden()
    name, scale, thres, ratio = _parse(key)
    field, x, y = g[name + "__field"], g[name + "__x"], g[name + "__y"]
    popt = OF.fit_gauss_abs(np.abs(field), x, y, thres, scale, ratio)
    np.testing.assert_array_equal(popt, g[key])


def test_oracle_main_beam_matches_reference():
    g = _golden()
    field, x, y = g["airy_ff__field"], g["airy_ff__x"], g["airy_ff__y"]
    for scale in (0, 2):
        popt = OF.fit_gauss_abs(np.abs(field), x, y, -11.0, scale, 1.0)
        eff = OF.main_beam(field, OF.gaussian(popt, x, y, OF.LIN))
        assert eff == pytest.approx(float(g[f"airy_ff__mainbeam_s{scale}"]), rel=1e-14)


def test_oracle_window_past_the_grid_raises_like_the_reference():
    g = _golden()
    assert "out of bounds" in str(g["gauss_xy__t-100__error"])
    with pytest.raises(IndexError):
        OF.fit_gauss_abs(np.abs(g["gauss_xy__field"]), g["gauss_xy__x"], g["gauss_xy__y"], -100.0, OF.LIN, None)


def test_amp_scale_has_no_gaussian():
    with pytest.raises(ValueError):
        OF.gaussian(np.ones(6), np.zeros(3), np.zeros(3), OF.AMP)


def _rosen(x):
    return float(np.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2))


def _bowl(x):
    k = np.arange(x.size)
    return float(np.sum((x - k) ** 2 * (1 + k)))


def _nan_past(x):
    return float("nan") if x[0] > 1.3 else _rosen(x)


FMIN_CASES = [
    (_rosen, [1.3, 0.7, 0.8, 1.9, 1.2], {}),
    (_rosen, [-1.2, 1.0], {}),
    (_bowl, [0.0, 0.0, 0.0], {}),
    (_rosen, [-1.2, 1.0], {"maxfun": 37}),     # aborted in the middle of a step
    (_rosen, [-1.2, 1.0], {"maxiter": 15}),
    (_nan_past, [1.0, 1.0, 0.5], {}),          # NaN values sort last
]


@pytest.mark.parametrize("case", range(len(FMIN_CASES)))
def test_native_simplex_follows_scipy_fmin_exactly(case):
    """Same vertices, same value, same iteration and call counts as scipy's
    fmin (objectives without exactly tied values: scipy orders ties with
    numpy's argsort, whose order for equal keys depends on the platform's
    sort; the native sort is stable)."""
    from scipy.optimize import fmin as scipy_fmin
    from pypo_gb300 import fitgauss as FG
    f, x0, kw = FMIN_CASES[case]
    xa, fa, ita, nfa = scipy_fmin(f, x0, full_output=True, disp=False, **kw)[:4]
    xb, fb, itb, nfb = FG.fmin(f, x0, full_output=True, **kw)
    np.testing.assert_array_equal(xb, xa)
    assert (fb == fa) or (np.isnan(fa) and np.isnan(fb))
    assert (itb, nfb) == (ita, nfa)


def test_native_simplex_carries_objective_errors():
    from pypo_gb300 import fitgauss as FG

    def bad(x):
        if x[0] > 0.5:
            raise ZeroDivisionError("planted")
        return float(x @ x)

    with pytest.raises(ZeroDivisionError):
        FG.fmin(bad, [0.49, 0.1])   # the initial simplex steps x[0] to 0.5145


def test_db_misfit_is_invariant_to_the_beam_scale():
    """In dB the reference's Gaussian is 20 log10(exp(-Q)) = -(20 / ln 10) Q, and
    scaling (x0, y0) by s scales Q by 1 / s^2; the misfit, a normalised overlap,
    does not change. So a dB fit has a valley of equal misfit along the beam's
    scale and ends wherever the simplex's path, set by last-bit rounding, leaves
    it. In LIN the misfit does change with the scale."""
    g = _golden()
    field, x, y = g["airy_ff__field"], g["airy_ff__x"], g["airy_ff__y"]
    p = g["airy_ff__s0__t-11__rnone"]
    for scale, same in ((OF.DB, True), (OF.LIN, False)):
        pat, sel = OF.fit_region(field, x, y, -11.0, scale)
        m = [OF.misfit(p * np.array([s, s, 1, 1, 1, 1]), x, y, pat, sel, scale) for s in (1.0, 0.5, 3.0)]
        if same:
            np.testing.assert_allclose(m, m[0], rtol=1e-9)
        else:
            assert min(abs(m[1] - m[0]), abs(m[2] - m[0])) > 1e-3
