"""TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's Gaussian fit.

Follows src/PyPO/FitGauss.py (calcEstimates :13-65, fitGaussAbs :67-163,
GaussAbs :165-195, generateGauss :197-228) and src/PyPO/MatUtils.py
findConnectedSubsets (:9-57), in numpy, with scipy.optimize.fmin as the
minimiser (the reference's own). Grids are passed in as arrays (x, y of the
surface's grid without transform, shaped like the field) instead of being
regenerated from a surface description. Pinned against the reference's own
module run on the same inputs (tests/golden/golden_fitgauss.npz).

Only tests/ import this module. The product (pypo_gb300) never does.
"""
import numpy as np
from scipy.optimize import fmin

LIN, AMP, DB = 0, 1, 2


def run_extent(mask, i0, j0):
    """Ends (inclusive) of the runs of set mask values through (i0, j0):
    along the row i0 (rows_lo, rows_hi, as offsets of i0) and along the
    column j0 (cols_lo, cols_hi, offsets of j0), the reference's crossed
    row/column roles (MatUtils.py:21-55)."""
    def run(line):
        k = 0
        for v in line:
            if not v:
                break
            k += 1
        return k
    up_r, lo_r = run(mask[i0, j0 + 1:]), run(mask[i0, :j0][::-1])
    up_c, lo_c = run(mask[i0 + 1:, j0]), run(mask[:i0, j0][::-1])
    return i0 - lo_r, i0 + up_r, j0 - lo_c, j0 + up_c


def estimates(x, y, f):
    """Image-moment estimates (x0, y0, xm, ym, theta) (FitGauss.py:13-65)."""
    w = np.sum(f)
    xm, ym = np.sum(x * f) / w, np.sum(y * f) / w
    sxx = np.sum(x ** 2 * f) / w - xm ** 2
    syy = np.sum(y ** 2 * f) / w - ym ** 2
    sxy = np.sum(x * y * f) / w - xm * ym
    d = 1 / (2 * (sxx * syy - sxy ** 2))
    a, b, c = syy * d, sxx * d, -sxy * d
    theta = 0.5 * np.arctan(2 * c / (a - b))
    if a - b > 0:
        theta += np.pi / 2
    p = np.sqrt((a - b) ** 2 + 4 * c ** 2)
    u, v = 1 / (a + b - p), 1 / (a + b + p)
    if u <= 0 and v > 0:
        u = v
    elif v <= 0 and u > 0:
        v = u
    elif v <= 0 and u <= 0:
        u, v = -u, -v
    return np.sqrt(u), np.sqrt(v), xm, ym, theta


def gaussian(p, x, y, scale):
    """Rotated elliptical Gaussian of parameters p (FitGauss.py:197-228)."""
    x0, y0, xs, ys, th = p[:5]
    a = np.cos(th) ** 2 / (2 * x0 ** 2) + np.sin(th) ** 2 / (2 * y0 ** 2)
    c = np.sin(2 * th) / (4 * x0 ** 2) - np.sin(2 * th) / (4 * y0 ** 2)
    b = np.sin(th) ** 2 / (2 * x0 ** 2) + np.cos(th) ** 2 / (2 * y0 ** 2)
    e = np.exp(-(a * (x - xs) ** 2 + 2 * c * (x - xs) * (y - ys) + b * (y - ys) ** 2))
    if scale == DB:
        return 20 * np.log10(e)
    if scale == LIN:
        return e
    raise ValueError("the reference's generateGauss defines no Gaussian for this scale")


def misfit(p, x, y, f, sel, scale):
    """|1 - overlap| of the Gaussian with the pattern over sel (FitGauss.py:165-195)."""
    g = gaussian(p, x, y, scale)[sel]
    fs = f[sel]
    c00 = np.sum(fs * g) ** 2 / np.sum(np.abs(fs) ** 2) / np.sum(np.abs(g) ** 2)
    return np.abs(1 - np.abs(c00))


def _fallback(shape):
    # an empty window falls back to an integer array of ones used as an index
    # (FitGauss.py:117-118): every entry picks grid row 1, so each sum runs
    # over row 1 repeated; kept literally, since where x (or y) is constant
    # along a row the moment variances are rounding residue of those sums
    return np.ones(shape, dtype=int)


def fit_region(field, x, y, thres, scale):
    """Pattern (LIN or dB) and the points a ratio-None fit runs over
    (FitGauss.py:84-120): the masked points strictly inside the window, or
    the row-1 fallback."""
    amp = np.abs(field) / np.max(np.abs(field))
    pat = 20 * np.log10(amp) if scale == DB else amp
    mask = pat >= (thres if scale == DB else 10 ** (thres / 20))
    i0, j0 = np.unravel_index(np.argmax(pat), pat.shape)
    r_lo, r_hi, c_lo, c_hi = run_extent(mask, i0, j0)
    window = (x > x[c_lo, i0]) & (x < x[c_hi, i0]) & (y > y[j0, r_lo]) & (y < y[j0, r_hi])
    region = mask & window
    return pat, (region if region.any() else _fallback(region.shape))


def start_point(field, x, y, thres, scale):
    """The simplex's starting point: moment estimates and the pattern maximum."""
    pat, sel = fit_region(field, x, y, thres, scale)
    return np.array([*estimates(x[sel], y[sel], pat[sel]), np.max(pat)])


def fit_gauss_abs(field, x, y, thres, scale, ratio=1.0):
    """Fitted (x0, y0, xs, ys, theta, amp) (FitGauss.py:67-163)."""
    amp = np.abs(field) / np.max(np.abs(field))

    def pattern(t):
        if scale == DB:
            pat = 20 * np.log10(amp)
            return pat, pat >= t
        pat = amp
        return pat, pat >= 10 ** (t / 20)

    pat, mask = pattern(thres)
    i0, j0 = np.unravel_index(np.argmax(pat), pat.shape)
    r_lo, r_hi, c_lo, c_hi = run_extent(mask, i0, j0)
    x_lo, x_hi = x[c_lo, i0], x[c_hi, i0]
    y_lo, y_hi = y[j0, r_lo], y[j0, r_hi]
    window = (x > x_lo) & (x < x_hi) & (y > y_lo) & (y < y_hi)
    region = mask & window
    sel = region if region.any() else _fallback(region.shape)
    p0 = np.array([*estimates(x[sel], y[sel], pat[sel]), np.max(pat)])

    def fit(sel):
        return fmin(lambda p: misfit(p, x, y, pat, sel, scale), p0, disp=False)

    if ratio is None:
        return fit(sel)
    got, rounds, t = ratio, 0, thres
    while got >= ratio:
        pat, mask = pattern(t)
        popt = fit(mask & window if rounds >= 1 else mask)
        got = np.sum(gaussian(popt, x, y, LIN) ** 2) / np.sum(amp ** 2)
        if rounds > 1 and t < -3:
            t += 0.5
        rounds += 1
    return popt


def main_beam(field, psi):
    """Main-beam efficiency of a field against its fitted Gaussian (Efficiencies.py:161-177)."""
    fn = field / np.max(np.abs(field))
    gn = psi / np.max(np.abs(psi))
    return np.sum(np.abs(gn) ** 2) / np.sum(np.abs(fn) ** 2)
