"""Gaussian beam fit on the device.

Mirrors the reference's src/PyPO/FitGauss.py (fitGaussAbs :67-163,
generateGauss :197-228) and the System methods built on it
(System.fitGaussAbs :1828-1874, System.calcMainBeam :1876-1908): same
argument meaning, same defaults (threshold -11 dB, scale LIN, ratio 1), same
parameter order (x0, y0, xs, ys, theta, amp). The work runs in
libpo_gb300 (po_fit_gauss_abs_dev): the pattern, its mask, the fit window,
the moment estimates and every objective value are FP64 reductions on the
device; the downhill simplex (po_fmin, scipy.optimize.fmin's method) runs
on the host between them.

Grids are device grids in the 7-row layout made WITHOUT transform or
spherical mapping (engine.generate_grid_dev(refl, transform=False,
spheric=False)), as the reference's fit regenerates them; fields are
(12, n) float64 device blocks in c2Bundle row order, the component 0-5
(Ex Ey Ez Hx Hy Hz), or a real (n,) amplitude with comp None.
fitGaussAbs and generateGauss take the reference's own arguments (a numpy
field and a reflector dict) and make the grid on the device.
"""
import ctypes

import numpy as np

from ._lib import OBJECTIVE, POError, check, load

#: the reference's Scales enum values (Enums.py:169-191)
SCALES = {"LIN": 0, "AMP": 1, "dB": 2}


def scale_id(scale):
    """0 (LIN), 1 (AMP) or 2 (dB) from an int, a name or an enum member."""
    if isinstance(scale, str):
        key = {"lin": "LIN", "amp": "AMP", "db": "dB"}.get(scale.lower())
        if key is None:
            raise ValueError(f"unknown scale {scale!r}")
        return SCALES[key]
    if hasattr(scale, "value"):
        scale = scale.value
    if int(scale) not in (0, 1, 2):
        raise ValueError(f"unknown scale {scale!r}")
    return int(scale)


def _device_rows(g7, fields, comp):
    import torch
    for name, t in (("g7", g7), ("fields", fields)):
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise POError(f"{name} must be a contiguous float64 CUDA tensor")
    n = g7.shape[1]
    if comp is None:
        if fields.numel() != n:
            raise ValueError("a real amplitude needs one value per grid point")
        return fields.data_ptr(), None
    if not 0 <= comp <= 5:
        raise ValueError("component must be 0-5 (Ex Ey Ez Hx Hy Hz)")
    if fields.dim() != 2 or fields.shape[1] != n or fields.shape[0] < 12:
        raise ValueError("fields must be a (12, n) block on the grid's points")
    r = comp if comp < 3 else comp + 3
    return fields[r].data_ptr(), fields[r + 3].data_ptr()


def _stream(t):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def fit_gauss_abs_dev(g7, ncx, ncy, fields, comp=None, thres=-11.0, scale="LIN", ratio=1.0, full_output=False):
    """Fitted Gaussian parameters (x0, y0, xs, ys, theta, amp) of |field comp|
    (FitGauss.fitGaussAbs, System.fitGaussAbs). ratio None fits once;
    otherwise the fit is repeated with a rising threshold until the fitted
    power over the pattern's is below ratio. With full_output, also the
    simplex's starting point (the image-moment estimates, calcEstimates)."""
    if g7.shape[1] != ncx * ncy:
        raise ValueError("the grid must hold ncx * ncy points")
    fr, fi = _device_rows(g7, fields, comp)
    popt, p0 = np.zeros(6), np.zeros(6)
    thres = -11.0 if thres is None else float(thres)
    use_ratio = ratio is not None
    check(load().po_fit_gauss_abs_dev(int(ncx), int(ncy), ctypes.c_void_p(g7.data_ptr()), ctypes.c_void_p(fr),
                                      ctypes.c_void_p(fi) if fi else None, thres, scale_id(scale), int(use_ratio),
                                      float(ratio) if use_ratio else 0.0, popt.ctypes.data, p0.ctypes.data,
                                      _stream(g7)))
    return (popt, p0) if full_output else popt


def generate_gauss_dev(g7, popt, scale="LIN"):
    """The Gaussian of parameters popt on the grid's points, an (n,) float64
    device tensor (FitGauss.generateGauss)."""
    import torch
    if not (g7.is_cuda and g7.dtype == torch.float64 and g7.is_contiguous()):
        raise POError("g7 must be a contiguous float64 CUDA tensor")
    n = g7.shape[1]
    p = np.ascontiguousarray(popt, dtype=np.float64)
    if p.size != 6:
        raise ValueError("popt holds 6 parameters")
    out = torch.empty(n, dtype=torch.float64, device=g7.device)
    check(load().po_generate_gauss_dev(n, ctypes.c_void_p(g7.data_ptr()), p.ctypes.data, scale_id(scale),
                                       ctypes.c_void_p(out.data_ptr()), _stream(g7)))
    return out


def calc_main_beam_dev(g7, ncx, ncy, fields, comp, thres=-11.0, scale="LIN"):
    """Main-beam efficiency (System.calcMainBeam): the fit at ratio 1, its
    Gaussian in LIN, and the power of the normalised Gaussian over the
    normalised field's (Efficiencies.calcMainBeam), all on the device."""
    import torch
    popt = fit_gauss_abs_dev(g7, ncx, ncy, fields, comp, thres, scale, 1.0)
    psi = generate_gauss_dev(g7, popt, "LIN")
    fr, fi = _device_rows(g7, fields, comp)
    sums = torch.empty(10, dtype=torch.float64, device=g7.device)
    check(load().po_efficiency_sums_dev(g7.shape[1], ctypes.c_void_p(g7.data_ptr()), ctypes.c_void_p(fr),
                                        ctypes.c_void_p(fi) if fi else None, ctypes.c_void_p(psi.data_ptr()),
                                        None, 0, None, ctypes.c_void_p(sums.data_ptr()), _stream(g7)))
    s = sums.cpu().numpy()
    return float((s[6] / s[8]) / (s[5] / s[7]))


def fmin(func, x0, args=(), xtol=1e-4, ftol=1e-4, maxiter=None, maxfun=None, full_output=False):
    """scipy.optimize.fmin's downhill simplex, run natively (po_fmin), on a
    Python objective func(x, *args) -> float. Returns xopt, or (xopt, fopt,
    iterations, function calls) with full_output."""
    x0 = np.ascontiguousarray(np.atleast_1d(x0), dtype=np.float64).ravel()
    n = x0.size
    err = []

    def obj(xp, fxp, _ctx):
        try:
            fxp[0] = float(func(np.ctypeslib.as_array(xp, (n,)).copy(), *args))
            return 0
        except BaseException as e:  # carried back out after the native call returns
            err.append(e)
            return 5

    cb = OBJECTIVE(obj)
    xopt = np.zeros(n)
    fopt = ctypes.c_double()
    nit, nfev = ctypes.c_long(), ctypes.c_long()
    rc = load().po_fmin(n, x0.ctypes.data, float(xtol), float(ftol), int(maxiter or 0), int(maxfun or 0), cb, None,
                        xopt.ctypes.data, ctypes.byref(fopt), ctypes.byref(nit), ctypes.byref(nfev))
    if err:
        raise err[0]
    check(rc)
    if full_output:
        return xopt, fopt.value, nit.value, nfev.value
    return xopt


# ------------------------------------------------- the reference's signatures
#
# FitGauss.fitGaussAbs and FitGauss.generateGauss with the reference's
# arguments: a numpy field component shaped like the surface's grid and the
# surface's reflector dict. The grid (restframe, no spherical mapping, as the
# reference regenerates it) and the fit run on the device.

def _surface(surfaceObject):
    from .engine import generate_grid_dev
    ncx, ncy = (int(v) for v in np.asarray(surfaceObject["gridsize"]).reshape(2))
    return generate_grid_dev(surfaceObject, transform=False, spheric=False), ncx, ncy


def fitGaussAbs(field, surfaceObject, thres, scale, ratio=1):
    """Gaussian parameters (x0, y0, xs, ys, theta, amp) fitted to |field|
    (FitGauss.fitGaussAbs, :71-163); ratio None fits once."""
    import torch
    g7, ncx, ncy = _surface(surfaceObject)
    amp = np.abs(np.asarray(field)).reshape(-1)
    if amp.size != ncx * ncy:
        raise ValueError(f"the field holds {amp.size} values, the surface {ncx * ncy} points")
    return fit_gauss_abs_dev(g7, ncx, ncy, torch.tensor(amp, dtype=torch.float64, device=g7.device), None,
                             thres, scale, ratio)


def generateGauss(p0, surfaceObject, scale):
    """The Gaussian of parameters p0 on the surface's grid, a numpy array
    shaped like the grid (FitGauss.generateGauss, :201-228); scale LIN or dB."""
    g7, ncx, ncy = _surface(surfaceObject)
    return generate_gauss_dev(g7, p0, scale).cpu().numpy().reshape(ncx, ncy)
