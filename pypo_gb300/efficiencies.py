"""Efficiencies of a field on a surface (far field or aperture).

Mirrors the reference's src/PyPO/Efficiencies.py: the aperture mask
(_generateMask, :11-41; ellipse or rectangle, its outer condition only, as in
the reference), spillover (calcSpillover, :90-115), taper (calcTaper,
:117-145), cross-polar (calcXpol, :147-159) and main-beam (calcMainBeam,
:161-177) efficiencies.

Every sum runs on the GPU (po_efficiency_sums_dev, FP64, deterministic)
and the functions return Python floats. The `*_dev` functions take a
(7, n) device grid and (12, n) device field blocks plus a component index;
calcSpillover, calcTaper, calcXpol and calcMainBeam take the reference's own
arguments (numpy field components and reflector dicts) and make the grid on
the device. Aperture dicts use the
reference's keys: {"shape": "ell", "center", "outer"} or {"shape": "rect",
"center", "outer_x", "outer_y"} ("shape" may also be the reference's enum).
"""
import numpy as np


def _shape(aper):
    if not aper:
        return 0
    s = aper["shape"]
    name = getattr(s, "name", s)
    name = str(name).lower()
    if name in ("ell", "ellipse"):
        return 1
    if name in ("rect", "rectangle"):
        return 2
    raise ValueError(f"unknown aperture shape {s!r}")


# ------------------------------------------------------------------ device

def _aper_params(aper):
    shape = _shape(aper)
    if shape == 1:
        p = np.r_[np.asarray(aper["center"], float), np.asarray(aper["outer"], float)]
    elif shape == 2:
        p = np.r_[np.asarray(aper["center"], float), np.asarray(aper["outer_x"], float),
                  np.asarray(aper["outer_y"], float)]
    else:
        p = np.zeros(1)
    return shape, np.ascontiguousarray(p, dtype=np.float64)


def _check_dev(**tensors):
    import torch
    from ._lib import POError
    for name, t in tensors.items():
        if t is not None and not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise POError(f"{name} must be a contiguous float64 CUDA tensor")


def _sums_rows(g7, fr, fi, aper=None, gr=None, gi=None):
    """The 10 device sums (po_efficiency_sums_dev) of field rows fr, fi and
    second-field rows gr, gi (device tensors of n values, or None) on the
    (7, n) device grid g7, as a numpy array."""
    import ctypes
    import torch
    from ._lib import check, load
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    shape, p = _aper_params(aper)
    sums = torch.empty(10, dtype=torch.float64, device=g7.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(g7.device).cuda_stream)
    check(load().po_efficiency_sums_dev(g7.shape[1], ptr(g7), ptr(fr), ptr(fi), ptr(gr), ptr(gi), shape,
                                        p.ctypes.data, ctypes.c_void_p(sums.data_ptr()), st))
    return sums.cpu().numpy()


def _sums_dev(g7, fields, comp, aper=None, fields2=None, comp2=None):
    """The 10 device sums of row comp (and comp + 3) of a (12, n) device block."""
    _check_dev(g7=g7, fields=fields, fields2=fields2)
    gr = fields2[comp2] if fields2 is not None else None
    gi = fields2[comp2 + 3] if fields2 is not None else None
    return _sums_rows(g7, fields[comp], fields[comp + 3], aper, gr, gi)


# The efficiencies from the sums (0 sum |f|^2 A, 1 the same in the aperture,
# 2, 3 sum Re f A, Im f A in the aperture, 4 aperture area, 5 sum |f|^2,
# 6 sum |g|^2, 7 max |f|^2, 8 max |g|^2): the reference's formulas with its
# NaN -> 0 rule. Spillover |sum_m conj(f) f A|^2 / (s0 s1) is s1 / s0.
def _spill(s):
    return 0.0 if s[0] == 0 or s[1] == 0 else float(s[1] / s[0])


def _taper(s):
    den = s[1] * s[4]
    return 0.0 if den == 0 else float((s[2] ** 2 + s[3] ** 2) / den)


def _xpol(s):
    return float(1 - s[6] / (s[5] + s[6]))


def _main_beam(s):
    return float((s[6] / s[8]) / (s[5] / s[7]))


def _row(c):
    """Real row of component c (0-5: Ex Ey Ez Hx Hy Hz) in a (12, n) block; the imaginary row is +3."""
    if not 0 <= c <= 5:
        raise ValueError("component must be 0-5 (Ex Ey Ez Hx Hy Hz)")
    return c if c < 3 else c + 3


def spillover_dev(g7, fields, comp, aper):
    return _spill(_sums_dev(g7, fields, _row(comp), aper))


def taper_dev(g7, fields, comp, aper=None):
    return _taper(_sums_dev(g7, fields, _row(comp), aper))


def xpol_dev(g7, fields, co_comp, x_comp, x_fields=None):
    x_fields = fields if x_fields is None else x_fields
    return _xpol(_sums_dev(g7, fields, _row(co_comp), None, x_fields, _row(x_comp)))


def main_beam_dev(g7, fields, comp, fit_fields, fit_comp):
    return _main_beam(_sums_dev(g7, fields, _row(comp), None, fit_fields, _row(fit_comp)))


# ------------------------------------------------- the reference's signatures
#
# Efficiencies.calcSpillover / calcTaper / calcXpol / calcMainBeam with the
# reference's arguments: numpy field components shaped like the surface's
# grid (any shape with one value per point) and reflector / aperture dicts.
# The surface's grid (restframe, as the reference regenerates it) and every
# sum are made on the device; the fields cross once, host to device.

def _field_rows(field, n, dev):
    """(2, n) float64 device rows (re, im) of a numpy field of n values."""
    import torch
    f = np.asarray(field).reshape(-1)
    if f.size != n:
        raise ValueError(f"the field holds {f.size} values, the surface {n} points")
    return torch.tensor(np.stack([f.real, f.imag]), dtype=torch.float64, device=dev)


def _surface_dev(surfaceObject, spheric):
    from .engine import generate_grid_dev
    return generate_grid_dev(surfaceObject, transform=False, spheric=spheric)


def _no_grid(n):
    """A zero grid for the sums that use no position or area (xpol, main beam)."""
    import torch
    return torch.zeros((7, n), dtype=torch.float64, device="cuda")


def calcSpillover(field, surfaceObject, aperDict):
    """Spillover efficiency of a field component on an aperture
    (Efficiencies.calcSpillover, :90-115)."""
    g7 = _surface_dev(surfaceObject, True)
    f = _field_rows(field, g7.shape[1], g7.device)
    return _spill(_sums_rows(g7, f[0], f[1], aperDict))


def calcTaper(field, surfaceObject, aperDict):
    """Taper efficiency of a field component, over an aperture or (aperDict
    None or empty) the whole surface (Efficiencies.calcTaper, :117-145)."""
    g7 = _surface_dev(surfaceObject, True)
    f = _field_rows(field, g7.shape[1], g7.device)
    return _taper(_sums_rows(g7, f[0], f[1], aperDict or None))


def calcXpol(Cofield, Xfield):
    """Cross-polar efficiency of a co- and a cross-polar component
    (Efficiencies.calcXpol, :147-159)."""
    n = np.size(Cofield)
    g7 = _no_grid(n)
    co, xp = _field_rows(Cofield, n, g7.device), _field_rows(Xfield, n, g7.device)
    return _xpol(_sums_rows(g7, co[0], co[1], None, xp[0], xp[1]))


def calcMainBeam(field, surfaceObject, fitGauss):
    """Main-beam efficiency of a field component against its fitted Gaussian
    (Efficiencies.calcMainBeam, :161-177; the surface is not used there
    either)."""
    n = np.size(field)
    g7 = _no_grid(n)
    f, g = _field_rows(field, n, g7.device), _field_rows(fitGauss, n, g7.device)
    return _main_beam(_sums_rows(g7, f[0], f[1], None, g[0], g[1]))
