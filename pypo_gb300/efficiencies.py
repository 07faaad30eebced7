"""Efficiencies of a field on a surface (far field or aperture).

Restates the reference's src/PyPO/Efficiencies.py: the aperture mask
(_generateMask, :11-41; ellipse or rectangle, its outer condition only, as in
the reference), spillover (calcSpillover, :90-115), taper (calcTaper,
:117-145), cross-polar (calcXpol, :147-159) and main-beam (calcMainBeam,
:161-177) efficiencies.

Host functions take numpy arrays (one complex field component and the
surface's x, y, area, from a grid generated with transform=False as the
reference does). The `*_dev` functions take a (7, n) device grid and
(12, n) device field blocks plus a component index, reduce on the GPU
(po_efficiency_sums_dev) and return Python floats. Aperture dicts use the
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


def aperture_mask(x, y, aper):
    """Boolean mask of the points inside the aperture (all points for None)."""
    shape = _shape(aper)
    if shape == 0:
        return np.ones(np.shape(x), dtype=bool)
    c = np.asarray(aper["center"], dtype=float)
    if shape == 1:
        t = np.arctan2(y, x) + np.pi
        o = np.asarray(aper["outer"], dtype=float)
        outer = (o[0] * np.cos(t)) ** 2 + (o[1] * np.sin(t)) ** 2
        return (x - c[0]) ** 2 + (y - c[1]) ** 2 < outer
    ox, oy = np.asarray(aper["outer_x"], dtype=float), np.asarray(aper["outer_y"], dtype=float)
    return ((x - c[0]) > ox[0]) & ((x - c[0]) < ox[1]) & ((y - c[1]) > oy[0]) & ((y - c[1]) < oy[1])


def spillover(field, x, y, area, aper):
    m = aperture_mask(x, y, aper)
    f_ap = field * m
    a_m = area * m
    eff = np.abs(np.sum(np.conj(f_ap) * field * area)) ** 2 / (
        np.sum(np.abs(field) ** 2 * area) * np.sum(np.abs(f_ap) ** 2 * a_m))
    return 0.0 if np.isnan(eff) else float(eff)


def taper(field, x, y, area, aper=None):
    if aper:
        m = aperture_mask(x, y, aper)
        field, area = field[m], area[m]
    eff = np.abs(np.sum(field * area)) ** 2 / np.sum(np.abs(field) ** 2 * area) / np.sum(area)
    return 0.0 if np.isnan(eff) else float(eff)


def xpol(co, x_field):
    return float(1 - np.sum(np.abs(x_field) ** 2) / (np.sum(np.abs(co) ** 2) + np.sum(np.abs(x_field) ** 2)))


def main_beam(field, fit):
    fn = field / np.max(np.abs(field))
    gn = fit / np.max(np.abs(fit))
    return float(np.sum(np.abs(gn) ** 2) / np.sum(np.abs(fn) ** 2))


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


def _sums_dev(g7, fields, comp, aper=None, fields2=None, comp2=None):
    """The 10 device sums (po_efficiency_sums_dev) as a numpy array."""
    import ctypes
    import torch
    from ._lib import POError, check, load
    for name, t in (("g7", g7), ("fields", fields)) + ((("fields2", fields2),) if fields2 is not None else ()):
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise POError(f"{name} must be a contiguous float64 CUDA tensor")
    n = g7.shape[1]
    row = lambda f, r: ctypes.c_void_p(f[r].data_ptr())
    gre = row(fields2, comp2) if fields2 is not None else None
    gim = row(fields2, comp2 + 3) if fields2 is not None else None
    shape, p = _aper_params(aper)
    sums = torch.empty(10, dtype=torch.float64, device=g7.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(g7.device).cuda_stream)
    check(load().po_efficiency_sums_dev(n, ctypes.c_void_p(g7.data_ptr()), row(fields, comp), row(fields, comp + 3),
                                        gre, gim, shape, p.ctypes.data, ctypes.c_void_p(sums.data_ptr()), st))
    return sums.cpu().numpy()


def _row(c):
    """Real row of component c (0-5: Ex Ey Ez Hx Hy Hz) in a (12, n) block; the imaginary row is +3."""
    if not 0 <= c <= 5:
        raise ValueError("component must be 0-5 (Ex Ey Ez Hx Hy Hz)")
    return c if c < 3 else c + 3


def spillover_dev(g7, fields, comp, aper):
    s = _sums_dev(g7, fields, _row(comp), aper)
    return 0.0 if s[0] == 0 or s[1] == 0 else float(s[1] / s[0])


def taper_dev(g7, fields, comp, aper=None):
    s = _sums_dev(g7, fields, _row(comp), aper)
    den = s[1] * s[4]
    return 0.0 if den == 0 else float((s[2] ** 2 + s[3] ** 2) / den)


def xpol_dev(g7, fields, co_comp, x_comp, x_fields=None):
    x_fields = fields if x_fields is None else x_fields
    s = _sums_dev(g7, fields, _row(co_comp), None, x_fields, _row(x_comp))
    return float(1 - s[6] / (s[5] + s[6]))


def main_beam_dev(g7, fields, comp, fit_fields, fit_comp):
    s = _sums_dev(g7, fields, _row(comp), None, fit_fields, _row(fit_comp))
    return float((s[6] / s[8]) / (s[5] / s[7]))
