"""Reflector dicts in the layout PyPO's bindings consume.

The keys are those read by reference src/PyPO/BindUtils.py:277-327
(allfill_reflparams): type (0 paraboloid, 1 hyperboloid, 2 ellipsoid,
3 plane), gmode (0 xy, 1 uv, 2 AoE), coeffs (a, b, c), lims_x/lims_y |
lims_u/lims_v (v in degrees) | lims_Az/lims_El (degrees), gcenter,
gridsize, flip, ecc_uv, rot_uv (degrees), transf (4x4, row major), rms,
rms_seed. Coefficient conventions follow reference src/PyPO/System.py:244-442:
a paraboloid z = x^2/a^2 + y^2/b^2 with focal length f has a = b = 2 sqrt(f);
a hyperboloid/ellipsoid z = c sqrt(1 +- ...) uses (a, b, c) directly.
"""
import numpy as np


def _base(rtype, gmode, gridsize, **kw):
    d = {"type": rtype, "gmode": gmode, "gridsize": np.asarray(gridsize, dtype=int),
         "coeffs": np.zeros(3), "gcenter": np.zeros(2), "flip": False, "ecc_uv": 0.0,
         "rot_uv": 0.0, "transf": np.eye(4), "rms": 0.0, "rms_seed": 0}
    d.update(kw)
    return d


def _lims(gmode, lims_a, lims_b):
    key = {0: ("lims_x", "lims_y"), 1: ("lims_u", "lims_v"), 2: ("lims_Az", "lims_El")}[gmode]
    return {key[0]: np.asarray(lims_a, dtype=float), key[1]: np.asarray(lims_b, dtype=float)}


def paraboloid(f, gridsize, gmode=1, lims_a=None, lims_b=None, **kw):
    """On-axis paraboloid z = (x^2 + y^2) / (4 f). gmode 1 (uv) by default."""
    a = 2.0 * np.sqrt(f)
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(0, gmode, gridsize, coeffs=np.array([a, a, -1.0]), **_lims(gmode, lims_a, lims_b), **kw)


def hyperboloid(a, b, c, gridsize, gmode=1, lims_a=None, lims_b=None, **kw):
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(1, gmode, gridsize, coeffs=np.array([a, b, c], dtype=float),
                 **_lims(gmode, lims_a, lims_b), **kw)


def ellipsoid(a, b, c, gridsize, gmode=0, lims_a=None, lims_b=None, **kw):
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(2, gmode, gridsize, coeffs=np.array([a, b, c], dtype=float),
                 **_lims(gmode, lims_a, lims_b), **kw)


def plane(gridsize, gmode=0, lims_a=(-1.0, 1.0), lims_b=None, **kw):
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(3, gmode, gridsize, **_lims(gmode, lims_a, lims_b), **kw)


def farfield(gridsize, lims_Az, lims_El, **kw):
    """Az-over-El far-field grid (degrees); the grid holds (polar, azimuth) in radians."""
    return _base(3, 2, gridsize, **_lims(2, lims_Az, lims_El), **kw)


def translate(d, dx=0.0, dy=0.0, dz=0.0):
    m = np.eye(4)
    m[:3, 3] = [dx, dy, dz]
    d = dict(d)
    d["transf"] = m @ np.asarray(d["transf"])
    return d


def rotate_x(d, deg):
    t = np.deg2rad(deg)
    m = np.eye(4)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = np.cos(t), -np.sin(t), np.sin(t), np.cos(t)
    d = dict(d)
    d["transf"] = m @ np.asarray(d["transf"])
    return d
