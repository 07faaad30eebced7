"""TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's efficiencies.

Follows src/PyPO/Efficiencies.py in numpy: the aperture mask (_generateMask,
:11-41; ellipse or rectangle, its outer condition only), spillover
(calcSpillover, :90-115), taper (calcTaper, :117-145), cross-polar
(calcXpol, :147-159) and main-beam (calcMainBeam, :161-177) efficiencies.
Grids are passed in as arrays (x, y, area of the surface's grid without
transform) instead of being regenerated. Pinned against the reference's own
module run on the same field (tests/golden/golden_eff.npz).

Only tests/ import this module. The product (pypo_gb300) never does.
"""
import numpy as np


def _shape(aper):
    if not aper:
        return 0
    name = str(getattr(aper["shape"], "name", aper["shape"])).lower()
    return {"ell": 1, "ellipse": 1, "rect": 2, "rectangle": 2}[name]


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


