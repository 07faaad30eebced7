"""TEST INFRASTRUCTURE ONLY: CPU restatement of the grid-size convergence
searches System.autoConverge and System.convergeOnTarget (reference
src/PyPO/System.py:2779-2880, :2882-3086), driving the FP64 oracle's scalar
propagation (oracle/po_oracle.c) on host grids. The loops, their start
sizes, stopping rules and returned sizes follow the reference line by line;
the grids come from pypo_gb300.engine.generate_grid, which the golden grid
vectors pin to the reference's generator.

Only tests/ import this module. The product (pypo_gb300) never does.
"""
import numpy as np

from oracle import oracle as O

_LIMS = {0: ("lims_x", "lims_y"), 1: ("lims_u", "lims_v")}


def strongest(block):
    """(2, n) scalar field of a (12, n) block's strongest component (or the
    (2, n) field itself)."""
    if block.shape[0] == 2:
        return block
    peaks = [np.max(np.abs(block[(c if c < 3 else c + 3)] + 1j * block[(c if c < 3 else c + 3) + 3]))
             for c in range(6)]
    c = int(np.argmax(peaks))
    r = c if c < 3 else c + 3
    return np.stack([block[r], block[r + 3]])


def _scalar(src7, s2, grid, t7, k, eps=1.0):
    out = O.run("scalar", src7, s2, grid[0], grid[1], grid[2], t7, k, eps, -1.0)
    return out[0] + 1j * out[1]


def auto_converge(src7, src_grid, fields, target, k, tol=1e-2, add=10, patch_size=1 / 9, max_iter=1000):
    from pypo_gb300 import engine
    kx, ky = _LIMS[int(target["gmode"])]
    patch = dict(target)
    patch[kx] = patch_size * np.asarray(target[kx], float)
    patch[ky] = patch_size * np.asarray(target[ky], float)
    s2 = strongest(fields)
    gridsize = np.array([1, 1])
    diff, p0, norm, n, powers = 1e99, 1e99, 1.0, 0, []
    while np.absolute(diff) > tol:
        gridsize = gridsize + add
        patch["gridsize"] = gridsize
        t7 = engine.generate_grid(patch)
        S = _scalar(src7, s2, src_grid, t7, k, eps=10.0)
        if n == 0:
            norm = np.max(np.absolute(S))
        p = np.sum(np.absolute(S / norm) ** 2 * t7[6])
        powers.append(p)
        diff = np.absolute(p0 - p)
        p0 = p
        n += 1
        if n >= max_iter:
            raise RuntimeError("no converged grid size")
    return (gridsize / patch_size).astype(int), powers


def converge_on_target(src7, src_grid, fields, scatterer, target, k, tol=1e-2, target_gridsize=None, mult=2,
                       div=3, max_iter=16):
    from pypo_gb300 import engine
    gm_t = int(target["gmode"])
    tgt = dict(target, gridsize=np.asarray(target_gridsize) if target_gridsize is not None
               else (np.array((3, 6)) if gm_t == 1 else np.array((5, 5))))
    scat = dict(scatterer, gridsize=np.array((10, 30)) if gm_t == 1 else np.array((10, 10)))
    s2 = strongest(fields)
    t7 = engine.generate_grid(tgt)
    trials = []

    def run():
        g = scat["gridsize"]
        s7 = engine.generate_grid(scat)
        on_scat = _scalar(src7, s2, src_grid, s7, k)
        return _scalar(s7, np.stack([on_scat.real, on_scat.imag]), (int(scat["gmode"]), int(g[0]), int(g[1])),
                       t7, k)

    init_field = run()
    conv_grid = np.array([10, 10])
    for i in range(2):
        field = init_field.copy()
        n, diff = 0, 1e99
        scat["gridsize"] = np.array([10, 10])
        while np.absolute(diff) > tol:
            last_field = field.copy()
            gridsize = scat["gridsize"][i] * mult
            scat["gridsize"][i] = gridsize
            field = run()
            diff = np.max(np.abs(np.abs(field - last_field))) / np.max(np.abs(field))
            trials.append((i, int(gridsize), float(diff)))
            n += 1
            if n >= max_iter:
                break
        if n >= max_iter:
            conv_grid[i] = gridsize
            break
        conv_gridsize, nonconv_gridsize = gridsize, gridsize / mult
        conv_field = last_field.copy()
        d = 0
        while d < div:
            next_grid = int((conv_gridsize + nonconv_gridsize) / 2)
            scat["gridsize"][i] = next_grid
            field = run()
            diff = np.max(np.abs(np.abs(field - conv_field))) / np.max(np.abs(field))
            trials.append((i, next_grid, float(diff)))
            if diff < tol:
                conv_gridsize, conv_field = next_grid, field.copy()
            else:
                nonconv_gridsize = next_grid
            d += 1
        conv_grid[i] = conv_gridsize
    return conv_grid, trials
