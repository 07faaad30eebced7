"""Grid-size convergence searches, kept on the device.

Mirrors System.autoConverge and System.convergeOnTarget (reference
src/PyPO/System.py:2779-2880, :2882-3086): each repeats scalar runPO
propagations on growing grids until a measure stops changing. Here every
propagation runs on the GPU (po_run_dev, scalar mode), every trial grid is
generated there (po_generate_grid_dev), the power sum of auto_converge is a
device reduction (po_efficiency_sums_dev), and only a few scalars per trial
come back to the host.

Kept from the reference, with their effects:
  * the scalar source is the source's strongest component: the one of its six
    (Ex ... Hz, or Jx ... Mz) whose largest magnitude is largest, first on
    ties;
  * auto_converge grows both axes from 1 by `add` per trial, starting at
    1 + add, on the target scaled by patch_size (its xy or uv limits); an AoE
    target has no limits it scales (the reference fails there); the power is
    sum |S / norm|^2 dA with norm = max |S| of the first trial; it stops when
    two successive powers differ by at most tol and returns the grid size
    divided by patch_size, truncated to integers;
  * converge_on_target uses a 3 x 6 (uv) or 5 x 5 test grid on the target
    and starts the scatterer at 10 x 30 for a uv target (10 x 10 otherwise;
    the choice follows the target's grid mode), then per axis from 10 x 10:
    multiplies that axis by mult until the largest change of the target
    field, over its largest magnitude, is at most tol, then bisects `div`
    times between the last unconverged and the converged size, each time
    against the field of the last size that passed (at first the field before
    the final growth step). An axis that does not converge in max_iter steps
    keeps its last size and ends the search (the reference logs it).
"""
import ctypes

import numpy as np

from ._lib import POError, check, load
from . import engine

_LIMS = {0: ("lims_x", "lims_y"), 1: ("lims_u", "lims_v")}


def _stream(t):
    import torch
    return torch.cuda.current_stream(t.device)


def strongest_component(g7, block):
    """Row index (0-5: Ex Ey Ez Hx Hy Hz, or Jx ... Mz) of the component of a
    (12, n) device block on grid g7 whose largest magnitude is largest (first
    on ties)."""
    import torch
    n = block.shape[1]
    best, best_c = -1.0, 0
    sums = torch.empty(10, dtype=torch.float64, device=block.device)
    st = ctypes.c_void_p(_stream(block).cuda_stream)
    lib = load()
    for c in range(6):
        r = c if c < 3 else c + 3
        check(lib.po_efficiency_sums_dev(n, ctypes.c_void_p(g7.data_ptr()), ctypes.c_void_p(block[r].data_ptr()),
                                         ctypes.c_void_p(block[r + 3].data_ptr()), None, None, 0, None,
                                         ctypes.c_void_p(sums.data_ptr()), st))
        m = float(sums[7].item())
        if m > best:
            best, best_c = m, c
    return best_c


def scalar_source(g7, block):
    """The scalar field a search propagates: a (2, n) (re, im) scalar field as
    given, or the strongest component of a (12, n) fields or currents block."""
    import torch
    if block.shape[0] == 2:
        return block.contiguous()
    c = strongest_component(g7, block)
    r = c if c < 3 else c + 3
    return torch.stack([block[r], block[r + 3]]).contiguous()


def _power_and_peak(g7, s2):
    """sum |S|^2 dA and max |S|^2 over a device grid (one reduction)."""
    import torch
    n = g7.shape[1]
    sums = torch.empty(10, dtype=torch.float64, device=g7.device)
    check(load().po_efficiency_sums_dev(n, ctypes.c_void_p(g7.data_ptr()), ctypes.c_void_p(s2[0].data_ptr()),
                                        ctypes.c_void_p(s2[1].data_ptr()), None, None, 0, None,
                                        ctypes.c_void_p(sums.data_ptr()), ctypes.c_void_p(_stream(g7).cuda_stream)))
    s = sums.cpu().numpy()
    return float(s[0]), float(s[7])


def _grid(refl, dev):
    return engine.generate_grid_dev(refl, device=dev)


def auto_converge(src7, src_grid, fields, target, k, tol=1e-2, add=10, patch_size=1 / 9, max_iter=1000,
                  precision="mixed", full_output=False):
    """System.autoConverge: the target grid size at which a scalar propagation
    of the source's strongest component converges in power on a central patch.

    src7: (7, ns) device grid of the source; src_grid: (gmode, ncx, ncy) of it;
    fields: (12, ns) device block (E then H, c2Bundle rows) or a (2, ns)
    scalar field; target: reflector
    dict. Returns the grid size (np.int64 array of 2), and with full_output also
    the powers of the trials."""
    gmode = int(target["gmode"])
    if gmode not in _LIMS:
        raise POError("auto_converge: an AoE target has no xy or uv limits to scale "
                      "(the reference fails here)")
    kx, ky = _LIMS[gmode]
    patch = dict(target)
    patch[kx] = patch_size * np.asarray(target[kx], float)
    patch[ky] = patch_size * np.asarray(target[ky], float)
    s2 = scalar_source(src7, fields)
    gridsize = np.array([1, 1])
    p_prev, diff, norm2, n = 1e99, 1e99, 1.0, 0
    powers = []
    while abs(diff) > tol:
        gridsize = gridsize + add
        patch["gridsize"] = gridsize
        t7 = _grid(patch, src7.device)
        out = engine.propagate_dev("scalar", src7, s2, *src_grid, t7, k, epsilon=10.0, t_dir=-1.0,
                                   precision=precision)
        p, peak2 = _power_and_peak(t7, out)
        if n == 0:
            norm2 = peak2
        p = p / norm2
        powers.append(p)
        diff = abs(p_prev - p)
        p_prev = p
        n += 1
        if n >= max_iter:
            raise POError(f"auto_converge: no converged grid size within {max_iter} trials "
                          f"(last difference {diff:.3e})")
    result = (gridsize / patch_size).astype(int)
    return (result, powers) if full_output else result


def converge_on_target(src7, src_grid, fields, scatterer, target, k, tol=1e-2, target_gridsize=None, mult=2,
                       div=3, max_iter=16, precision="mixed", full_output=False):
    """System.convergeOnTarget: the scatterer's grid size at which the field
    it scatters onto a few target points converges, axis by axis.

    src7, src_grid, fields: the source (device grid, its (gmode, ncx, ncy),
    (12, ns) fields or currents); scatterer, target: reflector dicts. Returns
    the grid size (np array of 2), and with full_output also the trials'
    (axis, grid size, difference)."""
    gm_t = int(target["gmode"])
    tgt = dict(target)
    if target_gridsize is not None and len(target_gridsize):
        tgt["gridsize"] = np.asarray(target_gridsize)
    else:
        tgt["gridsize"] = np.array((3, 6)) if gm_t == 1 else np.array((5, 5))
    scat = dict(scatterer)
    scat["gridsize"] = np.array((10, 30)) if gm_t == 1 else np.array((10, 10))
    dev = src7.device
    s2 = scalar_source(src7, fields)
    t7 = _grid(tgt, dev)
    trials = []

    def target_field():
        g = np.asarray(scat["gridsize"])
        s7 = _grid(scat, dev)
        on_scat = engine.propagate_dev("scalar", src7, s2, *src_grid, s7, k, precision=precision)
        on_tgt = engine.propagate_dev("scalar", s7, on_scat, int(scat["gmode"]), int(g[0]), int(g[1]), t7, k,
                                      precision=precision)
        a = on_tgt.cpu().numpy()
        return a[0] + 1j * a[1]

    def change(f, ref):
        return float(np.max(np.abs(np.abs(f - ref))) / np.max(np.abs(f)))

    init_field = target_field()
    conv_grid = np.array([10, 10])
    for i in range(2):
        field = init_field.copy()
        n, diff = 0, 1e99
        scat["gridsize"] = np.array([10, 10])
        while abs(diff) > tol:
            last_field = field.copy()
            gridsize = int(scat["gridsize"][i] * mult)
            scat["gridsize"][i] = gridsize
            field = target_field()
            diff = change(field, last_field)
            trials.append((i, gridsize, diff))
            n += 1
            if n >= max_iter:
                break
        if n >= max_iter:
            conv_grid[i] = gridsize
            break
        conv_gridsize, nonconv_gridsize = gridsize, gridsize / mult
        conv_field = last_field.copy()
        for _ in range(div):
            next_grid = int((conv_gridsize + nonconv_gridsize) / 2)
            scat["gridsize"][i] = next_grid
            field = target_field()
            diff = change(field, conv_field)
            trials.append((i, next_grid, diff))
            if diff < tol:
                conv_gridsize, conv_field = next_grid, field.copy()
            else:
                nonconv_gridsize = next_grid
        conv_grid[i] = conv_gridsize
    return (conv_grid, trials) if full_output else conv_grid
