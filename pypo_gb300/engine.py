"""Explicit-grid Python API over libpo_gb300.

`propagate` runs one physical-optics propagation on host numpy buffers
(po_run_d); `propagate_dev` on device buffers given as torch tensors
(po_run_dev, queued on the current torch stream); `generate_grid` is the FP64
grid generator (po_generate_grid).

Array layouts (all float64):
  src7 / tgt7 : (7, n) rows x y z nx ny nz area; row-major over the surface's
                (ncx, ncy) grid. For far-field targets x is the polar angle
                and y the azimuth in radians (the AoE grid's spheric form).
  cur         : (12, ns) rows in c2Bundle order r1x r1y r1z i1x i1y i1z r2x
                ... i2z (J then M), or (2, ns) (re, im) for scalar mode.
  result      : (n_out(mode), nt) rows in the mode's bundle order.
"""
import ctypes
import warnings

import numpy as np

from . import Structs as S
from . import marshal as M
from ._lib import MODE_ID, POError, check, load

PRECISION = {"mixed": 0, "fp64": 1}


def n_out(mode):
    return S.N_OUT[mode]


def generate_grid(refl, transform=True, spheric=True):
    """(7, n) float64 grid of a reflector dict (FP64 generator)."""
    lib = load()
    rp, keep = M.fill_reflparams(refl, ctypes.c_double)
    n = int(np.prod(refl["gridsize"]))
    ct, block = M.alloc_container(n, ctypes.c_double)
    check(lib.po_generate_grid(rp, ctypes.byref(ct), int(transform), int(spheric)))
    return block


def generate_grid_dev(refl, transform=True, spheric=True, device=None, stream=None):
    """(7, n) float64 CUDA tensor of a reflector dict, generated on the device
    (po_generate_grid_dev; the same FP64 formulas as generate_grid), queued
    on `stream` (default: torch's current stream)."""
    import torch
    lib = load()
    dev = torch.device("cuda") if device is None else torch.device(device)
    rp, keep = M.fill_reflparams(refl, ctypes.c_double)
    n = int(np.prod(refl["gridsize"]))
    out = torch.empty((7, n), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev) if stream is None else stream
    check(lib.po_generate_grid_dev(rp, ctypes.c_void_p(out.data_ptr()), int(transform), int(spheric),
                                   ctypes.c_void_p(st.cuda_stream)))
    return out


def correlated_error(g7, rms, corr_len, seed, n_modes=512, apply=False):
    """Correlated surface error at the points of a (7, n) host grid
    (po_correlated_error): covariance rms^2 exp(-r^2 / (2 corr_len^2)) over
    (x, y), spectral synthesis over n_modes modes from mt19937(seed). Returns
    delta (n,); with apply, g7 (C-contiguous float64) is also moved along
    its normals in place."""
    lib = load()
    if not (isinstance(g7, np.ndarray) and g7.dtype == np.float64 and g7.flags.c_contiguous and g7.shape[0] == 7):
        raise POError("g7 must be a C-contiguous (7, n) float64 array")
    n = g7.shape[1]
    delta = np.empty(n)
    check(lib.po_correlated_error(n, g7.ctypes.data, float(rms), float(corr_len), int(seed), int(n_modes),
                                  delta.ctypes.data, 1 if apply else 0))
    return delta


def correlated_error_dev(g7, rms, corr_len, seed, n_modes=512, apply=False, stream=None):
    """correlated_error on a (7, n) float64 CUDA tensor (po_correlated_error_dev),
    queued on `stream`; returns delta as a CUDA tensor."""
    import torch
    lib = load()
    if not (g7.is_cuda and g7.dtype == torch.float64 and g7.is_contiguous() and g7.shape[0] == 7):
        raise POError("g7 must be a contiguous (7, n) float64 CUDA tensor")
    n = g7.shape[1]
    delta = torch.empty(n, dtype=torch.float64, device=g7.device)
    st = torch.cuda.current_stream(g7.device) if stream is None else stream
    check(lib.po_correlated_error_dev(n, g7.data_ptr(), float(rms), float(corr_len), int(seed), int(n_modes),
                                      delta.data_ptr(), 1 if apply else 0, ctypes.c_void_p(st.cuda_stream)))
    return delta


def _shape_checks(mode, src7, cur, tgt7, gmode, ncx, ncy):
    if mode not in MODE_ID:
        raise POError(f"unknown mode {mode!r}; expected one of {tuple(MODE_ID)}")
    ns = src7.shape[1]
    if src7.shape[0] != 7 or tgt7.shape[0] != 7:
        raise POError("src7 and tgt7 must have 7 rows (x y z nx ny nz area)")
    want = 2 if mode == "scalar" else 12
    if cur.shape != (want, ns):
        raise POError(f"cur must have shape ({want}, {ns}) for mode {mode}")
    if gmode >= 0 and ncx * ncy != ns:
        raise POError("ncx * ncy must equal the number of source points")


#: frame half-extent, in wavelengths, up to which the mixed path was measured to
#: stay within its 1e-5 relative-L2 bar (the error grows linearly with it)
MIXED_EXTENT_LIMIT = 5.0e4


def mixed_extent(mode, src7, tgt7, k):
    """The frame half-extent in wavelengths that sets the mixed path's precision:
    positions are split into hi parts on a quantum ~ extent / 1024 and the lo
    parts' rounding grows with it. Near field and scalar: half the largest side
    of the bounding box of sources and targets (the frame is centred); far
    field: the largest source coordinate (the frame is the coordinate origin).
    A host computation for planning; the library reports the same value for
    each host-buffer call (last_extent)."""
    kappa = float(k) / (2 * np.pi)
    if src7.shape[1] == 0:
        return 0.0
    if mode == "FF":
        return float(np.abs(src7[0:3]).max()) * kappa
    pts = np.concatenate([src7[0:3], tgt7[0:3]], axis=1)
    return float((pts.max(axis=1) - pts.min(axis=1)).max()) * 0.5 * kappa


def last_extent():
    """Frame half-extent (wavelengths) of this thread's last mixed-precision
    host-buffer call, computed on the device (po_last_extent)."""
    return float(load().po_last_extent())


def last_band_pairs():
    """Near-tangent (source, target) pairs of this thread's last mixed-precision
    host-buffer call, decided and summed in FP64 (po_last_band_pairs)."""
    return int(load().po_last_band_pairs())


def _extent_warning(m, precision):
    """Warn when a mixed-precision call's frame half-extent m is beyond the
    measured range of the path."""
    if precision != "mixed":
        return
    if m > MIXED_EXTENT_LIMIT:
        warnings.warn(f"scene half-extent {m:.3g} wavelengths exceeds {MIXED_EXTENT_LIMIT:.3g}: the mixed path's "
                      "error grows with it (about 1e-5 relative at 1e5); use precision='fp64' for this call",
                      RuntimeWarning, stacklevel=3)


def propagate(mode, src7, cur, gmode, ncx, ncy, tgt7, k, epsilon=1.0, t_dir=-1.0, precision="mixed",
              out=None):
    """Host-buffer propagation; returns (n_out(mode), nt) float64 (into `out` when given)."""
    lib = load()
    src7 = np.ascontiguousarray(src7, dtype=np.float64)
    tgt7 = np.ascontiguousarray(tgt7, dtype=np.float64)
    cur = np.ascontiguousarray(cur, dtype=np.float64)
    _shape_checks(mode, src7, cur, tgt7, gmode, ncx, ncy)
    nt = tgt7.shape[1]
    if out is None:
        out = np.empty((n_out(mode), nt), dtype=np.float64)
    elif out.shape != (n_out(mode), nt) or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise POError(f"out must be a C-contiguous float64 array of shape {(n_out(mode), nt)}")
    check(lib.po_run_d(MODE_ID[mode], src7.shape[1], src7.ctypes.data, int(gmode), int(ncx), int(ncy),
                       cur.ctypes.data, nt, tgt7.ctypes.data, float(k), float(epsilon), float(t_dir),
                       PRECISION[precision], out.ctypes.data))
    _extent_warning(last_extent(), precision)
    return out


def propagate_dev(mode, src7, cur, gmode, ncx, ncy, tgt7, k, epsilon=1.0, t_dir=-1.0,
                  precision="mixed", m_zero=False, out=None, stream=None):
    """Device-buffer propagation on torch float64 CUDA tensors.

    Queued on `stream` (default: torch's current stream); returns `out`.
    """
    import torch
    lib = load()
    for name, t in (("src7", src7), ("cur", cur), ("tgt7", tgt7)):
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise POError(f"{name} must be a contiguous float64 CUDA tensor")
    _shape_checks(mode, src7, cur, tgt7, gmode, ncx, ncy)
    nt = tgt7.shape[1]
    if out is None:
        out = torch.empty((n_out(mode), nt), dtype=torch.float64, device=tgt7.device)
    if stream is None:
        stream = torch.cuda.current_stream(tgt7.device)
    check(lib.po_run_dev(MODE_ID[mode], src7.shape[1], src7.data_ptr(), int(gmode), int(ncx), int(ncy),
                         cur.data_ptr(), nt, tgt7.data_ptr(), float(k), float(epsilon), float(t_dir),
                         PRECISION[precision], 1 if m_zero else 0, out.data_ptr(), ctypes.c_void_p(stream.cuda_stream)))
    return out


def device_error(stream=None):
    """Synchronise `stream` and return the device error word (0 = fine)."""
    lib = load()
    code = ctypes.c_int(0)
    ptr = None
    if stream is not None:
        ptr = ctypes.c_void_p(stream.cuda_stream)
    check(lib.po_device_error(ptr, ctypes.byref(code)))
    return code.value


def last_launches():
    return load().po_last_launches()


def timing_enable(slots):
    check(load().po_timing_enable(int(slots)))


def timing_collect(max_n=4096):
    buf = (ctypes.c_float * max_n)()
    n = load().po_timing_collect(buf, max_n)
    if n < 0:
        raise POError("po_timing_collect failed")
    return [buf[i] for i in range(n)]


def adjoint(mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon=1.0, t_dir=-1.0, precision="mixed",
            want=("cur", "ds", "dt"), out=None):
    """Host-buffer adjoint (po_adjoint_d).

    cot: (n_out(mode), nt) float64, dL/d(output rows). Returns a dict with the
    requested gradients: "cur" (the shape of cur: 12 or, scalar, 2 rows), "ds"
    (ns,) and "dt" (nt,) (near field and scalar),
    written into the arrays of `out` (a dict of C-contiguous float64 arrays of
    those shapes, e.g. page-locked ones) where it has them.
    """
    lib = load()
    src7 = np.ascontiguousarray(src7, dtype=np.float64)
    tgt7 = np.ascontiguousarray(tgt7, dtype=np.float64)
    cur = np.ascontiguousarray(cur, dtype=np.float64)
    cot = np.ascontiguousarray(cot, dtype=np.float64)
    _shape_checks(mode, src7, cur, tgt7, gmode, ncx, ncy)
    ns, nt = src7.shape[1], tgt7.shape[1]
    if cot.shape != (n_out(mode), nt):
        raise POError(f"cot must have shape {(n_out(mode), nt)}")
    given = out or {}

    def buf(name, shape):
        a = given.get(name)
        if a is None:
            return np.zeros(shape)
        if a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise POError(f"out[{name!r}] must be a C-contiguous float64 array of shape {shape}")
        return a

    out = {}
    gc = buf("cur", cur.shape) if "cur" in want else None
    gs = buf("ds", (ns,)) if "ds" in want else None
    gt = buf("dt", (nt,)) if ("dt" in want and mode != "FF") else None
    ptr = lambda a: a.ctypes.data if a is not None else None
    check(lib.po_adjoint_d(MODE_ID[mode], ns, src7.ctypes.data, int(gmode), int(ncx), int(ncy), cur.ctypes.data,
                           nt, tgt7.ctypes.data, float(k), float(epsilon), float(t_dir), PRECISION[precision],
                           cot.ctypes.data, ptr(gc), ptr(gs), ptr(gt)))
    _extent_warning(last_extent(), precision)
    if gc is not None:
        out["cur"] = gc
    if gs is not None:
        out["ds"] = gs
    if gt is not None:
        out["dt"] = gt
    return out


def adjoint_dev(mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon=1.0, t_dir=-1.0, precision="mixed",
                m_zero=False, grad_cur=None, grad_ds=None, grad_dt=None, stream=None):
    """Device-buffer adjoint (po_adjoint_dev) on torch float64 CUDA tensors; queued on `stream`."""
    import torch
    lib = load()
    for name, t in (("src7", src7), ("cur", cur), ("tgt7", tgt7), ("cot", cot)):
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise POError(f"{name} must be a contiguous float64 CUDA tensor")
    _shape_checks(mode, src7, cur, tgt7, gmode, ncx, ncy)
    if stream is None:
        stream = torch.cuda.current_stream(tgt7.device)
    ptr = lambda t: t.data_ptr() if t is not None else None
    check(lib.po_adjoint_dev(MODE_ID[mode], src7.shape[1], src7.data_ptr(), int(gmode), int(ncx), int(ncy),
                             cur.data_ptr(), tgt7.shape[1], tgt7.data_ptr(), float(k), float(epsilon), float(t_dir),
                             PRECISION[precision], 1 if m_zero else 0, cot.data_ptr(), ptr(grad_cur), ptr(grad_ds),
                             ptr(grad_dt), ctypes.c_void_p(stream.cuda_stream)))
    return grad_cur, grad_ds, grad_dt
