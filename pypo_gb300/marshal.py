"""Zero-copy marshalling between numpy arrays and the PO C-ABI structs.

The reference fills its ctypes structs through `.tolist()` copies
(reference src/PyPO/BindUtils.py:277-455), which costs seconds at 1e6
points. Here every struct member points straight into a contiguous numpy
buffer; the returned `keep` list holds those buffers alive for the call.
"""
import ctypes

import numpy as np

from . import Structs as S

_NP = {ctypes.c_float: np.float32, ctypes.c_double: np.float64}


def _ptr(arr, ctype):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


def as_c(arr, ctype):
    """Contiguous copy (only when needed) of `arr` in the numpy type of `ctype`."""
    return np.ascontiguousarray(np.asarray(arr).ravel(), dtype=_NP[ctype])


def fill_reflparams(refl, ctype=ctypes.c_double):
    """Build a reflparams / reflparamsf from a reflector dict.

    Keys follow the reference's reflDict as read by
    reference src/PyPO/BindUtils.py:277-327 (allfill_reflparams).
    """
    st = S.reflparams() if ctype is ctypes.c_double else S.reflparamsf()
    keep = []
    gmode = int(refl["gmode"])
    lim_keys = {0: ("lims_x", "lims_y"), 1: ("lims_u", "lims_v"), 2: ("lims_Az", "lims_El")}[gmode]
    coeffs = as_c(refl.get("coeffs", np.zeros(3)), ctype)
    lxu = as_c(refl[lim_keys[0]], ctype)
    lyv = as_c(refl[lim_keys[1]], ctype)
    gcenter = as_c(refl.get("gcenter", np.zeros(2)), ctype)
    ncells = np.ascontiguousarray(np.asarray(refl["gridsize"]).ravel(), dtype=np.int32)
    transf = as_c(np.asarray(refl.get("transf", np.eye(4)), dtype=np.float64).ravel(), ctype)
    keep += [coeffs, lxu, lyv, gcenter, ncells, transf]
    st.coeffs = _ptr(coeffs, ctype)
    st.lxu = _ptr(lxu, ctype)
    st.lyv = _ptr(lyv, ctype)
    st.gcenter = _ptr(gcenter, ctype)
    st.n_cells = ncells.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    st.transf = _ptr(transf, ctype)
    st.flip = bool(refl.get("flip", False))
    st.gmode = gmode
    st.ecc_uv = float(refl.get("ecc_uv", 0.0))
    st.rot_uv = float(refl.get("rot_uv", 0.0))
    st.type = int(refl["type"])
    st.rms = float(refl.get("rms", 0.0))
    st.rms_seed = int(refl.get("rms_seed", 0))
    return st, keep


def alloc_container(n, ctype=ctypes.c_double):
    """reflcontainer(f) whose 7 arrays are one (7, n) numpy block."""
    st = S.reflcontainer() if ctype is ctypes.c_double else S.reflcontainerf()
    block = np.zeros((7, n), dtype=_NP[ctype])
    st.size = n
    for i, name in enumerate(("x", "y", "z", "nx", "ny", "nz", "area")):
        setattr(st, name, _ptr(block[i], ctype))
    st._block = block
    return st, block


def fill_container(block, ctype=ctypes.c_double):
    """reflcontainer(f) pointing at an existing (7, n) block (x y z nx ny nz area)."""
    block = np.ascontiguousarray(block, dtype=_NP[ctype])
    st = S.reflcontainer() if ctype is ctypes.c_double else S.reflcontainerf()
    st.size = block.shape[1]
    for i, name in enumerate(("x", "y", "z", "nx", "ny", "nz", "area")):
        setattr(st, name, _ptr(block[i], ctype))
    st._block = block
    return st, block


def bundle(cls, block, ctype):
    """Point a bundle struct's members, in field order, at the rows of `block`.
    The struct holds a reference to `block`, so a temporary block stays
    alive as long as the struct does."""
    st = cls()
    names = [f[0] for f in cls._fields_]
    assert block.shape[0] == len(names)
    for i, name in enumerate(names):
        setattr(st, name, _ptr(block[i], ctype))
    st._block = block
    return st


def currents_block(cur, ctype=ctypes.c_double):
    """(12, n) block in c2Bundle order from a (6, ...) complex array-like
    (Jx..Mz), written straight into the ctype's precision."""
    c = [np.asarray(a).ravel() for a in cur]
    out = np.empty((12, c[0].size), dtype=_NP[ctype])
    for g in range(2):
        for a in range(3):
            z = c[3 * g + a]
            out[6 * g + a] = np.real(z)
            out[6 * g + 3 + a] = np.imag(z)
    return out


def block_to_complex(block, n_complex):
    """Rows in bundle order (r1x r1y r1z i1x i1y i1z ...) to (3*n_complex, n) complex."""
    out = []
    for b in range(n_complex):
        re = block[6 * b:6 * b + 3]
        im = block[6 * b + 3:6 * b + 6]
        z = np.empty(re.shape, dtype=np.complex128)
        z.real = re
        z.imag = im
        out.append(z)
    return np.concatenate(out, axis=0)
