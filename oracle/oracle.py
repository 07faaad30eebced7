"""TEST INFRASTRUCTURE ONLY: Python handle on the FP64 oracle.

Two checkers live here:

* `run(...)` calls oracle/libpo_oracle.so, the plain-C restatement of the
  reference's CPU integrator (oracle/po_oracle.c). It is built on every
  machine by `__graft_entry__.build()`.
* `Reference` calls oracle/_ref/libpypo_ref.so, the reference's own CPU
  library compiled from its sources by oracle/build_ref.sh. It exists only
  where the reference sources exist; it pins `run` (tests/golden).

Only tests/, `__graft_entry__.smoke()` and bench.py's cpu_baseline /
reference legs import this module. The product (pypo_gb300) never does.
"""
import ctypes
import os
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libpo_oracle.so"
REF_PATH = HERE / "_ref" / "libpypo_ref.so"
MODES = {"JM": 0, "EH": 1, "JMEH": 2, "EHP": 3, "FF": 4, "scalar": 5}
N_OUT = {"JM": 12, "EH": 12, "JMEH": 24, "EHP": 15, "FF": 12, "scalar": 2}

_lib = None


def build(quiet=True):
    """Compile oracle/po_oracle.c with gcc (plain C, no arch flags; -O3 as
    oracle/build_ref.sh builds the reference's own library, and no FP
    contraction, so the sums are the reference's to the bit)."""
    import subprocess
    src = HERE / "po_oracle.c"
    tmp = str(LIB_PATH) + ".tmp"
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-std=c11", "-shared", "-fPIC", "-pthread", str(src), "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        lib = ctypes.CDLL(str(LIB_PATH))
        lib.po_oracle_run.restype = ctypes.c_int
        lib.po_oracle_run.argtypes = [
            ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
        lib.po_oracle_adjoint.restype = ctypes.c_int
        lib.po_oracle_adjoint.argtypes = [
            ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = lib
    return _lib


def run(mode, src7, cur, gmode, ncx, ncy, tgt7, k, epsilon=1.0, t_dir=-1.0,
        nthreads=None, tidx=None):
    """FP64 oracle propagation on explicit grids.

    src7, tgt7: (7, n) float64 rows x y z nx ny nz area (for FF the target's
    x is the polar angle and y the azimuth). cur: (12, ns) rows in c2Bundle
    order, or (2, ns) (re, im) for scalar mode. Returns (N_OUT[mode], npts).
    """
    lib = load()
    src7 = np.ascontiguousarray(src7, dtype=np.float64)
    tgt7 = np.ascontiguousarray(tgt7, dtype=np.float64)
    cur = np.ascontiguousarray(cur, dtype=np.float64)
    ns, nt = src7.shape[1], tgt7.shape[1]
    if tidx is not None:
        tidx = np.ascontiguousarray(tidx, dtype=np.int64)
        npts = tidx.size
    else:
        npts = nt
    out = np.zeros((N_OUT[mode], npts), dtype=np.float64)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = lib.po_oracle_run(MODES[mode], ns, src7.ctypes.data, cur.ctypes.data,
                           int(gmode), int(ncx), int(ncy), nt, tgt7.ctypes.data,
                           tidx.ctypes.data if tidx is not None else None, npts,
                           float(k), float(epsilon), float(t_dir), int(nthreads),
                           out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"po_oracle_run failed with status {rc}")
    return out


def adjoint(mode, src7, cur, gmode, ncx, ncy, tgt7, k, cot, epsilon=1.0, t_dir=-1.0,
            nthreads=None, want=("cur", "ds", "dt")):
    """FP64 vector-Jacobian product of `run` (po_oracle_adjoint): gradients of
    L = sum(cot * run(...)) with respect to the currents ("cur", the shape of
    cur), the normal displacement of every source ("ds", (ns,)) and, near
    field and scalar, of every target ("dt", (nt,)). Modes JM, EH, JMEH, FF,
    scalar."""
    lib = load()
    src7 = np.ascontiguousarray(src7, dtype=np.float64)
    tgt7 = np.ascontiguousarray(tgt7, dtype=np.float64)
    cur = np.ascontiguousarray(cur, dtype=np.float64)
    cot = np.ascontiguousarray(cot, dtype=np.float64)
    ns, nt = src7.shape[1], tgt7.shape[1]
    if cot.shape != (N_OUT[mode], nt):
        raise ValueError(f"cot must have shape {(N_OUT[mode], nt)}")
    gc = np.zeros(cur.shape) if "cur" in want else None
    gs = np.zeros(ns) if "ds" in want else None
    gt = np.zeros(nt) if ("dt" in want and mode != "FF") else None
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    ptr = lambda a: a.ctypes.data if a is not None else None
    rc = lib.po_oracle_adjoint(MODES[mode], ns, src7.ctypes.data, cur.ctypes.data, int(gmode), int(ncx), int(ncy),
                               nt, tgt7.ctypes.data, cot.ctypes.data, float(k), float(epsilon), float(t_dir),
                               int(nthreads), ptr(gc), ptr(gs), ptr(gt))
    if rc != 0:
        raise RuntimeError(f"po_oracle_adjoint failed with status {rc}")
    return {name: a for name, a in (("cur", gc), ("ds", gs), ("dt", gt)) if a is not None}


class Reference:
    """The reference's own CPU library (FP64), compiled from its sources."""

    def __init__(self, path=REF_PATH):
        import sys
        sys.path.insert(0, str(HERE.parent))
        from pypo_gb300 import Structs as S
        self.S = S
        if not pathlib.Path(path).exists():
            raise FileNotFoundError(f"{path} missing: run oracle/build_ref.sh")
        lib = ctypes.CDLL(str(path))
        P = ctypes.POINTER
        common = [S.reflparams, S.reflparams, P(S.reflcontainer), P(S.reflcontainer)]
        for name, res_t in (("propagateToGrid_JM", S.c2Bundle), ("propagateToGrid_EH", S.c2Bundle),
                            ("propagateToGrid_JMEH", S.c4Bundle), ("propagateToGrid_EHP", S.c2rBundle),
                            ("propagateToFarField", S.c2Bundle)):
            fn = getattr(lib, name)
            fn.argtypes = [P(res_t)] + common + [P(S.c2Bundle), ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_double]
            fn.restype = None
        lib.propagateToGrid_scalar.argtypes = [P(S.arrC1)] + common + [
            P(S.arrC1), ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        lib.propagateToGrid_scalar.restype = None
        lib.generateGrid.argtypes = [S.reflparams, P(S.reflcontainer), ctypes.c_bool, ctypes.c_bool]
        lib.generateGrid.restype = None
        lib.makeGaussBeam.argtypes = [S.vecGPODict, S.reflparams, P(S.c2Bundle), P(S.c2Bundle)]
        lib.makeGaussBeam.restype = None
        lib.calcCurrents.argtypes = [P(S.c2Bundle), P(S.c2Bundle), S.reflparams, ctypes.c_int]
        lib.calcCurrents.restype = None
        self.lib = lib

    def grid(self, refl, transform=True, spheric=True):
        from pypo_gb300 import marshal as M
        rp, keep = M.fill_reflparams(refl, ctypes.c_double)
        n = int(np.prod(refl["gridsize"]))
        ct, block = M.alloc_container(n, ctypes.c_double)
        self.lib.generateGrid(rp, ctypes.byref(ct), transform, spheric)
        return block

    def propagate(self, mode, source, target, cur, k, epsilon=1.0, t_dir=-1.0, nthreads=None):
        """Reference CPU runPO kernel; returns (out rows, source grid, target grid)."""
        from pypo_gb300 import marshal as M
        S = self.S
        if nthreads is None:
            nthreads = os.cpu_count() or 1
        sp, k1 = M.fill_reflparams(source, ctypes.c_double)
        tp, k2 = M.fill_reflparams(target, ctypes.c_double)
        ns = int(np.prod(source["gridsize"]))
        nt = int(np.prod(target["gridsize"]))
        cs, sblock = M.alloc_container(ns, ctypes.c_double)
        ct, tblock = M.alloc_container(nt, ctypes.c_double)
        cur = np.ascontiguousarray(cur, dtype=np.float64)
        out = np.zeros((N_OUT[mode], nt), dtype=np.float64)
        if mode == "scalar":
            cin = M.bundle(S.arrC1, cur, ctypes.c_double)
            res = M.bundle(S.arrC1, out, ctypes.c_double)
            fn = self.lib.propagateToGrid_scalar
        else:
            cin = M.bundle(S.c2Bundle, cur, ctypes.c_double)
            cls = {"JMEH": S.c4Bundle, "EHP": S.c2rBundle}.get(mode, S.c2Bundle)
            res = M.bundle(cls, out, ctypes.c_double)
            fn = {"JM": self.lib.propagateToGrid_JM, "EH": self.lib.propagateToGrid_EH,
                  "JMEH": self.lib.propagateToGrid_JMEH, "EHP": self.lib.propagateToGrid_EHP,
                  "FF": self.lib.propagateToFarField}[mode]
        fn(ctypes.byref(res), sp, tp, ctypes.byref(cs), ctypes.byref(ct), ctypes.byref(cin),
           float(k), int(nthreads), float(epsilon), float(t_dir))
        return out, sblock, tblock

    def gauss_beam(self, lam, w0, z, power, plane, n=1.0, mode=0):
        """Reference makeGaussBeam: returns (fields (12, n), currents (12, n))."""
        from pypo_gb300 import marshal as M
        S = self.S
        g = S.vecGPODict(lam=lam, w0=w0, z=z, n=n, power=power, mode=mode)
        rp, keep = M.fill_reflparams(plane, ctypes.c_double)
        npts = int(np.prod(plane["gridsize"]))
        f = np.zeros((12, npts))
        c = np.zeros((12, npts))
        self.lib.makeGaussBeam(g, rp, ctypes.byref(M.bundle(S.c2Bundle, f, ctypes.c_double)),
                               ctypes.byref(M.bundle(S.c2Bundle, c, ctypes.c_double)))
        return f, c

    def calc_currents(self, fields, surface, mode):
        """Reference calcCurrents (BeamInit.h:660-843, calcJM): equivalent
        currents (12, n) of fields (12, n) on the surface's grid."""
        from pypo_gb300 import marshal as M
        S = self.S
        rp, keep = M.fill_reflparams(surface, ctypes.c_double)
        f = np.ascontiguousarray(fields, dtype=np.float64)
        c = np.zeros_like(f)
        self.lib.calcCurrents(ctypes.byref(M.bundle(S.c2Bundle, f, ctypes.c_double)),
                              ctypes.byref(M.bundle(S.c2Bundle, c, ctypes.c_double)), rp, int(mode))
        return c
