"""Drop-in for PyPO's GPU physical-optics binding (reference src/PyPO/BindGPU.py).

`loadGPUlib()` returns libpo_gb300 with the reference's `callKernelf_*`
argtypes, and `PyPO_GPUf(source, target, runPODict)` has the reference's
arguments and return values (reference BindGPU.py:83-224):

  mode   JM -> currents     EH, FF -> fields     JMEH -> [currents, fields]
         EHP -> [fields, rfield]                 scalar -> scalarfield

Differences, all on the side of the reference's FP64 CPU path:
  * structs point straight into numpy buffers (no `.tolist()` copies);
  * grids are generated in FP64 inside the call and results follow the CPU
    path's conventions (see include/po_gb300.h);
  * a failing call raises POError instead of ending the process.

`PyPO_GPUd` is the same call through the double-precision explicit-grid
entry (po_run_d): grids are generated in FP64 on the host and never rounded
to float, so large reflectors keep their phase. runPODict["precision"]
= "fp64" selects the plain FP64 GPU sum.
"""
import ctypes

import numpy as np

from . import PyPOTypes as PTypes
from . import Structs as S
from . import marshal as M
from ._lib import POError, check, load
from .checks import check_runPODict_gpu
from . import engine


def loadGPUlib():
    """The libpo_gb300 handle (reference BindGPU.py:18-81 loads libpypogpu)."""
    return load()


def _t_direction(runPODict):
    return -1.0 if runPODict.get("exp", "fwd") == "fwd" else 1.0


def _source_values(runPODict, gs, ctype=ctypes.c_double):
    if runPODict["mode"] == "scalar":
        sf = runPODict["s_scalarfield"]
        S_ = np.asarray(sf.S).ravel()
        return np.stack([S_.real, S_.imag]).astype(M._NP[ctype])
    return M.currents_block([runPODict["s_current"][i] for i in range(6)], ctype)


def _unpack(mode, block, shape):
    cplx = lambda rows: [r.reshape(shape) for r in rows]
    if mode == "scalar":
        return PTypes.scalarfield((block[0] + 1j * block[1]).reshape(shape))
    if mode in ("JM", "EH", "FF"):
        c = cplx(M.block_to_complex(block, 2))
        return PTypes.currents(*c) if mode == "JM" else PTypes.fields(*c)
    if mode == "JMEH":
        c = cplx(M.block_to_complex(block, 4))
        return [PTypes.currents(*c[:6]), PTypes.fields(*c[6:])]
    c = cplx(M.block_to_complex(block[:12], 2))
    pr = [block[12 + i].astype(np.float64).reshape(shape) for i in range(3)]
    return [PTypes.fields(*c), PTypes.rfield(*pr)]


def PyPO_GPUf(source, target, runPODict):
    """PO propagation through the float drop-in ABI (callKernelf_*)."""
    check_runPODict_gpu(runPODict)
    if runPODict.get("precision", "mixed") == "fp64":
        return PyPO_GPUd(source, target, runPODict)
    lib = load()
    mode = runPODict["mode"]
    f = ctypes.c_float
    csp, k1 = M.fill_reflparams(source, f)
    ctp, k2 = M.fill_reflparams(target, f)
    gs = int(np.prod(source["gridsize"]))
    gt = int(np.prod(target["gridsize"]))
    cs, _sblock = M.alloc_container(gs, f)
    ct, _tblock = M.alloc_container(gt, f)
    vals = _source_values(runPODict, gs, f)
    in_cls = S.arrC1f if mode == "scalar" else S.c2Bundlef
    cin = M.bundle(in_cls, vals, f)
    out = np.zeros((S.N_OUT[mode], gt), dtype=np.float32)
    res = M.bundle(S.BUNDLE_F[mode], out, f)
    fn = getattr(lib, f"callKernelf_{mode}")
    nThreads = int(runPODict.get("nThreads", 256))
    nBlocks = (gt + nThreads - 1) // nThreads
    check(fn(ctypes.byref(res), csp, ctp, ctypes.byref(cs), ctypes.byref(ct), ctypes.byref(cin),
             f(runPODict["k"]), f(runPODict["epsilon"]), f(_t_direction(runPODict)), nBlocks, nThreads))
    shape = (int(target["gridsize"][0]), int(target["gridsize"][1]))
    return _unpack(mode, out, shape)


def PyPO_GPUd(source, target, runPODict):
    """PO propagation through the FP64-input explicit-grid entry (po_run_d)."""
    check_runPODict_gpu(runPODict)
    mode = runPODict["mode"]
    s7 = engine.generate_grid(source)
    t7 = engine.generate_grid(target)
    gs = s7.shape[1]
    vals = _source_values(runPODict, gs)
    out = engine.propagate(mode, s7, vals, int(source["gmode"]), int(source["gridsize"][0]),
                           int(source["gridsize"][1]), t7, runPODict["k"], runPODict["epsilon"],
                           _t_direction(runPODict), runPODict.get("precision", "mixed"))
    shape = (int(target["gridsize"][0]), int(target["gridsize"][1]))
    return _unpack(mode, out, shape)
