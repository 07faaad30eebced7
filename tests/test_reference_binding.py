"""The drop-in claim, checked with the reference's own Python binding.

PyPO's GPU path loads its CUDA library in BindGPU.loadGPUlib
(src/PyPO/BindGPU.py:18-81) and binds every entry point's argtypes there,
with the struct layouts of src/PyPO/Structs.py. Here the reference's own
modules are imported from its checkout, loadGPUlib is pointed at
libpo_gb300.so (only the library name changes), and:
  * every argtypes assignment of the unmodified loader binds, including the
    ray tracer's callRTKernel, which this library refuses with a status;
  * every ctypes struct of the reference's Structs.py has the field names,
    offsets and size of the C structs in include/po_gb300.h;
  * for every mode, the reference's own PyPO_GPUf and pypo_gb300's hand a
    recording stand-in library the same arguments (entry point, reflparamsf
    values, container sizes, source arrays, k, epsilon, direction) and turn
    the same result bundle into the same objects. With the GPU tests of
    pypo_gb300's PyPO_GPUf against the reference's outputs, this carries the
    parity to calls made by the reference's unmodified binding.
Runs on CPU (binding only, no kernel launch); skipped where the reference's
sources are absent.
"""
import ctypes
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "po_gb300.h"


def _reference_root():
    r = subprocess.run([str(ROOT / "oracle" / "build_ref.sh"), "--where"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("the reference's sources are not on this machine")
    return pathlib.Path(r.stdout.strip())


@pytest.fixture(scope="module")
def ref_pypo():
    src = _reference_root() / "src"
    sys.path.insert(0, str(src))
    try:
        import PyPO.BindGPU as BindGPU
        import PyPO.Structs as Structs
    finally:
        sys.path.remove(str(src))
    return BindGPU, Structs


def test_reference_loader_binds_libpo_gb300(lib, ref_pypo, monkeypatch):
    BindGPU, _ = ref_pypo
    ours = str(ROOT / "pypo_gb300" / "libpo_gb300.so")
    real_cdll = ctypes.CDLL
    opened = []

    def cdll(name, *a, **kw):   # the loader's one change: the library it opens
        if "pypogpu" in pathlib.Path(str(name)).name:
            name = ours
        opened.append(str(name))
        return real_cdll(name, *a, **kw)

    monkeypatch.setattr(ctypes, "CDLL", cdll)
    rlib = BindGPU.loadGPUlib()
    assert opened and opened[0] == ours
    for name in ("callKernelf_JM", "callKernelf_EH", "callKernelf_JMEH", "callKernelf_EHP", "callKernelf_FF",
                 "callKernelf_scalar", "callRTKernel"):
        fn = getattr(rlib, name)
        assert fn.argtypes and len(fn.argtypes) in (7, 11), name
        assert fn.restype is None   # as the reference binds them: the status is ignored
    # the ray tracer is not served: no frame is touched, the status says why
    S = ref_pypo[1]
    fr = S.cframef()
    rlib.callRTKernel(S.reflparamsf(), ctypes.byref(fr), ctypes.byref(fr), 1.0, 0.0, 1, 1)
    assert b"ray tracer is not part of libpo_gb300" in lib.po_last_error()


STRUCTS = ["reflparams", "reflparamsf", "reflcontainer", "reflcontainerf", "c2Bundle", "c2Bundlef", "c4Bundlef",
           "c2rBundlef", "arrC1", "arrC1f", "cframef"]


def test_reference_structs_match_the_header(ref_pypo, tmp_path):
    _, S = ref_pypo
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    for cname in STRUCTS:
        cls = getattr(S, cname)
        lines.append(f'printf("{cname} __sizeof__ %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln}
    for cname in STRUCTS:
        cls = getattr(S, cname)
        assert got[(cname, "__sizeof__")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


# ---- the reference's own marshalling against ours -------------------------

MODES = ("JM", "EH", "JMEH", "EHP", "FF", "scalar")
_PARAM_LEN = {"coeffs": 3, "lxu": 2, "lyv": 2, "gcenter": 2, "n_cells": 2, "transf": 16}


def _unwrap(a):
    a = getattr(a, "_obj", a)   # byref(...) -> the struct
    return a.value if hasattr(a, "value") else a


def _fields(struct, n):
    """Every field of a ctypes struct as plain values; pointer fields read as
    arrays (n elements for bundles, the fixed lengths for reflparams)."""
    import numpy as np
    out = {}
    for name, typ in struct._fields_:
        v = getattr(struct, name)
        if hasattr(typ, "contents"):   # a pointer type
            length = _PARAM_LEN.get(name, n)
            out[name] = np.ctypeslib.as_array(v, shape=(length,)).copy() if v else None
        else:
            out[name] = v
    return out


class _Recorder:
    """A stand-in for the loaded library: every callKernelf_* records its
    arguments as values and writes a known pattern into its result bundle."""

    def __init__(self, gs, gt):
        self.gs, self.gt, self.calls = gs, gt, []
        for mode in MODES:
            setattr(self, f"callKernelf_{mode}", self._make(mode))

    def _make(self, mode):
        def call(*args):
            import numpy as np
            a = [_unwrap(x) for x in args]
            res, csp, ctp, cs, ct, cin = a[:6]
            rec = {"mode": mode, "csp": _fields(csp, 0), "ctp": _fields(ctp, 0), "cs_size": cs.size,
                   "ct_size": ct.size, "cin": _fields(cin, self.gs), "scalars": [float(x) for x in a[6:9]]}
            self.calls.append(rec)
            for i, (name, _) in enumerate(res._fields_):
                np.ctypeslib.as_array(getattr(res, name), shape=(self.gt,))[:] = \
                    np.arange(self.gt, dtype=np.float32) * 0.25 + i
            return 0
        return call


def _same(a, b):
    import numpy as np
    if isinstance(a, dict):
        return a.keys() == b.keys() and all(_same(a[k], b[k]) for k in a)
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return a is not None and b is not None and np.array_equal(a, b)
    if isinstance(a, list):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    return a == b


def _obj_arrays(obj):
    import numpy as np
    objs = obj if isinstance(obj, list) else [obj]
    names = lambda o: getattr(o, "memlist", None) or (("x", "y", "z") if hasattr(o, "x") else ("S",))
    return [np.asarray(getattr(o, m)) for o in objs for m in names(o)]


@pytest.mark.parametrize("mode", MODES)
def test_reference_marshalling_equals_ours(ref_pypo, monkeypatch, mode):
    """The reference's own PyPO_GPUf (src/PyPO/BindGPU.py:83-224, its
    BindUtils marshalling and thread manager) and pypo_gb300.BindGPU.PyPO_GPUf
    on the same reflDicts and runPODict, each calling a recording stand-in
    for the library: the same entry point, the same reflparamsf field values,
    container sizes, source arrays, k, epsilon and time direction, and the
    same returned objects from the same result bundle."""
    import numpy as np
    from tests.common import load_case
    from pypo_gb300 import BindGPU as OurBind, PyPOTypes as PT
    BindGPU, _ = ref_pypo
    c = load_case("paruv_to_ff" if mode == "FF" else "paruv_to_plane")
    src, tgt = c["src"], c["tgt"]
    shape = tuple(int(v) for v in src["gridsize"])
    gs, gt = int(np.prod(shape)), int(np.prod(tgt["gridsize"]))
    d = {"mode": mode, "exp": "bwd", "epsilon": 1.7, "k": float(c["k"]), "nThreads": 256}
    if mode == "scalar":
        d["s_scalarfield"] = PT.scalarfield((c["cur"][0] + 1j * c["cur"][1]).reshape(shape))
    else:
        comps = [(c["cur"][6 * g + a] + 1j * c["cur"][6 * g + 3 + a]).reshape(shape) for g in range(2)
                 for a in range(3)]
        d["s_current"] = PT.currents(*comps)
    theirs, ours = _Recorder(gs, gt), _Recorder(gs, gt)
    monkeypatch.setattr(BindGPU, "loadGPUlib", lambda: theirs)
    got_ref = BindGPU.PyPO_GPUf(src, tgt, dict(d))
    monkeypatch.setattr(OurBind, "load", lambda: ours)
    got_ours = OurBind.PyPO_GPUf(src, tgt, dict(d))
    assert len(theirs.calls) == len(ours.calls) == 1
    a, b = theirs.calls[0], ours.calls[0]
    for key in ("mode", "csp", "ctp", "cs_size", "ct_size", "cin", "scalars"):
        assert _same(a[key], b[key]), (mode, key)
    ra, rb = _obj_arrays(got_ref), _obj_arrays(got_ours)
    assert len(ra) == len(rb) and all(np.array_equal(x, y) for x, y in zip(ra, rb)), mode
