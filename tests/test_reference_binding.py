"""The drop-in claim, checked with the reference's own Python binding.

PyPO's GPU path loads its CUDA library in BindGPU.loadGPUlib
(src/PyPO/BindGPU.py:18-81) and binds every entry point's argtypes there,
with the struct layouts of src/PyPO/Structs.py. Here the reference's own
modules are imported from its checkout, loadGPUlib is pointed at
libpo_gb300.so (only the library name changes), and:
  * every argtypes assignment of the unmodified loader binds, including the
    ray tracer's callRTKernel, which this library refuses with a status;
  * every ctypes struct of the reference's Structs.py has the field names,
    offsets and size of the C structs in include/po_gb300.h.
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
