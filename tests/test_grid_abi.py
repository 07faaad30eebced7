"""Host-side parts of libpo_gb300 that need no GPU: the exported C-ABI, the
struct layouts, argument validation, and the FP64 grid generator against the
reference's generateGrid (golden vectors)."""
import ctypes
import pathlib
import re
import subprocess

import numpy as np
import pytest

from tests.common import GOLDEN, from_json

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "po_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*typedef\b[^;]*;", "", text, flags=re.M)   # function-pointer types are not entry points
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:(?:unsigned|signed|long|short)\s+)*\w+(?:\s+|\s*\*\s*)(\w+)\s*\(",
                                 text, flags=re.M)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "pypo_gb300" / "libpo_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    from pypo_gb300 import _lib
    assert set(_lib.EXPORTS) == set(names)
    for n in names:
        getattr(lib, n)


def test_struct_layouts_match_ctypes(tmp_path):
    """Offsets of the C structs (compiled from include/po_gb300.h) equal the ctypes mirrors."""
    from pypo_gb300 import Structs as S
    specs = {"reflparams": S.reflparams, "reflparamsf": S.reflparamsf, "reflcontainer": S.reflcontainer,
             "reflcontainerf": S.reflcontainerf, "c2Bundlef": S.c2Bundlef, "c4Bundlef": S.c4Bundlef,
             "c2rBundlef": S.c2rBundlef, "arrC1f": S.arrC1f}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, cls in specs.items():
        lines.append(f'printf("{cname} __sizeof__ %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, cls in specs.items():
        assert got[(cname, "__sizeof__")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


@pytest.mark.parametrize("name", ["par_xy", "par_uv", "hyp_xy", "hyp_uv", "ell_xy", "ell_uv", "pl_xy",
                                  "pl_uv", "aoe", "par_rms"])
def test_grid_matches_reference(lib, name):
    from pypo_gb300 import engine
    g = np.load(GOLDEN / "golden_grids.npz")
    d = from_json(str(g[f"{name}_json"]))
    ref = g[f"{name}_grid"]
    got = engine.generate_grid(d)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * max(1.0, np.abs(ref).max()))


def test_invalid_arguments_are_rejected_before_any_device_work(lib):
    from pypo_gb300 import engine
    from pypo_gb300._lib import POError
    s7 = np.zeros((7, 4))
    s7[5] = 1.0
    s7[6] = 1.0
    t7 = np.zeros((7, 3))
    cur = np.zeros((12, 4))
    bad = [dict(mode="EH", gmode=0, ncx=3, ncy=3, k=1.0, t=-1.0, msg="ncx \\* ncy"),
           dict(mode="EH", gmode=0, ncx=2, ncy=2, k=-1.0, t=-1.0, msg="wavenumber"),
           dict(mode="EH", gmode=0, ncx=2, ncy=2, k=1.0, t=0.5, msg="t_direction")]
    for b in bad:
        with pytest.raises(POError, match=b["msg"]):
            engine.propagate(b["mode"], s7, cur, b["gmode"], b["ncx"], b["ncy"], t7, b["k"], t_dir=b["t"])
    # raw C-ABI: unknown mode and unknown precision give a status and a message
    out = np.zeros((12, 3))
    rc = lib.po_run_d(9, 4, s7.ctypes.data, 0, 2, 2, cur.ctypes.data, 3, t7.ctypes.data, 1.0, 1.0, -1.0, 0,
                      out.ctypes.data)
    assert rc != 0 and b"mode" in lib.po_last_error()
    rc = lib.po_run_d(1, 4, s7.ctypes.data, 0, 2, 2, cur.ctypes.data, 3, t7.ctypes.data, 1.0, 1.0, -1.0, 7,
                      out.ctypes.data)
    assert rc != 0 and b"precision" in lib.po_last_error()
    # sizes past 32-bit device indices (the buffers are never read: the check comes first)
    rc = lib.po_run_d(1, 1 << 31, s7.ctypes.data, -1, 0, 0, cur.ctypes.data, 3, t7.ctypes.data, 1.0, 1.0, -1.0, 0,
                      out.ctypes.data)
    assert rc == 1 and b"2^31 - 1" in lib.po_last_error()
    # empty target: nothing to do, success
    rc = lib.po_run_d(1, 4, s7.ctypes.data, 0, 2, 2, cur.ctypes.data, 0, t7.ctypes.data, 1.0, 1.0, -1.0, 0,
                      out.ctypes.data)
    assert rc == 0
    assert lib.po_n_out(2) == 24 and lib.po_n_out(3) == 15 and lib.po_n_out(5) == 2 and lib.po_n_out(6) == -1


def test_runpodict_validation():
    from pypo_gb300.checks import RunPOError, check_runPODict_gpu
    d = {"mode": "EH", "s_current": object(), "k": 1.0}
    check_runPODict_gpu(d)
    assert d["exp"] == "fwd" and d["epsilon"] == 1.0
    for bad in ({"mode": "XX", "s_current": 1, "k": 1}, {"mode": "EH", "k": 1},
                {"mode": "scalar", "s_current": 1, "k": 1}, {"mode": "EH", "s_current": 1, "k": 1, "exp": "up"},
                {"mode": "EH", "s_current": 1}):
        with pytest.raises(RunPOError):
            check_runPODict_gpu(dict(bad))


def test_mixed_extent_and_warning():
    """The frame half-extent that sets the mixed path's precision, and the
    host-side warning beyond the measured limit."""
    import warnings
    from pypo_gb300 import engine
    s7 = np.zeros((7, 2))
    s7[0] = [-1.0, 1.0]
    t7 = np.zeros((7, 1))
    t7[2] = 1000.0                                        # mm
    k = 2 * np.pi / 0.5                                   # 2 wavelengths per mm
    assert engine.mixed_extent("EH", s7, t7, k) == 1000.0   # half of the 1000 mm z side, x 2
    assert engine.mixed_extent("FF", s7, t7, k) == 2.0      # largest source coordinate only
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        engine._extent_warning(1.0e3, "mixed")             # 1e3 wavelengths: no warning
    far = t7.copy()
    far[2] = 1.0e5
    m = engine.mixed_extent("EH", s7, far, k)
    with pytest.warns(RuntimeWarning, match="fp64"):
        engine._extent_warning(m, "mixed")
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        engine._extent_warning(m, "fp64")


def test_adjoint_output_buffers_are_checked_before_any_device_work(lib):
    """engine.adjoint writes into caller-provided arrays (page-locked ones, for
    instance) only when their shape and layout fit."""
    from pypo_gb300 import engine
    from pypo_gb300._lib import POError
    s7 = np.zeros((7, 4))
    t7 = np.zeros((7, 3))
    cur = np.zeros((12, 4))
    cot = np.zeros((12, 3))
    for bad in ({"cur": np.zeros((12, 5))}, {"ds": np.zeros(4, dtype=np.float32)},
                {"dt": np.zeros((3, 1))}, {"cur": np.zeros((4, 12)).T}):
        with pytest.raises(POError, match="out\\["):
            engine.adjoint("EH", s7, cur, -1, 0, 0, t7, 1.0, cot, out=bad)


def test_bundles_keep_their_blocks_alive():
    """A bundle made from a temporary block keeps it alive: its pointers stay valid."""
    import gc
    import ctypes
    from pypo_gb300 import Structs as S, marshal as M
    st = M.bundle(S.c2Bundlef, np.arange(12 * 5, dtype=np.float32).reshape(12, 5) + 1.0, ctypes.c_float)
    junk = [np.zeros((12, 5), dtype=np.float32) for _ in range(50)]   # would reuse a freed block
    gc.collect()
    assert st.r1x[0] == 1.0 and st.i2z[4] == 60.0
    del junk
