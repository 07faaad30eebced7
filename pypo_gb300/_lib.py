"""ctypes handle on libpo_gb300.so (built in-tree by pypo_gb300/build.py).

There is no fallback: when the library is missing or cannot be loaded, every
entry point raises POError.
"""
import ctypes
import pathlib

from . import Structs as S

LIB_PATH = pathlib.Path(__file__).resolve().parent / "libpo_gb300.so"

#: every symbol declared in include/po_gb300.h
EXPORTS = ("po_last_error", "po_n_out", "po_last_launches", "po_generate_grid", "po_generate_grid_dev",
           "po_correlated_error", "po_correlated_error_dev", "po_gauss_beam_dev", "po_calc_jm_dev",
           "po_efficiency_sums_dev", "po_fit_gauss_abs_dev", "po_generate_gauss_dev", "po_fmin", "po_run_d",
           "po_run_dev", "po_run_dev_static", "po_last_extent", "po_last_band_pairs", "po_adjoint_dev", "po_adjoint_d", "po_device_error", "po_wait_selftest", "po_scratch_in_use", "po_timing_enable", "po_timing_collect", "po_fp32_probe",
           "callKernelf_JM", "callKernelf_EH", "callKernelf_JMEH", "callKernelf_EHP",
           "callKernelf_FF", "callKernelf_scalar", "callRTKernel")

#: po_objective: int f(const double *x, double *fx, void *ctx)
OBJECTIVE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                             ctypes.c_void_p)

MODE_ID = {"JM": 0, "EH": 1, "JMEH": 2, "EHP": 3, "FF": 4, "scalar": 5}


class POError(RuntimeError):
    """A libpo_gb300 call failed (the message is po_last_error())."""


_lib = None


def load():
    """Load the library once and declare argument types."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise POError(f"{LIB_PATH} is missing: build it with `python -m pypo_gb300.build` "
                      "(or __graft_entry__.build()); there is no CPU fallback")
    try:
        lib = ctypes.CDLL(str(LIB_PATH))
    except OSError as e:
        raise POError(f"cannot load {LIB_PATH}: {e}") from e
    P = ctypes.POINTER
    c_long, c_int, c_double, c_void_p = ctypes.c_long, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    lib.po_last_error.restype = ctypes.c_char_p
    lib.po_last_error.argtypes = []
    lib.po_n_out.restype = c_int
    lib.po_n_out.argtypes = [c_int]
    lib.po_last_launches.restype = c_int
    lib.po_last_launches.argtypes = []
    lib.po_generate_grid.restype = c_int
    lib.po_generate_grid.argtypes = [S.reflparams, P(S.reflcontainer), c_int, c_int]
    lib.po_generate_grid_dev.restype = c_int
    lib.po_generate_grid_dev.argtypes = [S.reflparams, c_void_p, c_int, c_int, c_void_p]
    lib.po_gauss_beam_dev.restype = c_int
    lib.po_gauss_beam_dev.argtypes = [c_long, c_void_p, c_double, c_double, c_double, c_double, c_int, c_void_p,
                                      c_void_p, c_void_p]
    lib.po_calc_jm_dev.restype = c_int
    lib.po_calc_jm_dev.argtypes = [c_long, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
    lib.po_efficiency_sums_dev.restype = c_int
    lib.po_efficiency_sums_dev.argtypes = [c_long, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                           c_void_p, c_void_p]
    lib.po_fit_gauss_abs_dev.restype = c_int
    lib.po_fit_gauss_abs_dev.argtypes = [c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_int, c_int,
                                         c_double, c_void_p, c_void_p, c_void_p]
    lib.po_generate_gauss_dev.restype = c_int
    lib.po_generate_gauss_dev.argtypes = [c_long, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
    lib.po_fmin.restype = c_int
    lib.po_fmin.argtypes = [c_int, c_void_p, c_double, c_double, c_long, c_long, OBJECTIVE, c_void_p, c_void_p,
                            c_void_p, c_void_p, c_void_p]
    lib.po_run_d.restype = c_int
    lib.po_run_d.argtypes = [c_int, c_long, c_void_p, c_int, c_int, c_int, c_void_p, c_long, c_void_p,
                             c_double, c_double, c_double, c_int, c_void_p]
    lib.po_last_extent.restype = c_double
    lib.po_last_extent.argtypes = []
    lib.po_last_band_pairs.restype = ctypes.c_ulonglong
    lib.po_last_band_pairs.argtypes = []
    lib.po_run_dev.restype = c_int
    lib.po_run_dev.argtypes = [c_int, c_long, c_void_p, c_int, c_int, c_int, c_void_p, c_long, c_void_p,
                               c_double, c_double, c_double, c_int, c_int, c_void_p, c_void_p]
    lib.po_run_dev_static.restype = c_int
    lib.po_run_dev_static.argtypes = [c_int, c_long, c_void_p, c_int, c_int, c_int, c_void_p, c_long,
                                      c_void_p, c_double, c_double, c_double, c_int, c_void_p, c_void_p,
                                      c_void_p]
    lib.po_adjoint_dev.restype = c_int
    lib.po_adjoint_dev.argtypes = [c_int, c_long, c_void_p, c_int, c_int, c_int, c_void_p, c_long, c_void_p,
                                   c_double, c_double, c_double, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                   c_void_p, c_void_p]
    lib.po_adjoint_d.restype = c_int
    lib.po_adjoint_d.argtypes = [c_int, c_long, c_void_p, c_int, c_int, c_int, c_void_p, c_long, c_void_p,
                                 c_double, c_double, c_double, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.po_device_error.restype = c_int
    lib.po_device_error.argtypes = [c_void_p, P(c_int)]
    lib.po_timing_enable.restype = c_int
    lib.po_timing_enable.argtypes = [c_int]
    lib.po_timing_collect.restype = c_int
    lib.po_timing_collect.argtypes = [P(ctypes.c_float), c_int]
    lib.po_fp32_probe.restype = c_int
    lib.po_fp32_probe.argtypes = [c_int, c_int, c_void_p, c_void_p]
    lib.po_correlated_error.restype = c_int
    lib.po_correlated_error.argtypes = [c_long, c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_uint, c_int,
                                        c_void_p, c_int]
    lib.po_correlated_error_dev.restype = c_int
    lib.po_correlated_error_dev.argtypes = lib.po_correlated_error.argtypes + [c_void_p]
    lib.po_wait_selftest.restype = c_int
    lib.po_wait_selftest.argtypes = [ctypes.c_uint, c_void_p, c_int, c_void_p]
    lib.po_scratch_in_use.restype = c_int
    lib.po_scratch_in_use.argtypes = [P(ctypes.c_ulonglong)]
    # Drop-in entry points: the reference's argtypes (src/PyPO/BindGPU.py:34-74).
    common = [S.reflparamsf, S.reflparamsf, P(S.reflcontainerf), P(S.reflcontainerf)]
    tail = [ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int, c_int]
    for name, res_t, in_t in (("callKernelf_JM", S.c2Bundlef, S.c2Bundlef),
                              ("callKernelf_EH", S.c2Bundlef, S.c2Bundlef),
                              ("callKernelf_JMEH", S.c4Bundlef, S.c2Bundlef),
                              ("callKernelf_EHP", S.c2rBundlef, S.c2Bundlef),
                              ("callKernelf_FF", S.c2Bundlef, S.c2Bundlef),
                              ("callKernelf_scalar", S.arrC1f, S.arrC1f)):
        fn = getattr(lib, name)
        fn.argtypes = [P(res_t)] + common + [P(in_t)] + tail
        fn.restype = c_int
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().po_last_error().decode(errors="replace")
        raise POError(f"libpo_gb300 status {rc}: {msg}")
