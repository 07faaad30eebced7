"""ctypes mirrors of the structs that cross PyPO's physical-optics C-ABI.

The field order and types must match the reference's C structs byte for byte,
because `callKernelf_*` in libpo_gb300 is a drop-in for the reference's
`libpypogpu` entry points (reference: src/include/Structs.h:42-147 for the
double variants, :243-348 for the float variants; ctypes side
src/PyPO/Structs.py:18-324). The double variants are also what the
reference's CPU library takes, which the test oracle uses.
"""
import ctypes

_C3 = ["x", "y", "z"]


def _bundle_fields(ctype, n_complex, n_real=0):
    fields = []
    for b in range(1, n_complex + 1):
        for part in ("r", "i"):
            for ax in _C3:
                fields.append((f"{part}{b}{ax}", ctypes.POINTER(ctype)))
    for b in range(n_complex + 1, n_complex + 1 + n_real):
        for ax in _C3:
            fields.append((f"r{b}{ax}", ctypes.POINTER(ctype)))
    return fields


def _reflparams_fields(ctype):
    return [("coeffs", ctypes.POINTER(ctype)),
            ("lxu", ctypes.POINTER(ctype)),
            ("lyv", ctypes.POINTER(ctype)),
            ("n_cells", ctypes.POINTER(ctypes.c_int)),
            ("flip", ctypes.c_bool),
            ("gmode", ctypes.c_int),
            ("gcenter", ctypes.POINTER(ctype)),
            ("ecc_uv", ctype),
            ("rot_uv", ctype),
            ("type", ctypes.c_int),
            ("transf", ctypes.POINTER(ctype)),
            ("rms", ctype),
            ("rms_seed", ctypes.c_uint)]


def _reflcontainer_fields(ctype):
    return [("size", ctypes.c_int)] + [(n, ctypes.POINTER(ctype))
                                        for n in ("x", "y", "z", "nx", "ny", "nz", "area")]


class arrC1(ctypes.Structure):
    _fields_ = [("x", ctypes.POINTER(ctypes.c_double)), ("y", ctypes.POINTER(ctypes.c_double))]


class arrC1f(ctypes.Structure):
    _fields_ = [("x", ctypes.POINTER(ctypes.c_float)), ("y", ctypes.POINTER(ctypes.c_float))]


class c2Bundle(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_double, 2)


class c2Bundlef(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_float, 2)


class c4Bundle(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_double, 4)


class c4Bundlef(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_float, 4)


class c2rBundle(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_double, 2, 1)


class c2rBundlef(ctypes.Structure):
    _fields_ = _bundle_fields(ctypes.c_float, 2, 1)


class reflparams(ctypes.Structure):
    _fields_ = _reflparams_fields(ctypes.c_double)


class reflparamsf(ctypes.Structure):
    _fields_ = _reflparams_fields(ctypes.c_float)


class reflcontainer(ctypes.Structure):
    _fields_ = _reflcontainer_fields(ctypes.c_double)


class reflcontainerf(ctypes.Structure):
    _fields_ = _reflcontainer_fields(ctypes.c_float)


class vecGPODict(ctypes.Structure):
    """Vector Gaussian beam parameters (reference src/include/Structs.h vecGPODict)."""
    _fields_ = [("lam", ctypes.c_double), ("w0", ctypes.c_double), ("z", ctypes.c_double),
                ("n", ctypes.c_double), ("power", ctypes.c_double), ("mode", ctypes.c_int)]


#: number of output arrays per mode in bundle order: JM/EH/FF c2Bundle (12),
#: JMEH c4Bundle (24), EHP c2rBundle (15), scalar arrC1 (2)
MODES = ("JM", "EH", "JMEH", "EHP", "FF", "scalar")
N_OUT = {"JM": 12, "EH": 12, "JMEH": 24, "EHP": 15, "FF": 12, "scalar": 2}
BUNDLE_F = {"JM": c2Bundlef, "EH": c2Bundlef, "JMEH": c4Bundlef, "EHP": c2rBundlef,
            "FF": c2Bundlef, "scalar": arrC1f}
BUNDLE_D = {"JM": c2Bundle, "EH": c2Bundle, "JMEH": c4Bundle, "EHP": c2rBundle,
            "FF": c2Bundle, "scalar": arrC1}
