"""Validation of the runPODict keys the GPU binding consumes.

Mirrors the propagation-relevant part of reference src/PyPO/Checks.py:1445-1602
(check_runPODict): `exp` defaults to "fwd", `epsilon` to 1, the mode must be
one of JM, EH, JMEH, EHP, FF, scalar, and errors raise RunPOError. Name
bookkeeping (name_JM, name_EH, ...) belongs to System and is not repeated here.
"""
PO_modelist = ["JM", "EH", "JMEH", "EHP", "FF", "scalar"]


class RunPOError(Exception):
    """Raised when a runPODict is not valid (reference Checks.py RunPOError)."""


def check_runPODict_gpu(runPODict):
    err = []
    runPODict.setdefault("exp", "fwd")
    runPODict.setdefault("epsilon", 1.0)
    mode = runPODict.get("mode")
    if mode is None:
        err.append("runPODict is missing field 'mode'")
    elif mode not in PO_modelist:
        err.append(f"{mode} is not a valid propagation mode.")
    if runPODict["exp"] not in ("fwd", "bwd"):
        err.append(f"exp must be 'fwd' or 'bwd', not {runPODict['exp']!r}")
    if mode == "scalar":
        if "s_scalarfield" not in runPODict:
            err.append("runPODict is missing field 's_scalarfield'")
    elif mode is not None and "s_current" not in runPODict:
        err.append("runPODict is missing field 's_current'")
    if "k" not in runPODict:
        src = runPODict.get("s_scalarfield" if mode == "scalar" else "s_current")
        if src is not None and hasattr(src, "k"):
            runPODict["k"] = src.k
        else:
            err.append("runPODict has no wavenumber: set 'k' or setMeta on the source")
    if runPODict.get("precision", "mixed") not in ("mixed", "fp64"):
        err.append("precision must be 'mixed' or 'fp64'")
    if err:
        raise RunPOError("\n".join(err))
    return runPODict
