"""Shared helpers of the test suite: golden fixtures and error metrics."""
import json
import pathlib

import numpy as np

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"

#: the accuracy bar of the mixed-precision path against the FP64 oracle
REL_L2_TOL = 1e-5
PHASE_TOL = 1e-4        # rad, on components within 20 dB of the peak
#: the FP64 GPU path against the FP64 oracle (same formula, different order)
FP64_TOL = 1e-10


def load_case(name):
    d = np.load(GOLDEN / f"golden_{name}.npz")
    out = {k: d[k] for k in d.files}
    out["src"] = from_json(str(out.pop("src_json")))
    out["tgt"] = from_json(str(out.pop("tgt_json")))
    return out


def from_json(s):
    d = json.loads(s)
    for k, v in d.items():
        if isinstance(v, list):
            d[k] = np.asarray(v)
    return d


def cplx_rows(block, mode):
    """Complex components (rows) of an output block in bundle order."""
    if mode == "scalar":
        return block[0:1] + 1j * block[1:2]
    n_c = {"JM": 2, "EH": 2, "FF": 2, "JMEH": 4, "EHP": 2}[mode]
    rows = []
    for b in range(n_c):
        rows.append(block[6 * b:6 * b + 3] + 1j * block[6 * b + 3:6 * b + 6])
    return np.concatenate(rows)


def rel_l2(got, ref):
    den = np.linalg.norm(ref)
    return np.linalg.norm(got - ref) / den if den > 0 else np.linalg.norm(got - ref)


def max_phase_err(got_c, ref_c, floor_db=20.0):
    """Largest |arg(got/ref)| over complex components within floor_db of the peak."""
    mag = np.abs(ref_c)
    peak = mag.max()
    if peak == 0:
        return 0.0
    sel = mag >= peak * 10 ** (-floor_db / 20)
    return float(np.abs(np.angle(got_c[sel] / ref_c[sel])).max())


def errors(got, ref, mode):
    """(rel L2 over all rows, max phase error over complex rows)."""
    e = rel_l2(got, ref)
    if mode == "EHP":
        p = max_phase_err(cplx_rows(got[:12], mode), cplx_rows(ref[:12], mode))
    else:
        p = max_phase_err(cplx_rows(got, mode), cplx_rows(ref, mode))
    return e, p
