"""The oracle (oracle/po_oracle.c) against the reference's own outputs.

The golden vectors were produced by the reference's compiled FP64 CPU
library (tests/golden/make_golden.py); the oracle must reproduce them to
rounding. Where the reference library is present (it is compiled from the
reference sources, so only where they exist) a live cross-check on fresh
random inputs runs as well.
"""
import numpy as np
import pytest

from tests.common import load_case

CASES = [("paruv_to_plane", ["JM", "EH", "JMEH", "EHP", "scalar"]),
         ("parxy_to_plane", ["EH", "JMEH"]),
         ("paruv_to_ff", ["FF"]),
         ("hyp_to_ell", ["JM", "EH", "EHP"]),
         ("tangent", ["EH"])]


@pytest.mark.parametrize("name,modes", CASES)
def test_oracle_matches_reference_golden(oracle_mod, name, modes):
    c = load_case(name)
    src = c["src"]
    for mode in modes:
        for tag, t in (("fwd", -1.0), ("bwd", 1.0)):
            cur = c["cur"][:2] if mode == "scalar" else c["cur"]
            got = oracle_mod.run(mode, c["src_grid"], cur, src["gmode"], *src["gridsize"], c["tgt_grid"],
                                 float(c["k"]), float(c["epsilon"]), t, nthreads=2)
            ref = c[f"out_{mode}_{tag}"]
            assert np.abs(ref).max() > 0, f"{name} {mode}: degenerate golden case"
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max(),
                                       err_msg=f"{name} {mode} {tag}")


def test_oracle_target_subset(oracle_mod):
    c = load_case("paruv_to_plane")
    src = c["src"]
    idx = np.array([0, 5, 77, 168])
    full = c["out_EH_fwd"]
    got = oracle_mod.run("EH", c["src_grid"], c["cur"], src["gmode"], *src["gridsize"], c["tgt_grid"],
                         float(c["k"]), float(c["epsilon"]), -1.0, tidx=idx)
    np.testing.assert_allclose(got, full[:, idx], rtol=0, atol=1e-12 * np.abs(full).max())


def test_oracle_live_against_reference(oracle_mod):
    if not oracle_mod.REF_PATH.exists():
        pytest.skip("reference library not built here (needs the reference sources)")
    from pypo_gb300 import surfaces as SF
    ref = oracle_mod.Reference()
    rng = np.random.default_rng(5)
    src = SF.paraboloid(2.0, [9, 14], gmode=1, lims_a=[0.5, 3.0], ecc_uv=0.2, rot_uv=10.0)
    tgt = SF.rotate_x(SF.translate(SF.plane([8, 6], gmode=0, lims_a=[-2, 2]), dz=4.0), 5.0)
    cur = rng.standard_normal((12, 9 * 14))
    for mode in ("JM", "EH", "JMEH", "EHP", "scalar"):
        cc = cur[:2] if mode == "scalar" else cur
        out, sg, tg = ref.propagate(mode, src, tgt, cc, k=3.1, epsilon=2.0, t_dir=-1.0, nthreads=2)
        got = oracle_mod.run(mode, sg, cc, 1, 9, 14, tg, 3.1, 2.0, -1.0, nthreads=3)
        np.testing.assert_allclose(got, out, rtol=0, atol=1e-12 * np.abs(out).max(), err_msg=mode)


def test_oracle_matches_reference_at_high_kr(oracle_mod):
    """The reference's own outputs at the benchmark's phase scale (kR ~ 3.2e3
    rad near field: EH, JM, EHP, scalar; k r' up to 6e2 rad far field: FF;
    golden_highkr.npz): the oracle's FP64 sums agree to rounding."""
    c = load_case("highkr")
    src = c["src"]
    for mode, tg in (("EH", "tgt_grid"), ("JM", "tgt_grid"), ("EHP", "tgt_grid"), ("scalar", "tgt_grid"),
                     ("FF", "ff_grid")):
        cur = c["cur"][:2] if mode == "scalar" else c["cur"]
        for tag, t in (("fwd", -1.0), ("bwd", 1.0)):
            got = oracle_mod.run(mode, c["src_grid"], cur, src["gmode"], *src["gridsize"], c[tg],
                                 float(c["k"]), float(c["epsilon"]), t, nthreads=4)
            ref = c[f"out_{mode}_{tag}"]
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max(), err_msg=f"{mode} {tag}")
