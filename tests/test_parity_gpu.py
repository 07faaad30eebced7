"""GPU parity: libpo_gb300 against the reference's own FP64 outputs.

Every mode, both time directions, both precisions, through the explicit-grid
C-ABI (po_run_d), the device-pointer C-ABI (po_run_dev) and the drop-in
float ABI (callKernelf_* via PyPO_GPUf). The bar: mixed precision within
1e-5 relative L2 and 1e-4 rad phase (components within 20 dB of the peak);
the plain FP64 path within 1e-10.
"""
import numpy as np
import pytest

from tests.common import FP64_TOL, PHASE_TOL, REL_L2_TOL, errors, load_case

pytestmark = pytest.mark.gpu

CASES = [("paruv_to_plane", ["JM", "EH", "JMEH", "EHP", "scalar"]),
         ("parxy_to_plane", ["EH", "JMEH"]),
         ("paruv_to_ff", ["FF"]),
         ("hyp_to_ell", ["JM", "EH", "EHP"])]


def _run(c, mode, t, precision):
    from pypo_gb300 import engine
    src = c["src"]
    cur = c["cur"][:2] if mode == "scalar" else c["cur"]
    return engine.propagate(mode, c["src_grid"], cur, src["gmode"], *src["gridsize"], c["tgt_grid"],
                            float(c["k"]), float(c["epsilon"]), t, precision)


@pytest.mark.parametrize("name,modes", CASES)
def test_mixed_precision_matches_reference(cuda, lib, name, modes):
    c = load_case(name)
    for mode in modes:
        for tag, t in (("fwd", -1.0), ("bwd", 1.0)):
            ref = c[f"out_{mode}_{tag}"]
            got = _run(c, mode, t, "mixed")
            e, p = errors(got, ref, mode)
            assert e <= REL_L2_TOL, f"{name} {mode} {tag}: rel L2 {e:.3e}"
            assert p <= PHASE_TOL, f"{name} {mode} {tag}: phase {p:.3e} rad"


@pytest.mark.parametrize("name,modes", CASES + [("tangent", ["EH"])])
def test_fp64_path_matches_reference(cuda, lib, name, modes):
    c = load_case(name)
    for mode in modes:
        for tag, t in (("fwd", -1.0), ("bwd", 1.0)):
            ref = c[f"out_{mode}_{tag}"]
            got = _run(c, mode, t, "fp64")
            np.testing.assert_allclose(got, ref, rtol=0, atol=FP64_TOL * np.abs(ref).max(),
                                       err_msg=f"{name} {mode} {tag}")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tangent_pairs(cuda, lib, oracle_mod):
    """Dyadic grids with pairs tangent in exact arithmetic (n . d == 0).

    The reference decides those pairs by the sign of its rounded FP64
    n . R_hat; the FP64 path repeats that rounding and matches exactly. The
    mixed path leaves every pair with |n . R_hat| below 1e-6 out of its FP32
    sums, lists it, and a fixup decides it the reference's way and adds its
    FP64 term, so it meets the bar at every target, the touched ones too
    (alone as well), and so does its adjoint against the oracle's."""
    c = load_case("tangent")
    s, t = c["src_grid"], c["tgt_grid"]
    d = t[:3, :, None] - s[:3, None, :]
    nd = (s[3:6, None, :] * d).sum(0)
    touched = np.any(np.abs(nd) <= 1e-12 * np.sqrt((d ** 2).sum(0)), axis=1)
    assert 0 < touched.sum() < 0.2 * t.shape[1]
    ref = c["out_EH_fwd"]
    got = _run(c, "EH", -1.0, "mixed")
    # every exactly tangent pair (36) is inside the band, and few others are
    n_tangent = int((np.abs(nd) <= 1e-12 * np.sqrt((d ** 2).sum(0))).sum())
    from pypo_gb300 import engine
    assert n_tangent == 36 and n_tangent <= engine.last_band_pairs() <= 4 * n_tangent
    for sel in (slice(None), touched):
        e, p = errors(got[:, sel], ref[:, sel], "EH")
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (e, p)
    from pypo_gb300 import engine
    src = c["src"]
    grid = (src["gmode"], *src["gridsize"])
    cot = np.random.default_rng(8).standard_normal((12, t.shape[1]))
    gm = engine.adjoint("EH", s, c["cur"], *grid, t, float(c["k"]), cot)
    go = oracle_mod.adjoint("EH", s, c["cur"], *grid, t, float(c["k"]), cot)
    for name, want in go.items():
        assert _rel(gm[name], want) <= REL_L2_TOL, (name, _rel(gm[name], want))
    assert _rel(gm["dt"][touched], go["dt"][touched]) <= REL_L2_TOL


def test_far_field_horizon_pairs(cuda, lib, oracle_mod):
    """Sources on z = 0 facing +z and directions within 1e-7 rad of their
    horizon on both sides (n . r_hat = cos theta from -1e-7 to 1e-7, and
    6e-17 at theta = pi/2 in FP64): every such pair is inside the tangent
    band, so the reference's own decision holds. Directions below the
    horizon give exactly zero, as in the reference; the rest meet the bar,
    forward and adjoint, against the oracle."""
    from pypo_gb300 import engine
    rng = np.random.default_rng(31)
    ns = 500
    s7 = np.zeros((7, ns))
    s7[0:2] = rng.uniform(-1, 1, (2, ns))
    s7[5] = 1.0
    s7[6] = rng.uniform(0.5, 1.5, ns) * 1e-3
    k = 2 * np.pi / 0.05
    offs = np.array([-1e-7, -3e-8, -1e-8, 0.0, 1e-8, 3e-8, 1e-7])
    d = np.zeros((7, 60 + 4 * offs.size))
    d[0, :60] = rng.uniform(0, np.radians(60), 60)
    d[0, 60:] = np.pi / 2 + np.repeat(offs, 4)
    d[1] = rng.uniform(0, 2 * np.pi, d.shape[1])
    below = np.cos(d[0]) < 0
    assert below.sum() == 12
    for m_zero in (True, False):
        cur = rng.standard_normal((12, ns))
        if m_zero:
            cur[6:] = 0.0
        got = engine.propagate("FF", s7, cur, -1, 0, 0, d, k)
        ref = oracle_mod.run("FF", s7, cur, -1, 0, 0, d, k)
        assert np.all(ref[:, below] == 0) and np.all(got[:, below] == 0)
        e, p = errors(got, ref, "FF")
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (m_zero, e, p)
        e, p = errors(got[:, 60:], ref[:, 60:], "FF")   # the horizon directions alone
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (m_zero, e, p)
        cot = rng.standard_normal((12, d.shape[1]))
        gm = engine.adjoint("FF", s7, cur, -1, 0, 0, d, k, cot, want=("cur", "ds"))
        go = oracle_mod.adjoint("FF", s7, cur, -1, 0, 0, d, k, cot)
        assert _rel(gm["cur"], go["cur"]) <= REL_L2_TOL, (m_zero, _rel(gm["cur"], go["cur"]))
        assert _rel(gm["ds"], go["ds"]) <= 1e-4, (m_zero, _rel(gm["ds"], go["ds"]))


def test_device_entry_equals_host_entry(cuda, lib):
    import torch
    from pypo_gb300 import engine
    c = load_case("paruv_to_plane")
    src = c["src"]
    for mode in ("EH", "JMEH", "EHP", "scalar"):
        cur = c["cur"][:2] if mode == "scalar" else c["cur"]
        host = engine.propagate(mode, c["src_grid"], cur, src["gmode"], *src["gridsize"], c["tgt_grid"],
                                float(c["k"]), float(c["epsilon"]), -1.0)
        dev = engine.propagate_dev(mode, torch.tensor(c["src_grid"], device=cuda), torch.tensor(cur, device=cuda),
                                   src["gmode"], *src["gridsize"], torch.tensor(c["tgt_grid"], device=cuda),
                                   float(c["k"]), float(c["epsilon"]), -1.0)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dev.cpu().numpy(), host)
    assert engine.device_error(torch.cuda.current_stream()) == 0


def _currents_obj(cur, shape, k):
    from pypo_gb300 import PyPOTypes as PT
    comps = [(cur[6 * g + a] + 1j * cur[6 * g + 3 + a]).reshape(shape) for g in range(2) for a in range(3)]
    obj = PT.currents(*comps)
    obj.setMeta("src", k)
    return obj


@pytest.mark.parametrize("name,modes", CASES)
def test_drop_in_float_abi(cuda, lib, name, modes):
    """PyPO_GPUf -> callKernelf_*: the reference's own binding call shape."""
    from pypo_gb300 import BindGPU, PyPOTypes as PT
    from pypo_gb300 import marshal as M
    c = load_case(name)
    src, tgt = c["src"], c["tgt"]
    shape = tuple(int(v) for v in src["gridsize"])
    for mode in modes:
        for tag in ("fwd", "bwd"):
            d = {"mode": mode, "exp": tag, "epsilon": float(c["epsilon"]), "k": float(c["k"])}
            if mode == "scalar":
                sf = PT.scalarfield((c["cur"][0] + 1j * c["cur"][1]).reshape(shape))
                sf.setMeta("src", float(c["k"]))
                d["s_scalarfield"] = sf
            else:
                d["s_current"] = _currents_obj(c["cur"], shape, float(c["k"]))
            out = BindGPU.PyPO_GPUf(src, tgt, d)
            if mode in ("JM", "EH", "FF"):
                got = M.currents_block(out.stack())
            elif mode == "JMEH":
                got = np.concatenate([M.currents_block(out[0].stack()), M.currents_block(out[1].stack())])
            elif mode == "EHP":
                got = np.concatenate([M.currents_block(out[0].stack()), np.stack([out[1].x, out[1].y, out[1].z]).reshape(3, -1)])
            else:
                got = np.stack([out.S.real.ravel(), out.S.imag.ravel()])
            ref = c[f"out_{mode}_{tag}"]
            e, p = errors(got, ref, mode)
            # float currents and float outputs add ~1e-7 on top of the kernel error
            assert e <= REL_L2_TOL, f"{name} {mode} {tag}: rel L2 {e:.3e}"
            assert p <= PHASE_TOL, f"{name} {mode} {tag}: phase {p:.3e}"
            # PyPO_GPUd (FP64 inputs) too
            got_d = BindGPU.PyPO_GPUd(src, tgt, d)
            if mode == "EH":
                e2, _ = errors(M.currents_block(got_d.stack()), ref, mode)
                assert e2 <= REL_L2_TOL


def test_coplanar_targets_every_pair_in_the_band(cuda, lib, oracle_mod):
    """Targets in the sources' own plane: n . d == 0 for every pair, so every
    pair is inside the tangent band (the reference counts them lit). The
    allocating entries list all of them (a call of up to 2^22 pairs can),
    and the fixups add every pair's FP64 term: forward and adjoint against
    the oracle at FP64 level. The allocation-free entry's list holds 16,384
    pairs, so with 18,000 it reports device error 103 through its status
    word instead of a wrong sum."""
    import ctypes
    import torch
    from pypo_gb300 import engine
    rng = np.random.default_rng(41)
    ns, nt = 150, 120
    s7 = np.zeros((7, ns))
    s7[0:2] = rng.uniform(-1, 1, (2, ns))
    s7[5] = 1.0
    s7[6] = rng.uniform(0.5, 1.5, ns) * 1e-3
    t7 = np.zeros((7, nt))
    t7[0:2] = rng.uniform(-1.3, 1.3, (2, nt))
    t7[5] = 1.0
    cur = rng.standard_normal((12, ns))
    k = 2 * np.pi / 0.1
    for mode in ("EH", "JM"):
        got = engine.propagate(mode, s7, cur, -1, 0, 0, t7, k)
        assert engine.last_band_pairs() == ns * nt
        ref = oracle_mod.run(mode, s7, cur, -1, 0, 0, t7, k)
        assert _rel(got, ref) <= 1e-12, (mode, _rel(got, ref))
    cot = rng.standard_normal((12, nt))
    gm = engine.adjoint("EH", s7, cur, -1, 0, 0, t7, k, cot)
    assert engine.last_band_pairs() == ns * nt
    go = oracle_mod.adjoint("EH", s7, cur, -1, 0, 0, t7, k, cot)
    for name, want in go.items():
        assert _rel(gm[name], want) <= 1e-10, (name, _rel(gm[name], want))
    # the allocation-free entry: its list overflows, and it says so
    d = {n: torch.tensor(a, device=cuda) for n, a in (("s7", s7), ("cur", cur), ("t7", t7))}
    out = torch.empty((12, nt), dtype=torch.float64, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    stream = torch.cuda.current_stream()
    rc = lib.po_run_dev_static(1, ns, d["s7"].data_ptr(), -1, 0, 0, d["cur"].data_ptr(), nt, d["t7"].data_ptr(),
                               float(k), 1.0, -1.0, 0, out.data_ptr(), status.data_ptr(),
                               ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.po_last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 103


def test_high_kr_against_reference_outputs(cuda, lib):
    """The reference's own FP64 outputs at the benchmark's phase scale
    (golden_highkr.npz: kR ~ 3.2e3 rad to the focal plane, EH, JM, EHP and
    scalar; the far field, FF; both time directions): the mixed path within
    the bar, the FP64 path to 1e-10."""
    from pypo_gb300 import engine
    c = load_case("highkr")
    src = c["src"]
    grid = (int(src["gmode"]), *[int(v) for v in src["gridsize"]])
    for mode, tg in (("EH", "tgt_grid"), ("JM", "tgt_grid"), ("EHP", "tgt_grid"), ("scalar", "tgt_grid"),
                     ("FF", "ff_grid")):
        cur = c["cur"][:2] if mode == "scalar" else c["cur"]
        for tag, t in (("fwd", -1.0), ("bwd", 1.0)):
            ref = c[f"out_{mode}_{tag}"]
            got = engine.propagate(mode, c["src_grid"], cur, *grid, c[tg], float(c["k"]), 1.0, t)
            e, p = errors(got, ref, mode)
            assert e <= REL_L2_TOL and p <= PHASE_TOL, (mode, tag, e, p)
            d = engine.propagate(mode, c["src_grid"], cur, *grid, c[tg], float(c["k"]), 1.0, t, "fp64")
            np.testing.assert_allclose(d, ref, rtol=0, atol=FP64_TOL * np.abs(ref).max(), err_msg=f"{mode} {tag}")


def test_no_band_pairs_on_the_dish_workloads(cuda, lib):
    """The dish workloads face their targets: no pair comes near tangency,
    so nothing is left to the FP64 fixup (and the near field's tiles are all
    proven lit)."""
    from pypo_gb300 import configs, engine
    for w in (configs.dish_eh(scale=0.2), configs.dish_ff(scale=0.1)):
        engine.propagate(w["mode"], w["s7"], w["cur"], w["gmode"], w["ncx"], w["ncy"], w["t7"], w["k"])
        assert engine.last_band_pairs() == 0, w["name"]


def test_drop_in_fills_the_grid_containers(cuda, lib):
    """callKernelf_* through the reference's call shape leaves the source and
    target grids in cs / ct, as the reference does: generated in FP64 (on the
    device here) and stored as float, equal to the reference's own grids
    (golden) to float rounding; and the result matches the golden output."""
    import ctypes
    from pypo_gb300 import Structs as S, marshal as M
    c = load_case("paruv_to_plane")
    src, tgt = c["src"], c["tgt"]
    f = ctypes.c_float
    csp, _k1 = M.fill_reflparams(src, f)
    ctp, _k2 = M.fill_reflparams(tgt, f)
    gs, gt = int(np.prod(src["gridsize"])), int(np.prod(tgt["gridsize"]))
    cs, sblock = M.alloc_container(gs, f)
    ct, tblock = M.alloc_container(gt, f)
    cur32 = np.ascontiguousarray(c["cur"], dtype=np.float32)   # kept alive: the bundle points into it
    cin = M.bundle(S.c2Bundlef, cur32, f)
    out = np.zeros((12, gt), dtype=np.float32)
    res = M.bundle(S.c2Bundlef, out, f)
    rc = lib.callKernelf_EH(ctypes.byref(res), csp, ctp, ctypes.byref(cs), ctypes.byref(ct), ctypes.byref(cin),
                            f(float(c["k"])), f(float(c["epsilon"])), f(-1.0), 1, 256)
    assert rc == 0, lib.po_last_error()
    for block, ref in ((sblock, c["src_grid"]), (tblock, c["tgt_grid"])):
        np.testing.assert_allclose(block, ref, rtol=0, atol=1e-6 * np.abs(ref).max())
    e, p = errors(out.astype(np.float64), c["out_EH_fwd"], "EH")
    assert e <= 1e-5 and p <= 1e-4, (e, p)
