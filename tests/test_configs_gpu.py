"""The benchmark workloads as parity cases (GPU).

Gaussian feed -> dish, JM (full size, 1e8 pairs) against the oracle; the
D 1000 mm dish to its focal plane (EH, 2.3e10 pairs) and the D 2000 mm dish to
its far field (FF, 1.6e11 pairs), full size, against the plain FP64 GPU sum on
a 2 % target sample and against the oracle (the reference's CPU algorithm)
on 128 / 64 targets, forward and adjoint; feed -> perturbed dish -> far field
with gradients of sum |E_ff - E_ideal|^2 against central finite differences
of the oracle chain (h = 1e-6 lambda) on 64 random dish nodes; the Cassegrain
chain at full size stage by stage (each stage's mixed output against the FP64
GPU sum on 2 % of its targets and the oracle on 16, from the same inputs) and
on reduced grids end to end against the FP64 chain, forward and gradients.
"""
import numpy as np
import pytest

from tests.common import PHASE_TOL, REL_L2_TOL, errors

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_feed_to_dish_jm_full_size(cuda, lib, oracle_mod):
    from pypo_gb300 import configs, engine
    w = configs.feed_dish_jm()
    args = (w["mode"], w["s7"], w["cur"], w["gmode"], w["ncx"], w["ncy"], w["t7"], w["k"])
    got = engine.propagate(*args)
    ref = oracle_mod.run(*args)
    e, p = errors(got, ref, "JM")
    assert e <= REL_L2_TOL and p <= PHASE_TOL, (e, p)


@pytest.mark.parametrize("name,n_oracle", [("dish_eh", 128), ("dish_ff", 64)])
def test_dish_workloads_full_size_sampled(cuda, lib, oracle_mod, name, n_oracle):
    """Full-size run; per-point error on a 2 % random target sample against the
    FP64 GPU sum, and on n_oracle targets against the oracle, forward (rel L2
    and phase) and adjoint (every source, those targets)."""
    import torch
    from pypo_gb300 import configs, engine
    w = getattr(configs, name)()
    dev = cuda
    s7, cur, t7 = (torch.tensor(w[k], device=dev) for k in ("s7", "cur", "t7"))
    grid = (w["gmode"], w["ncx"], w["ncy"])
    got = engine.propagate_dev(w["mode"], s7, cur, *grid, t7, w["k"], m_zero=True).cpu().numpy()
    rng = np.random.default_rng(0)
    nt = t7.shape[1]
    idx = np.sort(rng.choice(nt, size=max(16, nt // 50), replace=False))
    t7s = torch.tensor(np.ascontiguousarray(w["t7"][:, idx]), device=dev)
    ref = engine.propagate_dev(w["mode"], s7, cur, *grid, t7s, w["k"], precision="fp64").cpu().numpy()
    e, p = errors(got[:, idx], ref, w["mode"])
    assert e <= REL_L2_TOL and p <= PHASE_TOL, (name, e, p)
    sub = np.sort(rng.choice(nt, size=n_oracle, replace=False))
    oref = oracle_mod.run(w["mode"], w["s7"], w["cur"], *grid, w["t7"], w["k"], tidx=sub)
    e2, p2 = errors(got[:, sub], oref, w["mode"])
    assert e2 <= REL_L2_TOL and p2 <= PHASE_TOL, (name, e2, p2)
    # the adjoint over every source and those targets, against the oracle's
    cot = rng.standard_normal((engine.n_out(w["mode"]), sub.size))
    t7o = np.ascontiguousarray(w["t7"][:, sub])
    gm = engine.adjoint(w["mode"], w["s7"], w["cur"], *grid, t7o, w["k"], cot)
    go = oracle_mod.adjoint(w["mode"], w["s7"], w["cur"], *grid, t7o, w["k"], cot)
    for g_name, want in go.items():
        assert _rel(gm[g_name], want) <= REL_L2_TOL, (name, g_name, _rel(gm[g_name], want))


def _trap_weight(i, gmode, ncx, ncy):
    xu, yv = i // ncy, i % ncy
    w = 0.5 if xu in (0, ncx - 1) else 1.0
    if gmode != 1 and yv in (0, ncy - 1):
        w *= 0.5
    return w


def test_perturbed_dish_chain_gradients_against_finite_differences(cuda, lib, oracle_mod):
    """feed -> dish (JM) -> far field (FF), dish displaced by a correlated surface
    error; L = sum |E_ff - E_ideal|^2 (E rows). Autograd (mixed) gradients against
    central FD of the oracle chain on 64 random nodes, and against the FP64
    autograd gradients on every node."""
    import torch
    from pypo_gb300 import autograd as A, configs, engine
    c = configs.dish_chain()
    dev = cuda
    T = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    k, lam = c["k"], c["lam"]
    f7, fcur, d7, ff7 = c["feed7"], c["feed_cur"], c["dish7"], c["ff7"]
    fg, dg = c["feed_grid"], c["dish_grid"]
    nd = d7.shape[1]
    # ideal far field: unperturbed dish, FP64
    j0 = engine.propagate("JM", f7, fcur, *fg, d7, k, precision="fp64")
    ideal = engine.propagate("FF", d7, j0, *dg, ff7, k, precision="fp64")

    def grads(precision):
        dd = T(c["delta"]).requires_grad_(True)
        fc = T(fcur).requires_grad_(True)
        jm = A.propagate("JM", T(f7), fc, *fg, T(d7), k, dt=dd, precision=precision)
        ff = A.propagate("FF", T(d7), jm, *dg, T(ff7), k, ds=dd, precision=precision)
        loss = ((ff[0:6] - T(ideal)[0:6]) ** 2).sum()
        loss.backward()
        return dd.grad.cpu().numpy(), fc.grad.cpu().numpy(), float(loss.detach())

    g_mixed, gf_mixed, loss_mixed = grads("mixed")
    g_fp64, gf_fp64, loss_fp64 = grads("fp64")
    assert abs(loss_mixed - loss_fp64) <= 1e-5 * loss_fp64
    assert _rel(g_mixed, g_fp64) <= 1e-4
    assert _rel(gf_mixed, gf_fp64) <= 1e-4

    # central FD of the oracle chain (the reference's CPU algorithm), one node
    # at a time (exact by linearity: moving node i changes its induced current
    # and its far-field term only)
    disp = d7.copy()
    disp[:3] += c["delta"][None, :] * d7[3:6]
    jd = oracle_mod.run("JM", f7, fcur, *fg, disp, k)
    base = oracle_mod.run("FF", disp, jd, *dg, ff7, k)

    def one(i, pos):
        p7 = disp[:, i:i + 1].copy()
        p7[:3, 0] = pos
        ji = oracle_mod.run("JM", f7, fcur, *fg, p7, k, nthreads=1)
        s1 = p7.copy()
        s1[6, 0] = d7[6, i] * _trap_weight(i, *dg)
        return oracle_mod.run("FF", s1, ji, -1, 0, 0, ff7, k)

    def loss_at(i, pos):
        e = base - one(i, disp[:3, i]) + one(i, pos)
        return float(((e[0:6] - ideal[0:6]) ** 2).sum())

    h = 1e-6 * lam
    nodes = np.random.default_rng(2).choice(nd, 64, replace=False)
    fd = np.array([(loss_at(i, disp[:3, i] + h * d7[3:6, i]) - loss_at(i, disp[:3, i] - h * d7[3:6, i])) / (2 * h)
                   for i in nodes])
    assert _rel(g_mixed[nodes], fd) <= 1e-4, np.c_[g_mixed[nodes], fd][:8]
    assert _rel(g_fp64[nodes], fd) <= 1e-6


def test_cassegrain_chain_against_fp64(cuda, lib):
    """feed -> hyperboloid (JM) -> paraboloid (JM) -> far field on reduced grids:
    the mixed chain and its displacement gradients against the FP64 chain."""
    import torch
    from pypo_gb300 import autograd as A, configs
    c = configs.cassegrain(scale=0.2)
    dev = cuda
    T = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    k = c["k"]
    ref_ff = None
    out = {}
    for precision in ("fp64", "mixed"):
        ds = torch.zeros(c["sec7"].shape[1], dtype=torch.float64, device=dev, requires_grad=True)
        dp = torch.zeros(c["prim7"].shape[1], dtype=torch.float64, device=dev, requires_grad=True)
        j1 = A.propagate("JM", T(c["feed7"]), T(c["feed_cur"]), *c["feed_grid"], T(c["sec7"]), k, dt=ds,
                         precision=precision)
        j2 = A.propagate("JM", T(c["sec7"]), j1, *c["sec_grid"], T(c["prim7"]), k, ds=ds, dt=dp,
                         precision=precision)
        ff = A.propagate("FF", T(c["prim7"]), j2, *c["prim_grid"], T(c["ff7"]), k, ds=dp, precision=precision)
        if ref_ff is None:
            ref_ff = ff.detach().clone()
        loss = (ff[0:6] * ref_ff[0:6]).sum()
        loss.backward()
        out[precision] = (ff.detach().cpu().numpy(), ds.grad.cpu().numpy(), dp.grad.cpu().numpy())
    e, p = errors(out["mixed"][0], out["fp64"][0], "FF")
    assert e <= REL_L2_TOL and p <= PHASE_TOL, (e, p)
    assert _rel(out["mixed"][1], out["fp64"][1]) <= 1e-4
    assert _rel(out["mixed"][2], out["fp64"][2]) <= 1e-4


def test_cassegrain_full_size_stage_by_stage(cuda, lib, oracle_mod):
    """The Cassegrain chain at full size (feed 201^2 -> hyperboloid 401^2 ->
    paraboloid 1001^2 -> far field 201^2, 2.1e11 pairs): every stage's mixed
    output, from the previous stage's mixed output, against the plain FP64 GPU
    sum of the same inputs on 2 % of its targets and against the oracle on 16.
    The stages are linear, so the chain's error is bounded by theirs."""
    from pypo_gb300 import configs, engine
    c = configs.cassegrain()
    k = c["k"]
    rng = np.random.default_rng(5)
    stages = [("JM", "feed7", "feed_grid", "sec7"), ("JM", "sec7", "sec_grid", "prim7"),
              ("FF", "prim7", "prim_grid", "ff7")]
    cur = c["feed_cur"]
    for mode, sk, gk, tk in stages:
        src, tgt, grid = c[sk], c[tk], c[gk]
        out = engine.propagate(mode, src, cur, *grid, tgt, k)
        nt = tgt.shape[1]
        idx = np.sort(rng.choice(nt, size=max(16, nt // 50), replace=False))
        ref = engine.propagate(mode, src, cur, *grid, np.ascontiguousarray(tgt[:, idx]), k, precision="fp64")
        e, p = errors(out[:, idx], ref, mode)
        assert e <= REL_L2_TOL and p <= PHASE_TOL, (sk, tk, e, p)
        sub = np.sort(rng.choice(nt, size=16, replace=False))
        oref = oracle_mod.run(mode, src, cur, *grid, tgt, k, tidx=sub)
        e2, _ = errors(out[:, sub], oref, mode)
        assert e2 <= REL_L2_TOL, (sk, tk, e2)
        cur = out


@pytest.mark.parametrize("name", ["dish_eh", "dish_ff"])
def test_full_size_superposition(cuda, lib, name):
    """At full size, a size-independent property of the integral: it is
    linear in the currents, so out(J1 + c J2) = out(J1) + c out(J2) for a
    complex c, to FP32 rounding of the sums; the adjoint's current gradient
    is linear in the cotangent the same way."""
    import torch
    from pypo_gb300 import configs, engine
    w = getattr(configs, name)()
    dev = cuda
    s7, t7 = (torch.tensor(w[k], device=dev) for k in ("s7", "t7"))
    grid = (w["gmode"], w["ncx"], w["ncy"])
    rng = np.random.default_rng(11)
    j1 = torch.tensor(w["cur"], device=dev)
    j2 = torch.tensor(rng.standard_normal(w["cur"].shape) * np.abs(w["cur"]).max(), device=dev)
    j2[6:] = 0.0
    c = complex(0.6, -1.3)

    def cmul(x):   # c times a current block (rows: re xyz, im xyz per group)
        y = torch.empty_like(x)
        for g in range(2):
            re, im = x[6 * g:6 * g + 3], x[6 * g + 3:6 * g + 6]
            y[6 * g:6 * g + 3] = c.real * re - c.imag * im
            y[6 * g + 3:6 * g + 6] = c.real * im + c.imag * re
        return y
    run = lambda j: engine.propagate_dev(w["mode"], s7, j, *grid, t7, w["k"], m_zero=True)
    lhs = run(j1 + cmul(j2))
    rhs = run(j1) + cmul(run(j2))
    assert float(torch.linalg.norm(lhs - rhs) / torch.linalg.norm(rhs)) <= 2e-6
    nt = t7.shape[1]
    cot1 = torch.tensor(rng.standard_normal((12, nt)), device=dev)
    cot2 = torch.tensor(rng.standard_normal((12, nt)), device=dev)

    def grad(cot):
        gc = torch.empty_like(j1)
        engine.adjoint_dev(w["mode"], s7, j1, *grid, t7, w["k"], cot, m_zero=True, grad_cur=gc)
        return gc
    g = grad(cot1 + 0.7 * cot2)
    ref = grad(cot1) + 0.7 * grad(cot2)
    assert float(torch.linalg.norm(g - ref) / torch.linalg.norm(ref)) <= 2e-6


@pytest.mark.parametrize("mode", ["JMEH", "EHP"])
def test_dish_eh_other_modes_full_size_sampled(cuda, lib, mode):
    """The dish_eh configuration at full size in the other near-field modes:
    JMEH (PEC currents and fields in one call) and EHP (the reflected field
    from the normalised Poynting vector, nonlinear in E and H). Against the
    plain FP64 GPU sum on a 1 % target sample."""
    import torch
    from pypo_gb300 import configs, engine
    w = configs.dish_eh()
    dev = cuda
    s7, cur = (torch.tensor(w[k], device=dev) for k in ("s7", "cur"))
    t7n = w["t7"].copy()
    t7n[3:6] = [[0.0], [0.0], [-1.0]]   # the focal plane's normal faces the dish (JM, EHP use it)
    t7 = torch.tensor(t7n, device=dev)
    grid = (w["gmode"], w["ncx"], w["ncy"])
    got = engine.propagate_dev(mode, s7, cur, *grid, t7, w["k"], m_zero=True).cpu().numpy()
    idx = np.sort(np.random.default_rng(13).choice(t7n.shape[1], size=t7n.shape[1] // 100, replace=False))
    ts = torch.tensor(np.ascontiguousarray(t7n[:, idx]), device=dev)
    ref = engine.propagate_dev(mode, s7, cur, *grid, ts, w["k"], precision="fp64").cpu().numpy()
    e, p = errors(got[:, idx], ref, mode)
    assert e <= REL_L2_TOL and p <= PHASE_TOL, (mode, e, p)
