"""GPU adjoint: gradients of a real loss of the outputs with respect to the
source currents and to normal-direction displacements of source and target
points, checked against central finite differences of the FP64 oracle
(forward restatement of the reference) and against the plain FP64 GPU
adjoint. The bar: 1e-4 relative to the finite differences (mixed), 1e-6
(FP64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(rng, mode):
    from pypo_gb300 import engine, surfaces as SF
    src = SF.paraboloid(3.0, [9, 10], gmode=1, lims_a=[0.2, 2.0])
    s7 = engine.generate_grid(src)
    if mode == "FF":
        t7 = engine.generate_grid(SF.farfield([6, 5], [-20, 20], [-15, 15]))
    else:
        t7 = engine.generate_grid(SF.translate(SF.plane([6, 5], gmode=0, lims_a=[-1, 1]), dz=3.0))
        t7[3:6] *= -1.0
    cur = rng.standard_normal((2 if mode == "scalar" else 12, s7.shape[1]))
    cot = rng.standard_normal((engine.n_out(mode), t7.shape[1]))
    return s7, cur, t7, cot, (1, 9, 10)


def _loss(oracle_mod, mode, s7, cur, t7, cot, grid, k, t):
    out = oracle_mod.run(mode, s7, cur, grid[0], grid[1], grid[2], t7, k, 1.0, t)
    return float((cot * out).sum())


def _fd(oracle_mod, mode, s7, cur, t7, cot, grid, k, t, rng, nsamp=6):
    """Central FD of the oracle loss: current entries, source and target displacements."""
    f = lambda s, c, tt: _loss(oracle_mod, mode, s, c, tt, cot, grid, k, t)
    h_c, h_d = 1e-3, 1e-6 * (2 * np.pi / k)
    rows = rng.integers(0, cur.shape[0], nsamp)
    cols = rng.integers(0, s7.shape[1], nsamp)
    fc = []
    for r, c in zip(rows, cols):
        cp, cm = cur.copy(), cur.copy()
        cp[r, c] += h_c
        cm[r, c] -= h_c
        fc.append((f(s7, cp, t7) - f(s7, cm, t7)) / (2 * h_c))
    si = rng.choice(s7.shape[1], nsamp, replace=False)
    fs = []
    for i in si:
        sp, sm = s7.copy(), s7.copy()
        sp[:3, i] += h_d * s7[3:6, i]
        sm[:3, i] -= h_d * s7[3:6, i]
        fs.append((f(sp, cur, t7) - f(sm, cur, t7)) / (2 * h_d))
    ti = rng.choice(t7.shape[1], nsamp, replace=False)
    ft = []
    if mode != "FF":
        for j in ti:
            tp, tm = t7.copy(), t7.copy()
            tp[:3, j] += h_d * t7[3:6, j]
            tm[:3, j] -= h_d * t7[3:6, j]
            ft.append((f(s7, cur, tp) - f(s7, cur, tm)) / (2 * h_d))
    return (rows, cols, np.array(fc)), (si, np.array(fs)), (ti, np.array(ft))


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("mode", ["EH", "JM", "JMEH", "FF", "scalar"])
@pytest.mark.parametrize("t", [-1.0, 1.0])
def test_adjoint_matches_finite_differences(cuda, lib, oracle_mod, mode, t):
    from pypo_gb300 import engine
    rng = np.random.default_rng({"EH": 10, "JM": 20, "JMEH": 30, "FF": 40, "scalar": 50}[mode] + (t > 0))
    s7, cur, t7, cot, grid = _case(rng, mode)
    k = 2 * np.pi / 0.9
    (rows, cols, fc), (si, fs), (ti, ft) = _fd(oracle_mod, mode, s7, cur, t7, cot, grid, k, t, rng)
    for prec, tol in (("mixed", 1e-4), ("fp64", 1e-6)):
        g = engine.adjoint(mode, s7, cur, *grid, t7, k, cot, 1.0, t, prec)
        assert _rel(g["cur"][rows, cols], fc) <= tol, (prec, "cur", g["cur"][rows, cols], fc)
        assert _rel(g["ds"][si], fs) <= tol, (prec, "ds", g["ds"][si], fs)
        if mode != "FF":
            assert _rel(g["dt"][ti], ft) <= tol, (prec, "dt", g["dt"][ti], ft)


def test_mixed_adjoint_matches_fp64_adjoint_at_scale(cuda, lib):
    """A reduced dish_eh (kR ~ 3e3 rad): the mixed adjoint against the FP64 one."""
    from pypo_gb300 import configs, engine
    w = configs.dish_eh(scale=0.12)
    rng = np.random.default_rng(4)
    cot = rng.standard_normal((12, w["t7"].shape[1]))
    args = (w["mode"], w["s7"], w["cur"], w["gmode"], w["ncx"], w["ncy"], w["t7"], w["k"], cot)
    gm = engine.adjoint(*args, precision="mixed")
    gd = engine.adjoint(*args, precision="fp64")
    assert _rel(gm["cur"], gd["cur"]) <= 1e-5
    assert _rel(gm["ds"], gd["ds"]) <= 1e-4
    assert _rel(gm["dt"], gd["dt"]) <= 1e-4


def test_autograd_chain_feed_dish_farfield(cuda, lib, oracle_mod):
    """feed plane --JM--> dish --FF--> far field; loss sum |E_ff - E_ideal|^2 with
    E_ideal the unperturbed result. Gradients with respect to the feed currents
    and the dish's normal displacement against FD of the oracle chain."""
    import torch
    from pypo_gb300 import autograd as A, beams, engine, surfaces as SF
    lam = 2.0
    k = 2 * np.pi / lam
    feed = SF.plane([9, 9], gmode=0, lims_a=[-6, 6])
    f7 = engine.generate_grid(feed)
    _, fcur = beams.gauss_beam(f7, lam, 4.0, 0.0, 1.0)
    # dish opening downwards with its focus on the feed: the reflected beam goes to -z
    dish = SF.translate(SF.rotate_x(SF.paraboloid(40.0, [10, 12], gmode=1, lims_a=[0, 30]), 180.0), dz=40.0)
    d7 = engine.generate_grid(dish)
    aoe = engine.generate_grid(SF.farfield([5, 5], [-10, 10], [-10, 10]))
    ff7 = aoe.copy()
    ff7[0] = np.pi - aoe[0]          # polar angles around -z
    dev = cuda
    T = lambda a: torch.tensor(a, device=dev)
    fcur_t = T(fcur).requires_grad_(True)
    dd = torch.zeros(d7.shape[1], dtype=torch.float64, device=dev, requires_grad=True)
    jm = A.propagate("JM", T(f7), fcur_t, 0, 9, 9, T(d7), k, dt=dd)
    ff = A.propagate("FF", T(d7), jm, 1, 10, 12, T(ff7), k, ds=dd)
    ideal = torch.tensor(oracle_mod.run("FF", d7, oracle_mod.run("JM", f7, fcur, 0, 9, 9, d7, k), 1, 10, 12, ff7, k),
                         device=dev)
    # perturb the dish a little so that the loss is not at its minimum
    rng = np.random.default_rng(0)
    pert = rng.normal(0, lam / 40, d7.shape[1])
    with torch.no_grad():
        dd.copy_(T(pert))
    jm = A.propagate("JM", T(f7), fcur_t, 0, 9, 9, T(d7), k, dt=dd)
    ff = A.propagate("FF", T(d7), jm, 1, 10, 12, T(ff7), k, ds=dd)
    loss = ((ff - ideal) ** 2).sum()
    loss.backward()
    g_dd = dd.grad.cpu().numpy()
    g_cur = fcur_t.grad.cpu().numpy()

    def chain_loss(disp, c):
        dm = d7.copy()
        dm[:3] += disp[None, :] * d7[3:6]
        j = oracle_mod.run("JM", f7, c, 0, 9, 9, dm, k)
        o = oracle_mod.run("FF", dm, j, 1, 10, 12, ff7, k)
        return float(((o - ideal.cpu().numpy()) ** 2).sum())

    h = 1e-6 * lam
    nodes = rng.choice(d7.shape[1], 8, replace=False)
    fd = []
    for i in nodes:
        p, m = pert.copy(), pert.copy()
        p[i] += h
        m[i] -= h
        fd.append((chain_loss(p, fcur) - chain_loss(m, fcur)) / (2 * h))
    assert _rel(g_dd[nodes], np.array(fd)) <= 1e-4, (g_dd[nodes], fd)
    ent = [(0, 10), (3, 40), (7, 22)]
    fdc = []
    for r, c in ent:
        cp, cm = fcur.copy(), fcur.copy()
        cp[r, c] += 1e-3
        cm[r, c] -= 1e-3
        fdc.append((chain_loss(pert, cp) - chain_loss(pert, cm)) / 2e-3)
    assert _rel(np.array([g_cur[r, c] for r, c in ent]), np.array(fdc)) <= 1e-4


@pytest.mark.parametrize("mode", ["EH", "JMEH", "FF"])
def test_adjoint_odd_counts_and_padding(cuda, lib, mode):
    """Odd source and target counts (a padded lane in the last source pair and
    target pair of the packed kernels), M != 0, against the FP64 adjoint."""
    from pypo_gb300 import engine, surfaces as SF
    rng = np.random.default_rng(77)
    s7 = engine.generate_grid(SF.paraboloid(3.0, [9, 11], gmode=1, lims_a=[0.2, 2.0]))   # 99 sources
    if mode == "FF":
        t7 = engine.generate_grid(SF.farfield([7, 5], [-20, 20], [-15, 15]))            # 35 directions
    else:
        t7 = engine.generate_grid(SF.translate(SF.plane([7, 5], gmode=0, lims_a=[-1, 1]), dz=3.0))
        t7[3:6] *= -1.0
    cur = rng.standard_normal((12, s7.shape[1]))
    cot = rng.standard_normal((engine.n_out(mode), t7.shape[1]))
    args = (mode, s7, cur, 1, 9, 11, t7, 2 * np.pi / 0.9, cot)
    gm = engine.adjoint(*args, precision="mixed")
    gd = engine.adjoint(*args, precision="fp64")
    assert _rel(gm["cur"], gd["cur"]) <= 1e-5
    assert _rel(gm["ds"], gd["ds"]) <= 1e-4
    if mode != "FF":
        assert _rel(gm["dt"], gd["dt"]) <= 1e-4


def test_adjoint_many_chunks_and_determinism(cuda, lib):
    """Many more targets than one source block streams (several target chunks,
    atomic target-side sums across source blocks): against the FP64 adjoint,
    and two runs agree (bitwise except the atomically summed target side)."""
    from pypo_gb300 import engine, surfaces as SF
    rng = np.random.default_rng(5)
    s7 = engine.generate_grid(SF.paraboloid(20.0, [31, 29], gmode=1, lims_a=[0.5, 15.0]))   # 899 sources
    t7 = engine.generate_grid(SF.translate(SF.plane([67, 61], gmode=0, lims_a=[-4, 4]), dz=20.0))   # 4087
    t7[3:6] *= -1.0
    cur = rng.standard_normal((12, s7.shape[1]))
    cot = rng.standard_normal((12, t7.shape[1]))
    args = ("EH", s7, cur, 1, 31, 29, t7, 2 * np.pi / 1.3, cot)
    g1 = engine.adjoint(*args, precision="mixed")
    g2 = engine.adjoint(*args, precision="mixed")
    gd = engine.adjoint(*args, precision="fp64")
    assert np.array_equal(g1["cur"], g2["cur"]) and np.array_equal(g1["ds"], g2["ds"])
    assert _rel(g1["dt"], g2["dt"]) <= 1e-14
    assert _rel(g1["cur"], gd["cur"]) <= 1e-5
    assert _rel(g1["ds"], gd["ds"]) <= 1e-4
    assert _rel(g1["dt"], gd["dt"]) <= 1e-4


def test_adjoint_with_no_targets_or_no_sources(cuda, lib):
    """No targets: every gradient is zero. No sources: the target gradient is
    zero and the source gradients are empty."""
    from pypo_gb300 import engine, surfaces as SF
    rng = np.random.default_rng(4)
    s7 = engine.generate_grid(SF.paraboloid(3.0, [5, 6], gmode=1, lims_a=[0.2, 2.0]))
    cur = rng.standard_normal((12, s7.shape[1]))
    t7 = engine.generate_grid(SF.translate(SF.plane([4, 3], gmode=0, lims_a=[-1, 1]), dz=3.0))
    for mode in ("EH", "FF"):
        for prec in ("mixed", "fp64"):
            g = engine.adjoint(mode, s7, cur, 1, 5, 6, np.zeros((7, 0)), 3.0,
                               np.zeros((engine.n_out(mode), 0)), precision=prec)
            assert np.all(g["cur"] == 0) and np.all(g["ds"] == 0) and g["cur"].shape == (12, 30)
            if mode != "FF":
                g = engine.adjoint(mode, np.zeros((7, 0)), np.zeros((12, 0)), -1, 0, 0, t7, 3.0,
                                   rng.standard_normal((12, t7.shape[1])), precision=prec)
                assert g["cur"].shape == (12, 0) and g["ds"].shape == (0,) and np.all(g["dt"] == 0)


def test_empty_adjoints_write_their_zeros(cuda, lib):
    """Device buffers the caller hands in hold whatever was there before:
    the empty cases must write their zero gradients, not leave the buffers
    alone (a recycled allocation is not zero)."""
    import torch
    from pypo_gb300 import engine, surfaces as SF
    rng = np.random.default_rng(5)
    s7 = torch.tensor(engine.generate_grid(SF.paraboloid(3.0, [5, 6], gmode=1, lims_a=[0.2, 2.0])), device=cuda)
    t7 = torch.tensor(engine.generate_grid(SF.translate(SF.plane([4, 3], gmode=0, lims_a=[-1, 1]), dz=3.0)),
                      device=cuda)
    nan = lambda *shape: torch.full(shape, float("nan"), dtype=torch.float64, device=cuda)
    cur = torch.tensor(rng.standard_normal((12, 30)), device=cuda)
    for prec in ("mixed", "fp64"):
        # no targets: the source gradients are zero
        gc, gs, _ = engine.adjoint_dev("EH", s7, cur, 1, 5, 6, t7[:, :0].contiguous(), 3.0,
                                       nan(12, 0), precision=prec, grad_cur=nan(12, 30), grad_ds=nan(30))
        torch.cuda.synchronize()
        assert torch.all(gc == 0) and torch.all(gs == 0), prec
        # no sources: the target gradient is zero
        _, _, gt = engine.adjoint_dev("EH", s7[:, :0].contiguous(), cur[:, :0].contiguous(), -1, 0, 0, t7, 3.0,
                                      torch.tensor(rng.standard_normal((12, 12)), device=cuda), precision=prec,
                                      grad_dt=nan(12))
        torch.cuda.synchronize()
        assert torch.all(gt == 0), prec


@pytest.mark.parametrize("mode", ["EH", "JM", "JMEH", "FF", "scalar"])
@pytest.mark.parametrize("t", [-1.0, 1.0])
def test_adjoint_matches_oracle_adjoint(cuda, lib, oracle_mod, mode, t):
    """Every gradient, every source and target, against the oracle's FP64
    adjoint: mixed within 1e-5, FP64 within 1e-10 (relative L2)."""
    from pypo_gb300 import engine
    rng = np.random.default_rng({"EH": 11, "JM": 21, "JMEH": 31, "FF": 41, "scalar": 51}[mode] + (t > 0))
    s7, cur, t7, cot, grid = _case(rng, mode)
    k = 2 * np.pi / 0.9
    ref = oracle_mod.adjoint(mode, s7, cur, *grid, t7, k, cot, 1.0, t)
    for prec, tol in (("mixed", 1e-5), ("fp64", 1e-10)):
        g = engine.adjoint(mode, s7, cur, *grid, t7, k, cot, 1.0, t, prec)
        for name, want in ref.items():
            assert _rel(g[name], want) <= tol, (prec, name, _rel(g[name], want))


@pytest.mark.parametrize("t", [-1.0, 1.0])
def test_ehp_adjoint_matches_finite_differences(cuda, lib, oracle_mod, t):
    """EHP (nonlinear in the target's fields): the FP64 adjoint against
    central differences of the oracle (1e-4, the differences' own truncation
    at this nonlinearity), the mixed adjoint against the FP64 one (1e-5)."""
    from pypo_gb300 import engine
    rng = np.random.default_rng(60 + (t > 0))
    s7, cur, t7, cot, grid = _case(rng, "EHP")
    k = 2 * np.pi / 0.9
    (rows, cols, fc), (si, fs), (ti, ft) = _fd(oracle_mod, "EHP", s7, cur, t7, cot, grid, k, t, rng)
    gd = engine.adjoint("EHP", s7, cur, *grid, t7, k, cot, 1.0, t, "fp64")
    assert _rel(gd["cur"][rows, cols], fc) <= 1e-4, (gd["cur"][rows, cols], fc)
    assert _rel(gd["ds"][si], fs) <= 1e-4, (gd["ds"][si], fs)
    assert _rel(gd["dt"][ti], ft) <= 1e-4, (gd["dt"][ti], ft)
    gm = engine.adjoint("EHP", s7, cur, *grid, t7, k, cot, 1.0, t, "mixed")
    for name in ("cur", "ds", "dt"):
        assert _rel(gm[name], gd[name]) <= 1e-5, (name, _rel(gm[name], gd[name]))


def test_scalar_and_ehp_through_autograd(cuda, lib):
    """The autograd function covers the scalar and EHP modes: its gradients
    equal the C-ABI adjoint's."""
    import torch
    from pypo_gb300 import autograd as A, engine
    rng = np.random.default_rng(70)
    for mode in ("scalar", "EHP"):
        s7, cur, t7, cot, grid = _case(rng, mode)
        k = 2 * np.pi / 0.9
        T = lambda a: torch.tensor(a, device=cuda)
        c = T(cur).requires_grad_(True)
        ds = torch.zeros(s7.shape[1], dtype=torch.float64, device=cuda, requires_grad=True)
        dt = torch.zeros(t7.shape[1], dtype=torch.float64, device=cuda, requires_grad=True)
        out = A.propagate(mode, T(s7), c, *grid, T(t7), k, ds=ds, dt=dt)
        (out * T(cot)).sum().backward()
        g = engine.adjoint(mode, s7, cur, *grid, t7, k, cot)
        assert _rel(c.grad.cpu().numpy(), g["cur"]) <= 1e-12
        assert _rel(ds.grad.cpu().numpy(), g["ds"]) <= 1e-12
        assert _rel(dt.grad.cpu().numpy(), g["dt"]) <= 1e-12
