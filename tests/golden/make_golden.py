"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own FP64 CPU library (oracle/_ref/libpypo_ref.so,
compiled from the reference sources by oracle/build_ref.sh) on small seeded
cases shaped like the reference's test templates (reference
tests/TestTemplates.py: 13x13 / 13x12 grids, xy, uv and AoE): every PO mode
in both time directions, the grid generator for every surface type, and the
vector Gaussian feed (makeGaussBeam). Outputs go to golden_*.npz beside this
script. Needs the reference sources (this container); the fixtures then
travel without them.

Usage: python tests/golden/make_golden.py [--only-calcjm | --only-eff | --only-fitgauss | --only-converge |
       --only-highkr]
The reference checkout is read from $PYPO_REFERENCE (default /root/reference).
"""
import json
import os
import pathlib
import subprocess
import sys

import numpy as np

REFERENCE = pathlib.Path(os.environ.get("PYPO_REFERENCE", "/root/reference"))

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from pypo_gb300 import surfaces as SF  # noqa: E402


def dict_to_json(d):
    return json.dumps({k: (np.asarray(v).tolist() if isinstance(v, np.ndarray) else v) for k, v in d.items()})


def cases():
    par_uv = SF.paraboloid(0.25, [13, 12], gmode=1, lims_a=[0, 1])          # coeffs (1, 1), as the templates
    par_xy = SF.paraboloid(0.25, [13, 13], gmode=0, lims_a=[-1, 1])
    pl_tgt = SF.translate(SF.plane([13, 13], gmode=0, lims_a=[-1.5, 1.5]), dz=2.5)
    # Off-dyadic target: no source-target pair is tangent in exact arithmetic.
    pl_off = SF.translate(SF.plane([13, 13], gmode=0, lims_a=[-1.45, 1.45]), dz=2.45)
    hyp = SF.hyperboloid(2.0, 2.0, 3.0, [11, 10], gmode=1, lims_a=[0, 1.5])
    ell = SF.translate(SF.ellipsoid(3.0, 3.0, 5.0, [9, 11], gmode=0, lims_a=[-1, 1]), dz=8.0)
    ell = dict(ell, flip=True)
    ff = SF.farfield([11, 9], [-8, 8], [-6, 6])
    return [
        ("paruv_to_plane", par_uv, pl_tgt, ["JM", "EH", "JMEH", "EHP", "scalar"]),
        ("parxy_to_plane", par_xy, pl_off, ["EH", "JMEH"]),
        # Dyadic grids: 36 pairs are exactly tangent (n . d == 0); the reference
        # skips the ones whose rounded n . R_hat comes out negative.
        ("tangent", par_xy, pl_tgt, ["EH"]),
        ("paruv_to_ff", par_uv, ff, ["FF"]),
        ("hyp_to_ell", hyp, ell, ["JM", "EH", "EHP"]),
    ]


def calcjm(ref):
    """Reference calcCurrents on a rotated, shifted uv paraboloid with seeded
    random fields, every mode (0 full, 1 PMC, 2 PEC, 3 source)."""
    surf = SF.translate(SF.rotate_x(SF.paraboloid(0.4, [9, 8], gmode=1, lims_a=[0.1, 1.2]), 30.0), dz=0.5)
    n = int(np.prod(surf["gridsize"]))
    fields = np.random.default_rng(4242).standard_normal((12, n))
    out = {"surface_json": dict_to_json(surf), "fields": fields}
    for mode in range(4):
        out[f"currents{mode}"] = ref.calc_currents(fields, surf, mode)
    np.savez_compressed(HERE / "golden_calcjm.npz", **out)
    print("wrote calcjm")


def efficiencies(ref):
    """The reference's own Efficiencies.py (calcSpillover, calcTaper,
    calcXpol, calcMainBeam) on a seeded aperture field, with its grid binding
    served by the reference's compiled generateGrid."""
    sys.path.insert(0, str(REFERENCE / "src"))
    import PyPO.Efficiencies as E
    from PyPO.Enums import AperShapes

    class Grid:
        pass

    def generate(refl, transform=True, spheric=True):
        b = ref.grid(refl, transform, spheric)
        g = Grid()
        g.x, g.y, g.z, g.area = b[0], b[1], b[2], b[6]
        return g

    E.BRefl.generateGrid = generate
    surf = SF.plane([41, 37], gmode=0, lims_a=[-20.0, 20.0])
    b = ref.grid(surf)
    rng = np.random.default_rng(909)
    amp = np.exp(-(b[0] ** 2 + (1.3 * b[1]) ** 2) / (2 * 6.0 ** 2))
    co = amp * np.exp(1j * rng.normal(0, 0.3, amp.size))
    xp = 0.05 * amp * np.exp(1j * rng.uniform(0, 2 * np.pi, amp.size))
    fit = np.exp(-(b[0] ** 2 + b[1] ** 2) / (2 * 5.5 ** 2)).astype(complex)
    ell = {"shape": AperShapes.ELL, "center": np.array([1.0, -0.5]), "outer": np.array([12.0, 9.0]),
           "inner": np.array([0.0, 0.0])}
    rect = {"shape": AperShapes.RECT, "center": np.array([0.5, 0.0]), "outer_x": np.array([-10.0, 12.0]),
            "outer_y": np.array([-8.0, 7.0]), "inner_x": np.array([0.0, 0.0]), "inner_y": np.array([0.0, 0.0])}
    out = {"surface_json": dict_to_json(surf), "co": co, "xp": xp, "fit": fit,
           "ell": np.r_[ell["center"], ell["outer"], ell["inner"]],
           "rect": np.r_[rect["center"], rect["outer_x"], rect["outer_y"]],
           "spill_ell": E.calcSpillover(co, surf, ell), "spill_rect": E.calcSpillover(co, surf, rect),
           "taper_ell": E.calcTaper(co, surf, ell), "taper_rect": E.calcTaper(co, surf, rect),
           "taper_all": E.calcTaper(co, surf, None), "xpol": E.calcXpol(co, xp),
           "mainbeam": E.calcMainBeam(co, surf, fit)}
    np.savez_compressed(HERE / "golden_eff.npz", **out)
    print("wrote efficiencies", {k: v for k, v in out.items() if np.ndim(v) == 0 and not isinstance(v, str)})


def fitgauss(ref):
    """The reference's own FitGauss.fitGaussAbs (and System.calcMainBeam's use
    of it) on seeded beam patterns, with its grid binding served by the
    reference's compiled generateGrid (reshaped to the grid, as its binding
    returns it). Cases: an offset rotated Gaussian with phase noise on the
    reference's 13x13 test plane; a centred one at the reference test's
    -100 dB threshold; an elliptical Airy pattern on a 61x61 far-field grid;
    a peak narrower than the grid spacing (empty fit window, the fallback to
    grid row 1) on an xy grid and on a uv grid. Error cases are recorded as expectations: the offset
    Gaussian at -100 dB (IndexError in the reference) and the narrow peak
    with a ratio (the reference's ratio loop never ends)."""
    import signal
    from scipy.special import j1
    sys.path.insert(0, str(REFERENCE / "src"))
    import PyPO.Efficiencies as E
    import PyPO.FitGauss as FG
    from PyPO.Enums import Scales

    class Grid:
        pass

    def generate(refl, transform=True, spheric=True):
        b = ref.grid(refl, transform, spheric)
        shp = tuple(int(v) for v in refl["gridsize"])
        g = Grid()
        g.x, g.y, g.z, g.area = (b[k].reshape(shp) for k in (0, 1, 2, 6))
        return g

    FG.BRefl.generateGrid = generate

    def beam(g, xs, ys, wx, wy, th, kind):
        c, s = np.cos(th), np.sin(th)
        u = ((g.x - xs) * c + (g.y - ys) * s) / wx
        v = (-(g.x - xs) * s + (g.y - ys) * c) / wy
        r = np.sqrt(u * u + v * v)
        if kind == "gauss":
            return np.exp(-r * r / 2)
        r = np.where(r == 0, 1e-30, r)
        return np.abs(2 * j1(r) / r)

    rng = np.random.default_rng(5)
    pl13 = SF.plane([13, 13], gmode=0, lims_a=[-1.0, 1.0])
    g13 = generate(pl13, False, False)
    gauss_xy = beam(g13, 0.1, -0.15, 0.35, 0.25, 0.4, "gauss") * np.exp(1j * rng.normal(0, 0.2, g13.x.shape)) \
        + 1e-3 * rng.standard_normal(g13.x.shape)
    centred = beam(g13, 0.0, 0.0, 0.3, 0.4, 0.0, "gauss").astype(complex)
    ff = SF.farfield([61, 61], [-0.5, 0.5], [-0.5, 0.5])
    gff = generate(ff, False, False)
    airy = beam(gff, 0.03, -0.02, 0.045, 0.06, 0.3, "airy") * np.exp(1j * rng.normal(0, 0.1, gff.x.shape))
    pl15 = SF.plane([15, 15], gmode=0, lims_a=[-1.0, 1.0])
    narrow = (beam(generate(pl15, False, False), 0.0, 0.0, 0.02, 0.02, 0.0, "gauss") + 0.05).astype(complex)
    # on a uv grid the fallback's row 1 is a ring, where x and y both vary
    uv = SF.plane([15, 16], gmode=1, lims_a=[0.05, 1.0])
    guv = generate(uv, False, False)
    ring = 0.05 + 0.01 * np.cos(3 * np.arctan2(guv.y, guv.x)) + 0.02 * guv.x
    narrow_uv = (ring + np.where((np.arange(guv.x.size) == 9 * 16 + 5).reshape(guv.x.shape), 1.0, 0.0)).astype(complex)

    out = {}
    every = [(sid, t, r) for sid in (0, 2) for t in (-11.0, -25.0) for r in (None, 1.0)]
    # (the centred dB fit at -100 dB with a ratio, and the narrow peak with
    # one, never end in the reference: recorded below, not run)
    runs = [("gauss_xy", pl13, gauss_xy, every),
            ("centred_xy", pl13, centred, [(0, -100.0, None), (0, -100.0, 1.0), (2, -100.0, None)]),
            ("airy_ff", ff, airy, every),
            ("narrow_xy", pl15, narrow, [(0, -11.0, None), (2, -11.0, None)]),
            ("narrow_uv", uv, narrow_uv, [(0, -11.0, None), (2, -11.0, None)])]
    scales = {0: Scales.LIN, 2: Scales.dB}
    for name, surf, field, combos in runs:
        g = generate(surf, False, False)
        out[name + "__surface_json"] = dict_to_json(surf)
        out[name + "__field"] = field
        out[name + "__x"], out[name + "__y"] = g.x, g.y
        for sid, thres, ratio in combos:
            key = f"{name}__s{sid}__t{thres:g}__r{'none' if ratio is None else f'{ratio:g}'}"
            out[key] = FG.fitGaussAbs(np.abs(field), surf, thres, scales[sid], ratio)
    # System.calcMainBeam (System.py:1886-1908): fit at ratio 1, Gaussian in LIN, efficiency
    for scale, sid in ((Scales.LIN, 0), (Scales.dB, 2)):
        popt = FG.fitGaussAbs(np.abs(airy), ff, -11.0, scale, 1)
        psi = FG.generateGauss(popt, ff, scale=Scales.LIN)
        out[f"airy_ff__mainbeam_s{sid}"] = E.calcMainBeam(airy, ff, psi)
    # expected failures
    try:
        FG.fitGaussAbs(np.abs(gauss_xy), pl13, -100.0, Scales.LIN, None)
        raise SystemExit("expected the reference to raise IndexError")
    except IndexError as e:
        out["gauss_xy__t-100__error"] = str(e)

    def _alarm(*_):
        raise TimeoutError

    signal.signal(signal.SIGALRM, _alarm)
    signal.alarm(20)
    try:
        FG.fitGaussAbs(np.abs(narrow), pl15, -11.0, Scales.LIN, 1)
        raise SystemExit("expected the reference's ratio loop not to end")
    except TimeoutError:
        out["narrow_xy__ratio_loop"] = "no end within 20 s (the threshold stops at -3 dB and every round repeats)"
        out["centred_xy__s2__t-100__r1__loop"] = "the same: no end (24,578 rounds in 120 s with oracle/fitgauss.py, which follows it)"
    finally:
        signal.alarm(0)
    np.savez_compressed(HERE / "golden_fitgauss.npz", **out)
    print("wrote fitgauss", len(out), "entries")


def converge(ref):
    """The reference's own System.autoConverge and System.convergeOnTarget
    (System.py:2779-3086) on a Gaussian feed (createGaussian on a 21 x 21
    plane, lambda 2 mm) and a dish facing it (uv or xy grid), with a target
    plane behind the feed (xy or uv). System is imported with its plotting
    modules replaced by mocks (matplotlib is not installed here), and its
    bindings load the reference's library compiled from its sources
    (oracle/build_ref.sh) in place of the libpypocpu / libpyporefl /
    libpypobeam it looks for beside itself. Stores the feed's fields, the
    reflectors' internal dicts and the grid sizes found."""
    import ctypes
    import copy
    import types
    from unittest import mock
    for m in ("matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.colors", "matplotlib.ticker",
              "matplotlib.patches", "matplotlib.collections", "mpl_toolkits", "mpl_toolkits.axes_grid1",
              "mpl_toolkits.mplot3d"):
        sys.modules.setdefault(m, mock.MagicMock())
    sys.path.insert(0, str(REFERENCE / "src"))
    import PyPO.BindBeam as BBeam
    import PyPO.BindCPU as BCPU
    import PyPO.BindRefl as BRefl
    shim = types.ModuleType("ctypes_for_reference")
    shim.__dict__.update(ctypes.__dict__)

    def cdll(path, *a, **k):
        base = pathlib.Path(str(path)).name
        if base.startswith(("libpypo", "pypo")):
            if not base.endswith(".so"):
                raise OSError(base)
            return ctypes.CDLL(str(O.REF_PATH))
        return ctypes.CDLL(path, *a, **k)

    shim.CDLL = cdll
    for mod in (BCPU, BRefl, BBeam):
        mod.ctypes = shim
    from PyPO.System import System

    out = {}
    for dish_mode in ("uv", "xy"):
        for tgt_mode in ("xy", "uv"):
            s = System(verbose=False)
            s.addPlane({"name": "feed", "gmode": "xy", "lims_x": np.array([-15.0, 15.0]),
                        "lims_y": np.array([-15.0, 15.0]), "gridsize": np.array([21, 21])})
            lims = ({"lims_u": np.array([0, 60.0]), "lims_v": np.array([0, 360.0])} if dish_mode == "uv"
                    else {"lims_x": np.array([-60.0, 60.0]), "lims_y": np.array([-60.0, 60.0])})
            s.addParabola(dict(name="dish", pmode="focus", vertex=np.zeros(3), focus_1=np.array([0, 0, 60.0]),
                               gmode=dish_mode, gridsize=np.array([11, 11]), **lims))
            s.rotateGrids("dish", np.array([180.0, 0, 0]))
            s.translateGrids("dish", np.array([0, 0, 60.0]))
            tl = ({"lims_u": np.array([0, 20.0]), "lims_v": np.array([0, 360.0])} if tgt_mode == "uv"
                  else {"lims_x": np.array([-20.0, 20.0]), "lims_y": np.array([-20.0, 20.0])})
            s.addPlane(dict(name="tplane", gmode=tgt_mode, gridsize=np.array([5, 5]), **tl))
            s.translateGrids("tplane", np.array([0, 0, -150.0]))
            s.createGaussian({"name": "gfield", "lam": 2.0, "w0x": 6.0, "w0y": 6.0, "n": 1, "E0": 1.0,
                              "dxyz": 0.0, "pol": np.array([1, 0, 0])}, "feed")
            key = f"{dish_mode}_{tgt_mode}"
            dish0, tpl0 = copy.deepcopy(s.system["dish"]), copy.deepcopy(s.system["tplane"])
            f = s.fields["gfield"]
            blk = np.zeros((12, 441))
            for c, comp in enumerate(("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
                v = np.asarray(getattr(f, comp)).ravel()
                r = c if c < 3 else c + 3
                blk[r], blk[r + 3] = v.real, v.imag
            out[key + "__feed_json"] = dict_to_json(s.system["feed"])
            out[key + "__dish_json"] = dict_to_json(dish0)
            out[key + "__target_json"] = dict_to_json(tpl0)
            out[key + "__fields"] = blk
            out[key + "__k"] = f.k
            out[key + "__auto"] = np.asarray(s.autoConverge("gfield", "dish"))
            s.system["dish"] = copy.deepcopy(dish0)
            out[key + "__on_target"] = np.asarray(s.convergeOnTarget("gfield", "dish", "tplane"))
    np.savez_compressed(HERE / "golden_converge.npz", **out)
    print("wrote converge", {k: v for k, v in out.items() if k.endswith(("__auto", "__on_target"))})


def high_kr(ref):
    """The reference's own CPU library at the benchmark's phase scale: a
    paraboloid f 500 mm, D 200 mm (uv 41 x 40) at lambda 1 mm radiating a
    tapered x-polarised current with phase noise (and a small random M) to
    its focal plane (15 x 15 over +-5 mm; kR ~ 3.2e3 rad: EH, JM, EHP,
    scalar) and to a
    15 x 15 far-field grid over +-1 deg (k r' up to 6e2 rad: FF), both time
    directions."""
    rng = np.random.default_rng(20261204)
    src = SF.paraboloid(500.0, [41, 40], gmode=1, lims_a=[0, 100])
    tgt = SF.translate(SF.plane([15, 15], gmode=0, lims_a=[-5, 5]), dz=500.0)
    ff = SF.farfield([15, 15], [-1, 1], [-1, 1])
    s7 = ref.grid(src)
    r = np.hypot(s7[0], s7[1])
    amp = np.exp(-0.5 * np.log(10) * (r / 100.0) ** 2)
    ph = rng.normal(0.0, 0.05, r.size)
    cur = 1e-3 * rng.standard_normal((12, r.size))
    cur[0] += amp * np.cos(ph)
    cur[3] += amp * np.sin(ph)
    k = 2 * np.pi
    data = {"src_json": dict_to_json(src), "tgt_json": dict_to_json(tgt), "ff_json": dict_to_json(ff), "k": k,
            "epsilon": 1.0, "cur": cur}
    for mode, t_dict in (("EH", tgt), ("JM", tgt), ("EHP", tgt), ("scalar", tgt), ("FF", ff)):
        for t in (-1.0, 1.0):
            c = cur[:2] if mode == "scalar" else cur
            out, sg, tg = ref.propagate(mode, src, t_dict, c, k=k, epsilon=1.0, t_dir=t, nthreads=8)
            data[f"out_{mode}_{'fwd' if t < 0 else 'bwd'}"] = out
            data["ff_grid" if mode == "FF" else "tgt_grid"] = tg
    data["src_grid"] = sg
    np.savez_compressed(HERE / "golden_highkr.npz", **data)
    print("wrote highkr")


def main():
    if not O.REF_PATH.exists():
        subprocess.run([str(ROOT / "oracle" / "build_ref.sh")], check=True)
    ref = O.Reference()
    if "--only-highkr" in sys.argv:
        high_kr(ref)
        return
    if "--only-calcjm" in sys.argv:
        calcjm(ref)
        return
    if "--only-eff" in sys.argv:
        efficiencies(ref)
        return
    if "--only-fitgauss" in sys.argv:
        fitgauss(ref)
        return
    if "--only-converge" in sys.argv:
        converge(ref)
        return
    calcjm(ref)
    efficiencies(ref)
    fitgauss(ref)
    converge(ref)
    high_kr(ref)
    rng = np.random.default_rng(20261203)
    k = 2 * np.pi / 0.7
    for name, src, tgt, modes in cases():
        ns = int(np.prod(src["gridsize"]))
        cur = rng.standard_normal((12, ns))
        data = {"src_json": dict_to_json(src), "tgt_json": dict_to_json(tgt), "k": k, "epsilon": 1.7,
                "cur": cur}
        for mode in modes:
            for t in (-1.0, 1.0):
                c = cur[:2] if mode == "scalar" else cur
                out, sg, tg = ref.propagate(mode, src, tgt, c, k=k, epsilon=1.7, t_dir=t, nthreads=4)
                data[f"out_{mode}_{'fwd' if t < 0 else 'bwd'}"] = out
        data["src_grid"] = sg
        data["tgt_grid"] = tg
        np.savez_compressed(HERE / f"golden_{name}.npz", **data)
        print("wrote", name, modes)

    # Grid generator, every surface type and grid mode.
    grids = {
        "par_xy": SF.paraboloid(0.25, [13, 13], gmode=0, lims_a=[-1, 1]),
        "par_uv": SF.paraboloid(300.0, [11, 12], gmode=1, lims_a=[0, 150], ecc_uv=0.3, rot_uv=20.0,
                                gcenter=np.array([3.0, -2.0])),
        "hyp_xy": SF.hyperboloid(2.0, 3.0, 5.0, [9, 7], gmode=0, lims_a=[-1, 1], lims_b=[-2, 2],
                                 gcenter=np.array([1.0, 2.0])),
        "hyp_uv": SF.hyperboloid(2.0, 3.0, 5.0, [9, 8], gmode=1, lims_a=[0, 1], flip=True),
        "ell_xy": SF.ellipsoid(4.0, 5.0, 6.0, [9, 7], gmode=0, lims_a=[-1, 1]),
        "ell_uv": SF.ellipsoid(4.0, 5.0, 6.0, [9, 8], gmode=1, lims_a=[0, 1], ecc_uv=0.5),
        "pl_xy": SF.rotate_x(SF.translate(SF.plane([7, 9], gmode=0, lims_a=[-3, 3]), 1, 2, 3), 30),
        "pl_uv": SF.plane([7, 9], gmode=1, lims_a=[0, 3]),
        "aoe": SF.farfield([11, 9], [-5, 5], [-4, 4]),
        "par_rms": dict(SF.paraboloid(0.25, [13, 13], gmode=0, lims_a=[-1, 1]), rms=0.01, rms_seed=7),
    }
    gdata = {}
    for name, d in grids.items():
        gdata[f"{name}_json"] = dict_to_json(d)
        gdata[f"{name}_grid"] = ref.grid(d)
    np.savez_compressed(HERE / "golden_grids.npz", **gdata)
    print("wrote grids")

    # Vector Gaussian feed (reference makeGaussBeam), 3 mm, w0 10 mm on a plane.
    plane = SF.plane([21, 21], gmode=0, lims_a=[-50, 50])
    f, c = ref.gauss_beam(lam=3.0, w0=10.0, z=0.0, power=4 * np.pi, plane=plane)
    f2, c2 = ref.gauss_beam(lam=1.0, w0=5.0, z=50.0, power=1.0,
                            plane=SF.plane([15, 15], gmode=0, lims_a=[-20, 20]), mode=2)
    np.savez_compressed(HERE / "golden_gauss.npz", plane_json=dict_to_json(plane), fields=f, currents=c,
                        fields2=f2, currents2=c2)
    print("wrote gauss")


if __name__ == "__main__":
    main()
