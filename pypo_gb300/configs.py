"""Synthetic workloads with the shapes of the engine's benchmark configurations.

Each builder returns a dict: mode, s7 (7, ns), cur (12, ns), gmode, ncx, ncy,
t7 (7, nt), k, pairs, and the reflector dicts. Sizes, wavelengths and
geometry follow the configuration descriptions; the currents are seeded
synthetic illuminations (there is no measured data).

  dish_eh        paraboloid D 1000 mm, f 500 mm, uv 501x501, lambda 1 mm;
                 J: x-polarised, projected tangential to the dish, amplitude
                 exp(-ln(10)/2 (r/R)^2) (-10 dB power at the rim) times
                 exp(j phi), phi ~ N(0, 0.05 rad) (seed 1); M = 0.
                 Target: plane 301x301 over +-50 mm at the focal plane. EH.
  dish_ff        paraboloid D 2000 mm, f 800 mm, uv 1001x1001, lambda 1 mm,
                 currents as dish_eh; far field 401x401 over +-0.5 deg. FF.
"""
import numpy as np

from . import engine
from . import surfaces as SF


def tapered_currents(s7, radius, seed=1, phase_rms=0.05, taper_db=10.0):
    """x-polarised tangential J with a Gaussian power taper and random phase; M = 0."""
    x, y = s7[0], s7[1]
    n = s7[3:6]
    r = np.hypot(x, y)
    amp = np.exp(-0.5 * np.log(10 ** (taper_db / 10)) * (r / radius) ** 2)
    phi = np.random.default_rng(seed).normal(0.0, phase_rms, r.size)
    pol = np.array([1.0, 0.0, 0.0])[:, None]
    jt = pol - (pol * n).sum(0) * n          # tangential projection of x-hat
    c = amp * np.exp(1j * phi)
    J = jt * c
    cur = np.zeros((12, r.size))
    cur[0:3] = J.real
    cur[3:6] = J.imag
    return cur


def dish_eh(scale=1.0):
    """The EH workload; `scale` < 1 shrinks both grids (parity tests)."""
    nsg = max(3, int(round(501 * scale)))
    ntg = max(3, int(round(301 * scale)))
    f, D, lam = 500.0, 1000.0, 1.0
    src = SF.paraboloid(f, [nsg, nsg], gmode=1, lims_a=[0.0, D / 2])
    tgt = SF.translate(SF.plane([ntg, ntg], gmode=0, lims_a=[-50.0, 50.0]), dz=f)
    s7 = engine.generate_grid(src)
    t7 = engine.generate_grid(tgt)
    cur = tapered_currents(s7, D / 2)
    return dict(name="dish_eh", mode="EH", s7=s7, cur=cur, gmode=1, ncx=nsg, ncy=nsg, t7=t7,
                k=2 * np.pi / lam, pairs=s7.shape[1] * t7.shape[1], src=src, tgt=tgt,
                desc=f"paraboloid D{D:.0f} f{f:.0f} uv {nsg}x{nsg} -> focal plane {ntg}x{ntg} "
                     f"+-50 mm, lambda {lam} mm, EH, M=0")


def dish_ff(scale=1.0):
    nsg = max(3, int(round(1001 * scale)))
    ntg = max(3, int(round(401 * scale)))
    f, D, lam = 800.0, 2000.0, 1.0
    src = SF.paraboloid(f, [nsg, nsg], gmode=1, lims_a=[0.0, D / 2])
    tgt = SF.farfield([ntg, ntg], [-0.5, 0.5], [-0.5, 0.5])
    s7 = engine.generate_grid(src)
    t7 = engine.generate_grid(tgt)
    cur = tapered_currents(s7, D / 2)
    return dict(name="dish_ff", mode="FF", s7=s7, cur=cur, gmode=1, ncx=nsg, ncy=nsg, t7=t7,
                k=2 * np.pi / lam, pairs=s7.shape[1] * t7.shape[1], src=src, tgt=tgt,
                desc=f"paraboloid D{D:.0f} f{f:.0f} uv {nsg}x{nsg} -> far field {ntg}x{ntg} "
                     f"+-0.5 deg, lambda {lam} mm, FF, M=0")


WORKLOADS = {"dish_eh": dish_eh, "dish_ff": dish_ff}


# ---------------------------------------------------------------- feeds, chains

def feed_plane(lam, w0, half_width, n, power=4 * np.pi, z_shift=0.0):
    """Vector Gaussian feed (waist on the plane) on an n x n plane over +-half_width,
    then moved by z_shift along z (the currents move with the plane)."""
    from . import beams
    plane = SF.plane([n, n], gmode=0, lims_a=[-half_width, half_width])
    s7 = engine.generate_grid(plane)
    _, cur = beams.gauss_beam(s7, lam, w0, 0.0, power)
    s7[2] += z_shift
    return plane, s7, np.ascontiguousarray(cur)


def dish_facing_feed(f, D, n, gmode=1):
    """Paraboloid with focal length f and aperture D whose focus is at the origin
    and which opens towards -z (vertex at z = f): it faces a feed at the origin."""
    lims = [0.0, D / 2] if gmode == 1 else [-D / 2, D / 2]
    return SF.translate(SF.rotate_x(SF.paraboloid(f, [n, n], gmode=gmode, lims_a=lims), 180.0), dz=f)


def farfield_minus_z(n, half_deg):
    """Far-field (polar, azimuth) grid of n x n directions within +-half_deg of -z."""
    g = engine.generate_grid(SF.farfield([n, n], [-half_deg, half_deg], [-half_deg, half_deg]))
    g[0] = np.pi - g[0]
    return g


def feed_dish_jm(scale=1.0):
    """Gaussian feed (lambda 3 mm, w0 10 mm, 101x101 plane over +-50 mm) radiating
    onto an f 300 mm, D 300 mm paraboloid (uv 101x101) that faces it. JM."""
    n = max(5, int(round(101 * scale)))
    lam = 3.0
    plane, s7, cur = feed_plane(lam, 10.0, 50.0, n)
    dish = dish_facing_feed(300.0, 300.0, n)
    t7 = engine.generate_grid(dish)
    return dict(name="feed_dish_jm", mode="JM", s7=s7, cur=cur, gmode=0, ncx=n, ncy=n, t7=t7, k=2 * np.pi / lam,
                pairs=s7.shape[1] * t7.shape[1], src=plane, tgt=dish,
                desc=f"Gaussian feed {n}x{n} -> f300 D300 dish uv {n}x{n}, lambda 3 mm, JM")


def dish_chain(scale=1.0):
    """Feed (lambda 2 mm, w0 10 mm, 101x101 over +-50 mm) -> paraboloid D 600,
    f 400 (uv 301x301) with a seeded Gaussian-correlated normal surface error
    (rms lambda/40, correlation 30 mm) -> far field 101x101 over +-1 deg."""
    lam = 2.0
    nf = max(5, int(round(101 * scale)))
    nd = max(5, int(round(301 * scale)))
    nff = max(5, int(round(101 * scale)))
    plane, f7, fcur = feed_plane(lam, 10.0, 50.0, nf)
    dish = dish_facing_feed(400.0, 600.0, nd)
    d7 = engine.generate_grid(dish)
    # the error is a function of the dish's own aperture coordinates (x, -y after the flip):
    # a Gaussian-correlated surface, rms lambda/40, correlation length 30 mm
    delta = engine.correlated_error(d7, lam / 40.0, 30.0, seed=4)
    ff7 = farfield_minus_z(nff, 1.0)
    return dict(name="dish_chain", lam=lam, k=2 * np.pi / lam, feed7=f7, feed_cur=fcur, feed_grid=(0, nf, nf),
                dish7=d7, dish_grid=(1, nd, nd), delta=delta, ff7=ff7,
                desc=f"feed {nf}^2 -> dish {nd}^2 (+surface error) -> FF {nff}^2, lambda 2 mm")


def cassegrain(scale=1.0):
    """Feed (201x201) -> hyperboloid secondary D 200 (foci 1000 mm apart,
    eccentricity 1.2, uv 401x401, JM) -> paraboloid primary D 2000, f 800
    (uv 1001x1001, JM) -> far field 201x201 over +-0.3 deg. lambda 1 mm.
    The primary's focus is the secondary's first focus; the feed sits at the
    second focus, 1000 mm below it."""
    lam = 1.0
    nfe = max(5, int(round(201 * scale)))
    nse = max(5, int(round(401 * scale)))
    npr = max(5, int(round(1001 * scale)))
    nff = max(5, int(round(201 * scale)))
    fprim = 800.0
    f1 = np.array([0.0, 0.0, fprim])
    f2 = np.array([0.0, 0.0, fprim - 1000.0])
    c = np.linalg.norm(f1 - f2) / 2
    a = c / 1.2
    b = np.sqrt(c * c - a * a)
    centre = (f1 + f2) / 2
    sec = SF.translate(SF.hyperboloid(b, b, a, [nse, nse], gmode=1, lims_a=[0.0, 100.0], flip=True), *centre)
    prim = SF.paraboloid(fprim, [npr, npr], gmode=1, lims_a=[0.0, 1000.0])
    # feed waist 3.2 mm: about -10 dB power at the secondary's rim
    plane, fe7, fcur = feed_plane(lam, 3.2, 12.0, nfe, z_shift=f2[2])
    ff7 = engine.generate_grid(SF.farfield([nff, nff], [-0.3, 0.3], [-0.3, 0.3]))
    return dict(name="cassegrain", lam=lam, k=2 * np.pi / lam, feed7=fe7, feed_cur=fcur, feed_grid=(0, nfe, nfe),
                sec7=engine.generate_grid(sec), sec_grid=(1, nse, nse), prim7=engine.generate_grid(prim),
                prim_grid=(1, npr, npr), ff7=ff7,
                desc=f"feed {nfe}^2 -> hyperboloid {nse}^2 -> paraboloid {npr}^2 -> FF {nff}^2, lambda 1 mm")


WORKLOADS["feed_dish_jm"] = feed_dish_jm
