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
