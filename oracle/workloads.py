"""TEST INFRASTRUCTURE ONLY: the benchmark workloads built on the CPU side.

The same configurations as pypo_gb300/configs.py (dish_eh, dish_ff,
feed_dish_jm, dish_chain, cassegrain), built from oracle/grids.py and the
Gaussian feed below instead of the CUDA library, so that the CPU baseline
(bench.py --impl reference) neither loads nor imports the product.
tests/test_oracle_workloads.py checks that both builders give the same
inputs.

`gauss_beam` restates the reference's vector Gaussian feed (initGaussBeam,
src/common/BeamInit.h:407-596): the field of an x-polarised complex source
point at z + j zc (zc = k w0^2 / 2) with the 1/kr series s1, s2, s3; fields of
points with z + z0 < 0 are conjugated; currents J = F n x H, M = -F n x E with
F = 1 (mode 0), PMC M only and PEC J only with F = 2.
"""
import numpy as np

from . import grids as G


def gauss_beam(s7, lam, w0, z0, power, mode=0):
    """(fields, currents), each (12, n) in c2Bundle row order."""
    k = 2 * np.pi / lam
    zc = k * w0 * w0 / 2.0
    amp = w0 * k * np.sqrt(power / (8 * np.pi))
    z = s7[2] + z0
    R = [s7[0].astype(complex), s7[1].astype(complex), np.abs(z) + 1j * zc]
    r = np.sqrt(R[0] ** 2 + R[1] ** 2 + R[2] ** 2)
    ex = amp * np.exp(-1j * k * r - k * k * w0 * w0 / 2.0)
    q = 1.0 / (k * r)
    s1 = -1j * q - q * q + 1j * q ** 3
    s2 = 1j * q + 3.0 * q * q - 3.0j * q ** 3
    s3 = 1j * q + q * q
    rr = r * r
    E = np.array([ex * (s1 + s2 * R[0] * R[0] / rr - s3 * R[2] / r), ex * s2 * R[0] * R[1] / rr,
                  ex * (s2 * R[0] * R[2] / rr - s3 * R[0] / r)])
    H = np.array([ex * s2 * R[0] * R[1] / rr, ex * (s1 + s2 * R[1] * R[1] / rr - s3 * R[2] / r),
                  ex * (s2 * R[1] * R[2] / rr - s3 * R[1] / r)])
    back = z < 0.0
    E[:, back] = np.conj(E[:, back])
    H[:, back] = np.conj(H[:, back])
    n = s7[3:6]
    F = 2.0 if mode in (1, 2) else 1.0
    J = F * np.cross(n, H, axis=0) if mode in (0, 2) else np.zeros_like(H)
    M = -F * np.cross(n, E, axis=0) if mode in (0, 1) else np.zeros_like(E)
    rows = lambda A, B: np.concatenate([A.real, A.imag, B.real, B.imag])
    return rows(E, H), rows(J, M)


def tapered_currents(s7, radius, seed=1, phase_rms=0.05, taper_db=10.0):
    """x-polarised J projected tangential to the surface, Gaussian power taper
    of taper_db at `radius`, random phase N(0, phase_rms) (numpy seed); M = 0."""
    r = np.hypot(s7[0], s7[1])
    amp = np.exp(-0.5 * np.log(10 ** (taper_db / 10)) * (r / radius) ** 2)
    phi = np.random.default_rng(seed).normal(0.0, phase_rms, r.size)
    n = s7[3:6]
    jt = np.array([1.0, 0.0, 0.0])[:, None] - n[0][None, :] * n
    J = jt * (amp * np.exp(1j * phi))
    cur = np.zeros((12, r.size))
    cur[0:3], cur[3:6] = J.real, J.imag
    return cur


def dish_eh(scale=1.0):
    nsg = max(3, int(round(501 * scale)))
    ntg = max(3, int(round(301 * scale)))
    f, D, lam = 500.0, 1000.0, 1.0
    s7 = G.generate(G.paraboloid(f, [nsg, nsg], gmode=1, lims_a=[0.0, D / 2]))
    t7 = G.generate(G.translate(G.plane([ntg, ntg], gmode=0, lims_a=[-50.0, 50.0]), dz=f))
    return dict(name="dish_eh", mode="EH", s7=s7, cur=tapered_currents(s7, D / 2), gmode=1, ncx=nsg, ncy=nsg,
                t7=t7, k=2 * np.pi / lam, pairs=s7.shape[1] * t7.shape[1])


def dish_ff(scale=1.0):
    nsg = max(3, int(round(1001 * scale)))
    ntg = max(3, int(round(401 * scale)))
    f, D, lam = 800.0, 2000.0, 1.0
    s7 = G.generate(G.paraboloid(f, [nsg, nsg], gmode=1, lims_a=[0.0, D / 2]))
    t7 = G.generate(G.farfield([ntg, ntg], [-0.5, 0.5], [-0.5, 0.5]))
    return dict(name="dish_ff", mode="FF", s7=s7, cur=tapered_currents(s7, D / 2), gmode=1, ncx=nsg, ncy=nsg,
                t7=t7, k=2 * np.pi / lam, pairs=s7.shape[1] * t7.shape[1])


def feed_plane(lam, w0, half_width, n, power=4 * np.pi, z_shift=0.0):
    s7 = G.generate(G.plane([n, n], gmode=0, lims_a=[-half_width, half_width]))
    _, cur = gauss_beam(s7, lam, w0, 0.0, power)
    s7[2] += z_shift
    return s7, np.ascontiguousarray(cur)


def dish_facing_feed(f, D, n):
    return G.translate(G.rotate_x(G.paraboloid(f, [n, n], gmode=1, lims_a=[0.0, D / 2]), 180.0), dz=f)


def feed_dish_jm(scale=1.0):
    n = max(5, int(round(101 * scale)))
    lam = 3.0
    s7, cur = feed_plane(lam, 10.0, 50.0, n)
    t7 = G.generate(dish_facing_feed(300.0, 300.0, n))
    return dict(name="feed_dish_jm", mode="JM", s7=s7, cur=cur, gmode=0, ncx=n, ncy=n, t7=t7, k=2 * np.pi / lam,
                pairs=s7.shape[1] * t7.shape[1])


WORKLOADS = {"dish_eh": dish_eh, "dish_ff": dish_ff, "feed_dish_jm": feed_dish_jm}


def cassegrain(scale=1.0):
    """Stage geometry of the Cassegrain chain (feed -> hyperboloid -> paraboloid -> far field)."""
    lam = 1.0
    nfe = max(5, int(round(201 * scale)))
    nse = max(5, int(round(401 * scale)))
    npr = max(5, int(round(1001 * scale)))
    nff = max(5, int(round(201 * scale)))
    fprim = 800.0
    c = 500.0
    a = c / 1.2
    b = np.sqrt(c * c - a * a)
    sec = G.translate(G.hyperboloid(b, b, a, [nse, nse], gmode=1, lims_a=[0.0, 100.0], flip=True), 0.0, 0.0,
                      fprim - c)
    fe7, fcur = feed_plane(lam, 3.2, 12.0, nfe, z_shift=fprim - 1000.0)
    return dict(k=2 * np.pi / lam, feed7=fe7, feed_cur=fcur, feed_grid=(0, nfe, nfe), sec7=G.generate(sec),
                sec_grid=(1, nse, nse),
                prim7=G.generate(G.paraboloid(fprim, [npr, npr], gmode=1, lims_a=[0.0, 1000.0])),
                prim_grid=(1, npr, npr), ff7=G.generate(G.farfield([nff, nff], [-0.3, 0.3], [-0.3, 0.3])))


def dish_chain(scale=1.0):
    """Stage geometry of the perturbed-dish chain (feed -> dish -> far field);
    the dish's surface error enters the chain as a displacement input, so the
    grid here is the unperturbed one, as in the product's builder."""
    lam = 2.0
    nf = max(5, int(round(101 * scale)))
    nd = max(5, int(round(301 * scale)))
    nff = max(5, int(round(101 * scale)))
    f7, fcur = feed_plane(lam, 10.0, 50.0, nf)
    ff7 = G.generate(G.farfield([nff, nff], [-1.0, 1.0], [-1.0, 1.0]))
    ff7[0] = np.pi - ff7[0]
    return dict(k=2 * np.pi / lam, feed7=f7, feed_cur=fcur, feed_grid=(0, nf, nf),
                dish7=G.generate(dish_facing_feed(400.0, 600.0, nd)), dish_grid=(1, nd, nd), ff7=ff7)


CHAINS = {"cassegrain": cassegrain, "dish_chain": dish_chain}
