"""Soundness of the lit-tile proof (pypo_gb300/csrc/po_kernels.cu: tile_lit,
po_src_box_kernel and the CTA target box of po_pk_kernel), restated in numpy
FP32 on the CPU: whenever the proof says a tile is lit for a block of
targets, every (source, target) pair of the two passes the kernel's own
per-pair test, computed the kernel's way (hi/lo split positions in turns,
FP32 differences; lit when n.d >= 1e-6 R, the tangent band's edge). Seeded random scenes, among them ones
whose targets graze the sources' tangent planes, where the margins matter.
"""
import numpy as np
import pytest

F = np.float32
BAND = F(1e-6)   # kTangentBand: lit at n.d >= BAND R, deferred to FP64 inside +-BAND R


def split(x, q):
    """hi on the quantum q (exact in FP32) and the FP32 rounded remainder."""
    hi = np.rint(x / q) * q
    return hi.astype(F), (x - hi).astype(F)


def source_box(sh, sl, n):
    """po_src_box_kernel: lowest / highest normal per axis, max n.s, max |s|_1."""
    s = sh + sl                                             # FP32 add, as in the kernel
    ns = (n[:, 2] * s[:, 2] + (n[:, 1] * s[:, 1] + n[:, 0] * s[:, 0])).astype(F)
    return n.min(0), n.max(0), ns.max(), np.abs(s).sum(1).astype(F).max()


def target_box(th, tl):
    t = th + tl
    lo, hi = t.min(0), t.max(0)
    return lo, hi, F(np.maximum(np.abs(lo), np.abs(hi)).sum())


def lit(sbox, tbox):
    nlo, nhi, nsmax, sabs = sbox
    tlo, thi, tabs = tbox
    L = F(0)
    for c in range(3):
        a, b = nlo[c], nhi[c]
        L = F(L + min(a * tlo[c], a * thi[c], b * tlo[c], b * thi[c]))
    return F(L - nsmax) >= F(1e-5) * F(tabs + sabs)


def pair_test(sh, sl, n, th, tl):
    """The kernel's per-pair illumination test for every pair (FP32)."""
    dh = th[None, :, :] - sh[:, None, :]
    dl = tl[None, :, :] - sl[:, None, :]
    d = (dh + dl).astype(F)
    R = np.sqrt((d.astype(np.float64) ** 2).sum(-1)).astype(F)
    nd = (n[:, None, 2] * d[..., 2] + (n[:, None, 1] * d[..., 1] + n[:, None, 0] * d[..., 0])).astype(F)
    return nd >= BAND * R


def scene(seed):
    """Sources on a plane patch (the tile), targets in front of it (the CTA):
    family 0, normals exactly along a coordinate axis and target heights of
    1 to 100 times the proof's margin; family 1, normals tilted up to 0.02
    rad and heights of 30 % to 100 % of the scene (the interval bound
    decouples normals from positions, so it needs heights well above the
    normals' spread times the scene); family 2, grazing targets (heights
    down to 1e-9 of the scene), mostly unlit."""
    rng = np.random.default_rng(seed)
    fam = seed % 3
    m = 10.0 ** rng.uniform(0, 4)                          # scene half-extent in turns
    q = 2.0 ** np.ceil(np.log2(m / 1024))                  # the frame's quantum
    ns = nt = 128
    if fam == 0:
        axis = np.zeros(3)
        axis[rng.integers(3)] = rng.choice([-1.0, 1.0])
    else:
        axis = rng.standard_normal(3)
        axis /= np.linalg.norm(axis)
    e1 = np.cross(axis, rng.standard_normal(3))
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(axis, e1)
    p0 = rng.uniform(-0.5, 0.5, 3) * m if fam != 1 else rng.uniform(-0.1, 0.1, 3) * m
    uv = rng.uniform(-0.1, 0.1, (ns, 2)) * m
    s = p0 + uv[:, :1] * e1 + uv[:, 1:] * e2
    n = np.tile(axis, (ns, 1))
    if fam:
        n = n + rng.uniform(-0.02, 0.02, (ns, 3)) * (1 if fam == 1 else 2.5)
        n /= np.linalg.norm(n, axis=1)[:, None]
    lat = rng.uniform(-0.1, 0.1, (nt, 2)) * m
    if fam == 0:
        eps = 1e-5 * 2 * 3 * (np.abs(p0).max() + 0.2 * m)
        h = eps * 10.0 ** rng.uniform(0, 2, nt)
    elif fam == 1:
        h = m * rng.uniform(0.3, 1.0, nt)
    else:
        h = m * 10.0 ** rng.uniform(-9, 0, nt)
    t = p0 + lat[:, :1] * e1 + lat[:, 1:] * e2 + h[:, None] * axis
    sh, sl = split(s, q)
    th, tl = split(t, q)
    return sh, sl, n.astype(F), th, tl


@pytest.mark.parametrize("seed", range(60))
def test_a_proven_tile_passes_every_pair_test(seed):
    sh, sl, n, th, tl = scene(seed)
    if lit(source_box(sh, sl, n), target_box(th, tl)):
        passes = pair_test(sh, sl, n, th, tl)
        assert passes.all(), (seed, np.argwhere(~passes)[:3])


def test_the_scenes_exercise_the_proof():
    """Not vacuous: the proof holds for most facing scenes, including ones
    whose targets stand only a few margins above the sources' plane, and
    fails for scenes with unlit pairs."""
    proven = [lit(source_box(sh, sl, n), target_box(th, tl)) for sh, sl, n, th, tl in map(scene, range(60))]
    unlit = [not pair_test(*scene(i)).all() for i in range(60)]
    assert sum(proven[0::3]) >= 10 and sum(proven[1::3]) >= 5
    assert not any(p and u for p, u in zip(proven, unlit))
    assert sum(unlit) >= 5


def test_the_proof_holds_for_plain_facing_scenes():
    """A dish facing its focal plane (the benchmark's geometry) is proven lit."""
    rng = np.random.default_rng(1)
    r = np.sqrt(rng.uniform(0, 1, 128)) * 500.0
    ph = rng.uniform(0, 2 * np.pi, 128)
    s = np.stack([r * np.cos(ph), r * np.sin(ph), r * r / 2000.0], 1)     # z = r^2 / 4f, f = 500
    n = np.stack([-s[:, 0], -s[:, 1], np.full(128, 1000.0)], 1)
    n /= np.linalg.norm(n, axis=1)[:, None]
    t = np.stack([rng.uniform(-50, 50, 128), rng.uniform(-50, 50, 128), np.full(128, 500.0)], 1)
    o = np.array([0.0, 0.0, 250.0])                                       # frame origin: box centre
    q = 2.0 ** np.ceil(np.log2(500 / 1024))
    sh, sl = split(s - o, q)
    th, tl = split(t - o, q)
    assert lit(source_box(sh, sl, n.astype(F)), target_box(th, tl))
    assert pair_test(sh, sl, n.astype(F), th, tl).all()
