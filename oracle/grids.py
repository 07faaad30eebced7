"""TEST INFRASTRUCTURE ONLY: FP64 reflector grids in numpy.

A vectorised restatement of the reference's grid generator, used where a
checker or the CPU baseline needs geometry without the CUDA library:
  paraboloid xy / uv   src/common/InterfaceReflector.cpp:84-135, :166-244
  hyperboloid xy / uv  :271-322, :353-434
  ellipsoid xy / uv    :460-509, :540-621
  plane xy / uv / AoE  :645-686, :712-768, :794-849
  4x4 transform        :35-57 (points get the affine map, normals its 3x3 part)
  surface error        :852-866 (uncorrelated, along the normals), drawn as
                       src/include/Random.h:112-116 does: mt19937 seeded with
                       rms_seed and a fresh normal distribution per point.
Pinned to the reference's own grids by tests/test_oracle_grids.py
(tests/golden/golden_grids.npz).

Reflector dicts use the keys of the reference's allfill_reflparams
(src/PyPO/BindUtils.py:277-327); the builders below make the ones the
benchmark workloads need. Index order is row-major over (x/u, y/v).
"""
import numpy as np

PI = 3.14159265358979323846


# ------------------------------------------------------------ reflector dicts

def _base(rtype, gmode, gridsize, **kw):
    d = {"type": rtype, "gmode": gmode, "gridsize": np.asarray(gridsize, dtype=int),
         "coeffs": np.zeros(3), "gcenter": np.zeros(2), "flip": False, "ecc_uv": 0.0,
         "rot_uv": 0.0, "transf": np.eye(4), "rms": 0.0, "rms_seed": 0}
    d.update(kw)
    return d


def _lims(gmode, lims_a, lims_b):
    key = {0: ("lims_x", "lims_y"), 1: ("lims_u", "lims_v"), 2: ("lims_Az", "lims_El")}[gmode]
    return {key[0]: np.asarray(lims_a, dtype=float), key[1]: np.asarray(lims_b, dtype=float)}


def paraboloid(f, gridsize, gmode=1, lims_a=None, lims_b=None, **kw):
    """z = (x^2 + y^2) / (4 f): a = b = 2 sqrt(f) (reference System.py:244-282)."""
    a = 2.0 * np.sqrt(f)
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(0, gmode, gridsize, coeffs=np.array([a, a, -1.0]), **_lims(gmode, lims_a, lims_b), **kw)


def hyperboloid(a, b, c, gridsize, gmode=1, lims_a=None, lims_b=None, **kw):
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(1, gmode, gridsize, coeffs=np.array([a, b, c], dtype=float), **_lims(gmode, lims_a, lims_b), **kw)


def plane(gridsize, gmode=0, lims_a=(-1.0, 1.0), lims_b=None, **kw):
    if lims_b is None:
        lims_b = [0.0, 360.0] if gmode == 1 else lims_a
    return _base(3, gmode, gridsize, **_lims(gmode, lims_a, lims_b), **kw)


def farfield(gridsize, lims_Az, lims_El, **kw):
    return _base(3, 2, gridsize, **_lims(2, lims_Az, lims_El), **kw)


def translate(d, dx=0.0, dy=0.0, dz=0.0):
    m = np.eye(4)
    m[:3, 3] = [dx, dy, dz]
    d = dict(d)
    d["transf"] = m @ np.asarray(d["transf"])
    return d


def rotate_x(d, deg):
    t = np.deg2rad(deg)
    m = np.eye(4)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = np.cos(t), -np.sin(t), np.sin(t), np.cos(t)
    d = dict(d)
    d["transf"] = m @ np.asarray(d["transf"])
    return d


# ---------------------------------------------------------------- generator

def _quadric(rtype, a, b, c, x, y):
    """Height and unnormalised normal of the surface at (x, y)."""
    one = np.ones_like(x)
    if rtype == 0:
        return x * x / (a * a) + y * y / (b * b), (-2 * x / (a * a), -2 * y / (b * b), one)
    if rtype == 1:
        z = c * np.sqrt(x * x / (a * a) + y * y / (b * b) + 1)
        return z, (-2 * x / (a * a), -2 * y / (b * b), 2 * z / (c * c))
    if rtype == 2:
        z = c * np.sqrt(1 - x * x / (a * a) - y * y / (b * b))
        return z, (2 * x / (a * a), 2 * y / (b * b), 2 * z / (c * c))
    return np.zeros_like(x), (0 * x, 0 * x, one)


def _slope(rtype, a, b, c, x, y, z):
    if rtype == 0:
        return 2 * x / (a * a), 2 * y / (b * b)
    if rtype == 1:
        return c * c / z * x / (a * a), c * c / z * y / (b * b)
    if rtype == 2:
        return -c * c / z * x / (a * a), -c * c / z * y / (b * b)
    return 0 * x, 0 * x


def _normals(rtype, n, nfac, shape):
    if rtype == 3:
        return np.zeros(shape), np.zeros(shape), nfac * np.ones(shape), None
    nrm = np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
    return nfac * n[0] / nrm, nfac * n[1] / nrm, nfac * n[2] / nrm, nrm


def _grid_xy(d, nfac):
    ncx, ncy = (int(v) for v in d["gridsize"])
    a, b, c = (float(v) for v in d["coeffs"])
    lx, ly = np.asarray(d["lims_x"], float), np.asarray(d["lims_y"], float)
    dx = (lx[1] - lx[0]) / (ncx - 1)
    dy = (ly[1] - ly[0]) / (ncy - 1)
    centred = d["type"] in (0, 1)
    gc = np.asarray(d["gcenter"], float) if centred else np.zeros(2)
    x = (np.arange(ncx) * dx + lx[0] + gc[0])[:, None] * np.ones((1, ncy))
    y = np.ones((ncx, 1)) * (np.arange(ncy) * dy + ly[0] + gc[1])[None, :]
    z, n = _quadric(d["type"], a, b, c, x, y)
    nx, ny, nz, nrm = _normals(d["type"], n, nfac, x.shape)
    area = dx * dy * (np.ones_like(x) if nrm is None else nrm)
    return np.stack([x, y, z, nx, ny, nz, area]).reshape(7, -1)


def _grid_uv(d, nfac):
    ncx, ncy = (int(v) for v in d["gridsize"])
    a, b, c = (float(v) for v in d["coeffs"])
    lu, lv = np.asarray(d["lims_u"], float), np.asarray(d["lims_v"], float)
    gc = np.asarray(d["gcenter"], float)
    du0 = (lu[1] - lu[0]) / (ncx - 1)
    dv = (lv[1] - lv[0]) / ncy
    ecc = float(d["ecc_uv"])
    rot = float(d["rot_uv"]) * PI / 180
    cr, sr = np.cos(rot), np.sin(rot)
    i = np.arange(ncx)[:, None] * np.ones((1, ncy))
    v = np.ones((ncx, 1)) * ((np.arange(ncy) * dv + lv[0]) * PI / 180)[None, :]
    sv, cv = np.sin(v), np.cos(v)
    ef = np.sqrt(1 - ecc * ecc * sv * sv)
    duv = du0 / ef
    u = i * duv + lu[0] / ef
    dudv = u / (ef * ef) * ecc * ecc * cv * sv
    x = u * cv * cr - u * sv * sr + gc[0]
    y = u * cv * sr + u * sv * cr + gc[1]
    z, n = _quadric(d["type"], a, b, c, x, y)
    nx, ny, nz, nrm = _normals(d["type"], n, nfac, x.shape)
    if nrm is None:
        area = u * duv * dv * PI / 180
    else:
        xu = cv * cr - sv * sr
        xv = cv * cr * dudv - u * sv * cr - sv * sr * dudv - u * cv * sr
        yu = cv * sr + sv * cr
        yv = cv * sr * dudv - u * sv * sr + sv * cr * dudv + u * cv * cr
        zx, zy = _slope(d["type"], a, b, c, x, y, z)
        zu = zx * xu + zy * yu
        zv = zx * xv + zy * yv
        cx = yu * zv - zu * yv
        cy = zu * xv - xu * zv
        cz = xu * yv - yu * xv
        area = np.sqrt(cx * cx + cy * cy + cz * cz) * duv * dv * PI / 180
    return np.stack([x, y, z, nx, ny, nz, area]).reshape(7, -1)


def _grid_aoe(d, spheric):
    ncx, ncy = (int(v) for v in d["gridsize"])
    la, le = np.asarray(d["lims_Az"], float), np.asarray(d["lims_El"], float)
    dA = (la[1] - la[0]) / (ncx - 1)
    dE = (le[1] - le[0]) / (ncy - 1)
    az = (np.arange(ncx) * dA + la[0])[:, None] * np.ones((1, ncy))
    el = np.ones((ncx, 1)) * (np.arange(ncy) * dE + le[0])[None, :]
    x, y = az, el
    if spheric:
        x = np.sqrt(az * az + el * el) * PI / 180
        y = np.nan_to_num(np.arctan2(el, az))
    area = np.cos(el * PI / 180) * dA * dE * PI * PI / 180 / 180
    z = np.zeros_like(x)
    return np.stack([x, y, z, z, z, np.ones_like(x), area]).reshape(7, -1)


def generate(d, transform=True, spheric=True):
    """(7, n) float64 rows x y z nx ny nz area of a reflector dict."""
    nfac = -1.0 if d.get("flip", False) else 1.0
    gm = int(d["gmode"])
    if gm == 0:
        g = _grid_xy(d, nfac)
    elif gm == 1:
        g = _grid_uv(d, nfac)
    elif gm == 2:
        return _grid_aoe(d, spheric)
    else:
        raise ValueError("gmode must be 0 (xy), 1 (uv) or 2 (AoE)")
    if transform:
        m = np.asarray(d["transf"], dtype=float).reshape(4, 4)
        p = m[:3, :3] @ g[0:3] + m[:3, 3:4]
        q = m[:3, :3] @ g[3:6]
        g = np.concatenate([p, q, g[6:7]])
    rms = float(d.get("rms", 0.0))
    if rms > 0:
        g[0:3] += normal_deviates(int(d.get("rms_seed", 0)), g.shape[1], rms)[None, :] * g[3:6]
    return np.ascontiguousarray(g)


# ------------------------------------------- mt19937 and the normal deviates
#
# MT19937 (Matsumoto and Nishimura, 1998): 624-word state, seeded by the
# recurrence x_i = 1812433253 (x_{i-1} ^ (x_{i-1} >> 30)) + i; each block of
# 624 outputs is the twist of the state (tap 397, matrix 0x9908b0df) followed
# by tempering. The reference draws a double in [0, 1) from two outputs
# (low word first: (w0 + w1 2^32) / 2^64, at most the double below 1) and a
# normal deviate by Marsaglia's polar method: x, y = 2U - 1 until
# 0 < r2 = x^2 + y^2 <= 1, then y sqrt(-2 ln r2 / r2). A fresh distribution
# per point discards the method's second deviate, so each point takes the
# next accepted (x, y) pair: four 32-bit outputs per attempt.

_N, _M = 624, 397


def _mt_seed(seed):
    mt = np.zeros(_N, dtype=np.uint64)
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, _N):
        prev = int(mt[i - 1])
        mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
    return mt


def _mt_twist(mt):
    """The next 624-word state (in place semantics of the sequential twist)."""
    up, lo, mag = np.uint64(0x80000000), np.uint64(0x7FFFFFFF), np.uint64(0x9908B0DF)
    one = np.uint64(1)
    new = mt.copy()

    def step(idx, nxt, tap):
        y = (new[idx] & up) | (nxt & lo)
        return tap ^ (y >> one) ^ np.where((y & one) != 0, mag, np.uint64(0))

    a = np.arange(0, _N - _M)
    new[a] = step(a, mt[a + 1], mt[a + _M])
    b = np.arange(_N - _M, 2 * (_N - _M))
    new[b] = step(b, mt[b + 1], new[b - (_N - _M)])
    c = np.arange(2 * (_N - _M), _N - 1)
    new[c] = step(c, mt[c + 1], new[c - (_N - _M)])
    last = np.array([_N - 1])
    new[last] = step(last, new[np.array([0])], new[np.array([_M - 1])])
    return new


def _temper(y):
    y = y ^ (y >> np.uint64(11))
    y = y ^ ((y << np.uint64(7)) & np.uint64(0x9D2C5680))
    y = y ^ ((y << np.uint64(15)) & np.uint64(0xEFC60000))
    y = y ^ (y >> np.uint64(18))
    return y & np.uint64(0xFFFFFFFF)


def mt19937_words(seed, count):
    """The first `count` 32-bit outputs of mt19937 seeded with `seed`."""
    mt = _mt_seed(seed)
    out = []
    have = 0
    while have < count:
        mt = _mt_twist(mt)
        out.append(_temper(mt))
        have += _N
    return np.concatenate(out)[:count] if out else np.zeros(0, dtype=np.uint64)


def normal_deviates(seed, n, stdev):
    """n deviates N(0, stdev), each from a fresh distribution on one mt19937."""
    if n == 0:
        return np.zeros(0)
    words = 4 * (n + n // 2 + 64)
    while True:
        w = mt19937_words(seed, words).astype(np.float64)
        u = (w[0::2] + w[1::2] * 4294967296.0) / 18446744073709551616.0
        u = np.minimum(u, np.nextafter(1.0, 0.0))
        x = 2.0 * u[0::2] - 1.0
        y = 2.0 * u[1::2] - 1.0
        r2 = x * x + y * y
        ok = (r2 <= 1.0) & (r2 != 0.0)
        if ok.sum() >= n:
            ya, ra = y[ok][:n], r2[ok][:n]
            return ya * np.sqrt(-2.0 * np.log(ra) / ra) * stdev
        words *= 2


# -------------------------------------------------- correlated surface error

def correlated_error(x, y, rms, corr_len, seed, n_modes=512):
    """Gaussian-correlated random surface by spectral synthesis, evaluated at
    the points (x, y): delta = rms sqrt(2 / M) sum_m cos(kx_m x + ky_m y + ph_m)
    over M = n_modes modes, whose covariance is rms^2 exp(-r^2 / (2 corr_len^2)).
    The modes come from the reference's generator (mt19937 seeded with `seed`,
    a fresh normal deviate per draw, as normal_deviates): four deviates g per
    mode, kx = g0 / corr_len, ky = g1 / corr_len, ph = atan2(g2, g3) (uniform
    for independent normals)."""
    m = int(n_modes)
    g = normal_deviates(int(seed), 4 * m, 1.0).reshape(m, 4)
    kx, ky = g[:, 0] / corr_len, g[:, 1] / corr_len
    ph = np.arctan2(g[:, 2], g[:, 3])
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    out = np.zeros(x.shape)
    for c in range(0, m, 64):   # modes in blocks, points vectorised
        arg = np.outer(x, kx[c:c + 64]) + np.outer(y, ky[c:c + 64]) + ph[c:c + 64]
        out += np.cos(arg).sum(axis=1)
    return rms * np.sqrt(2.0 / m) * out
