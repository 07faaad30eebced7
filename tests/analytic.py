"""Closed-form fields for the analytic known-answer tests (test helper).

The fields of infinitesimal current elements, derived independently of the
reference's code: the oscillating electric dipole of Jackson, Classical
Electrodynamics (3rd ed., section 9.2), written for exp(+j w t) time
dependence (outgoing waves exp(-j k R)), with the current element
I l = j w p, in the units the reference's kernel uses (medium impedance 1,
prefactor k^2 / (4 pi) with its float-literal pi). Magnetic current
elements follow by duality (J -> M, E -> H, H -> -E).
"""
import numpy as np

PI_F = float(np.float32(3.14159265359))   # the reference's float-literal pi


def unit_cloud(points, normals, areas):
    """(7, n) point cloud rows x y z nx ny nz area."""
    p = np.asarray(points, float).reshape(-1, 3)
    n = np.broadcast_to(np.asarray(normals, float).reshape(-1, 3), p.shape)
    a = np.broadcast_to(np.asarray(areas, float), (p.shape[0],))
    return np.ascontiguousarray(np.vstack([p.T, n.T, a[None, :]]))


def currents(J=None, M=None, n=1):
    """(12, n) c2Bundle rows from complex (n, 3) or (3,) J and M."""
    out = np.zeros((12, n))
    for off, v in ((0, J), (6, M)):
        if v is None:
            continue
        v = np.broadcast_to(np.asarray(v, complex), (n, 3))
        out[off:off + 3] = v.real.T
        out[off + 3:off + 6] = v.imag.T
    return out


def to_complex(out):
    """(12, nt) E, H rows -> two complex (nt, 3) arrays."""
    e = out[0:3] + 1j * out[3:6]
    h = out[6:9] + 1j * out[9:12]
    return e.T, h.T


def dipole(k, r0, r, J, M, A=1.0):
    """E and H at points r (m, 3) of current elements J, M (complex 3-vectors)
    of area A at r0, outgoing waves."""
    d = np.asarray(r, float) - np.asarray(r0, float)
    R = np.linalg.norm(d, axis=1)[:, None]
    n = d / R
    u = 1.0 / (k * R)
    g = k * k / (4 * PI_F) * A * np.exp(-1j * k * R)
    J = np.asarray(J, complex)[None, :]
    M = np.asarray(M, complex)[None, :]

    def e_of(C):
        cn = np.sum(C * n, axis=1, keepdims=True)
        return g * -1j * (C * (u - 1j * u ** 2 - u ** 3) + cn * n * (-u + 3j * u ** 2 + 3 * u ** 3))

    def h_of(C):
        return g * np.cross(C, n) * (1j * u + u ** 2)

    E = e_of(J) - h_of(M)
    H = h_of(J) + e_of(M)
    return E, H


def far_field(k, r0, rhat, J, M, A=1.0):
    """The elements' far fields in directions rhat (m, 3): the dipole fields
    times k R exp(j k R) as R -> infinity (the phase referred to the origin)."""
    rh = np.asarray(rhat, float)
    g = k * k / (4 * PI_F) * A * np.exp(1j * k * (rh @ np.asarray(r0, float)))[:, None]
    J = np.asarray(J, complex)[None, :]
    M = np.asarray(M, complex)[None, :]

    def e_of(C):
        return g * -1j * (C - np.sum(C * rh, axis=1, keepdims=True) * rh)

    def h_of(C):
        return g * 1j * np.cross(C, rh)

    return e_of(J) - h_of(M), h_of(J) + e_of(M)


def polar_azimuth(rhat):
    """(7, m) far-field target rows: x = polar angle, y = azimuth (radians)."""
    rh = np.asarray(rhat, float)
    th = np.arccos(np.clip(rh[:, 2], -1, 1))
    ph = np.arctan2(rh[:, 1], rh[:, 0])
    t = np.zeros((7, rh.shape[0]))
    t[0], t[1], t[5], t[6] = th, ph, 1.0, 1.0
    return t


def rel(a, b):
    """Relative L2 difference of b against a."""
    return float(np.linalg.norm(np.asarray(b) - np.asarray(a)) / np.linalg.norm(np.asarray(a)))
