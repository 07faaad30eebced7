"""Source producers: the vector Gaussian feed.

`gauss_beam` restates the reference's complex-source-point Gaussian beam
(reference src/common/BeamInit.h:407-596, initGaussBeam, reached through
BindBeam.makeGaussBeam, src/PyPO/BindBeam.py:160-199) in vectorised FP64
numpy: the field of an x-polarised source displaced to z + j zc
(zc = k w0^2 / 2), evaluated on a grid, and the equivalent surface currents
J = F n x H, M = -F n x E (mode 0 full, F = 1; mode 1 PMC: M only, F = 2;
mode 2 PEC: J only, F = 2). For points with z + z0 < 0 the fields are
complex-conjugated, as in the reference.
"""
import numpy as np


def gauss_beam(s7, lam, w0, z, power, mode=0):
    """Fields (E, H) and currents (J, M) as (12, n) c2Bundle-order blocks."""
    x, y, zz = s7[0], s7[1], s7[2]
    n = s7[3:6]
    k = 2 * np.pi / lam
    zc = k * w0 * w0 / 2.0
    pref = w0 * k * np.sqrt(power / (8 * np.pi))
    Rx = x.astype(complex)
    Ry = y.astype(complex)
    Rz = np.abs(zz + z) + 1j * zc
    r = np.sqrt(Rx * Rx + Ry * Ry + Rz * Rz)
    expo = np.exp(-1j * k * r - k * k * w0 * w0 / 2.0)
    u = 1.0 / (k * r)
    s1 = -1j * u - u * u + 1j * u ** 3
    s2 = 1j * u + 3.0 * u * u - 3.0j * u ** 3
    s3 = 1j * u + u * u
    a = pref * expo
    E = np.stack([a * (s1 + s2 * Rx * Rx / (r * r) - s3 * Rz / r),
                  a * s2 * Rx * Ry / (r * r),
                  a * (s2 * Rx * Rz / (r * r) - s3 * Rx / r)])
    H = np.stack([a * s2 * Rx * Ry / (r * r),
                  a * (s1 + s2 * Ry * Ry / (r * r) - s3 * Rz / r),
                  a * (s2 * Ry * Rz / (r * r) - s3 * Ry / r)])
    behind = (zz + z) < 0
    E = np.where(behind, np.conj(E), E)
    H = np.where(behind, np.conj(H), H)
    M_ = np.cross(n, E, axis=0)
    J_ = np.cross(n, H, axis=0)
    F = 2.0 if mode in (1, 2) else 1.0
    J = F * J_ if mode in (0, 2) else np.zeros_like(J_)
    M = -F * M_ if mode in (0, 1) else np.zeros_like(M_)

    def block(A, B):
        return np.concatenate([A.real, A.imag, B.real, B.imag])

    return block(E, H), block(J, M)
