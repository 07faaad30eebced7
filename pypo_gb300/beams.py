"""Source producers: the vector Gaussian feed and equivalent currents.

`gauss_beam` restates the reference's complex-source-point Gaussian beam
(reference src/common/BeamInit.h:407-596, initGaussBeam, reached through
BindBeam.makeGaussBeam, src/PyPO/BindBeam.py:160-199) in vectorised FP64
numpy: the field of an x-polarised source displaced to z + j zc
(zc = k w0^2 / 2), evaluated on a grid, and the equivalent surface currents
J = F n x H, M = -F n x E (mode 0 full, F = 1; mode 1 PMC: M only, F = 2;
mode 2 PEC: J only, F = 2). For points with z + z0 < 0 the fields are
complex-conjugated, as in the reference.

`calc_jm` restates calcJM (reference src/common/BeamInit.h:660-843, reached
through BindBeam.calcCurrents, src/PyPO/BindBeam.py:236-280): the equivalent
surface currents of given fields on a surface, mode 0 J = n x H, M = -n x E;
mode 1 (PMC) M = -2 n x E; mode 2 (PEC) J = 2 n x H; mode 3 J = 2 n x E.

`gauss_beam_dev` and `calc_jm_dev` compute the same on the GPU
(po_gauss_beam_dev, po_calc_jm_dev) from a device grid, so a chain can start
from a feed without host work.
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


def calc_jm(s7, fields, mode=0):
    """Equivalent currents (12, n) of fields (12, n, c2Bundle rows E then H) on
    the points of s7 (normals in rows 3-5)."""
    n = s7[3:6]
    E = fields[0:3] + 1j * fields[3:6]
    H = fields[6:9] + 1j * fields[9:12]
    nE = np.cross(n, E, axis=0)
    nH = np.cross(n, H, axis=0)
    zero = np.zeros_like(nE)
    J, M = {0: (nH, -nE), 1: (zero, -2.0 * nE), 2: (2.0 * nH, zero), 3: (2.0 * nE, zero)}[mode]
    return np.concatenate([J.real, J.imag, M.real, M.imag])


def _dev_args(s7):
    import ctypes
    import torch
    from ._lib import POError
    if not (s7.is_cuda and s7.dtype == torch.float64 and s7.is_contiguous() and s7.shape[0] == 7):
        raise POError("s7 must be a contiguous (7, n) float64 CUDA tensor")
    return ctypes, torch, ctypes.c_void_p(torch.cuda.current_stream(s7.device).cuda_stream)


def gauss_beam_dev(s7, lam, w0, z, power, mode=0):
    """gauss_beam on the GPU: (fields, currents) as (12, n) float64 CUDA tensors."""
    from ._lib import check, load
    ctypes, torch, stream = _dev_args(s7)
    n = s7.shape[1]
    f = torch.empty((12, n), dtype=torch.float64, device=s7.device)
    c = torch.empty((12, n), dtype=torch.float64, device=s7.device)
    check(load().po_gauss_beam_dev(n, ctypes.c_void_p(s7.data_ptr()), float(lam), float(w0), float(z),
                                   float(power), int(mode), ctypes.c_void_p(f.data_ptr()),
                                   ctypes.c_void_p(c.data_ptr()), stream))
    return f, c


def calc_jm_dev(s7, fields, mode=0):
    """calc_jm on the GPU: currents (12, n) float64 CUDA tensor."""
    from ._lib import POError, check, load
    ctypes, torch, stream = _dev_args(s7)
    n = s7.shape[1]
    if not (fields.is_cuda and fields.dtype == torch.float64 and fields.is_contiguous()
            and tuple(fields.shape) == (12, n)):
        raise POError("fields must be a contiguous (12, n) float64 CUDA tensor")
    c = torch.empty((12, n), dtype=torch.float64, device=s7.device)
    check(load().po_calc_jm_dev(n, ctypes.c_void_p(s7.data_ptr()), ctypes.c_void_p(fields.data_ptr()), int(mode),
                                ctypes.c_void_p(c.data_ptr()), stream))
    return c
