// po_sources_dev.cu -- source producers on the device (FP64).
//
//   po_gauss_kernel   the vector Gaussian feed of reference
//                     src/common/BeamInit.h:407-596 (initGaussBeam): the field
//                     of an x-polarised source displaced to z + j zc
//                     (zc = k w0^2 / 2), conjugated for points with z + z0 < 0,
//                     and its equivalent currents;
//   po_calc_jm_kernel the equivalent currents of given fields
//                     (BeamInit.h:660-843, calcJM): mode 0 J = n x H,
//                     M = -n x E; 1 (PMC) M = -2 n x E; 2 (PEC) J = 2 n x H;
//                     3 J = 2 n x E.
// One thread per point; grids and outputs in the engine's row layouts
// (grid 7 x n; fields and currents 12 x n in c2Bundle row order).
#include <cuda_runtime.h>

#include <string>

#include "po_internal.h"

namespace po {
namespace {

struct cd {
    double r, i;
};
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.r + b.r, a.i + b.i}; }
__device__ __forceinline__ cd csub(cd a, cd b) { return {a.r - b.r, a.i - b.i}; }
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.r * s, a.i * s}; }
__device__ __forceinline__ cd cconj(cd a) { return {a.r, -a.i}; }
// a / b with the larger component of b scaled out first (Smith's method).
__device__ __forceinline__ cd cdiv(cd a, cd b)
{
    if (fabs(b.r) >= fabs(b.i)) {
        const double t = b.i / b.r, d = b.r + b.i * t;
        return {(a.r + a.i * t) / d, (a.i - a.r * t) / d};
    }
    const double t = b.r / b.i, d = b.r * t + b.i;
    return {(a.r * t + a.i) / d, (a.i * t - a.r) / d};
}
// Principal square root: with m = |z|, sqrt((m + |re|) / 2) is formed without
// cancellation and the other component follows as im / (2 that).
__device__ __forceinline__ cd csqrt_p(cd z)
{
    if (z.r == 0.0 && z.i == 0.0) return {0.0, z.i};
    const double m = hypot(z.r, z.i);
    const double t = sqrt(0.5 * (m + fabs(z.r)));
    if (z.r >= 0.0) return {t, z.i / (2.0 * t)};
    return {fabs(z.i) / (2.0 * t), copysign(t, z.i)};
}
__device__ __forceinline__ cd cexp_(cd z)
{
    double s, c;
    sincos(z.i, &s, &c);
    const double e = exp(z.r);
    return {e * c, e * s};
}
// (real n) x (complex v)
__device__ __forceinline__ void ncross(const double n[3], const cd v[3], cd o[3])
{
    o[0] = csub(cscale(v[2], n[1]), cscale(v[1], n[2]));
    o[1] = csub(cscale(v[0], n[2]), cscale(v[2], n[0]));
    o[2] = csub(cscale(v[1], n[0]), cscale(v[0], n[1]));
}

__device__ void currents(int mode, const double n[3], const cd E[3], const cd H[3], double *cur, long n_pts, long i)
{
    cd nE[3], nH[3], J[3], M[3];
    ncross(n, E, nE);
    ncross(n, H, nH);
    const cd zero = {0.0, 0.0};
    for (int c = 0; c < 3; ++c) {
        switch (mode) {
        case 0: J[c] = nH[c]; M[c] = cscale(nE[c], -1.0); break;
        case 1: J[c] = zero; M[c] = cscale(nE[c], -2.0); break;
        case 2: J[c] = cscale(nH[c], 2.0); M[c] = zero; break;
        default: J[c] = cscale(nE[c], 2.0); M[c] = zero; break;
        }
        cur[(long)c * n_pts + i] = J[c].r;
        cur[(long)(3 + c) * n_pts + i] = J[c].i;
        cur[(long)(6 + c) * n_pts + i] = M[c].r;
        cur[(long)(9 + c) * n_pts + i] = M[c].i;
    }
}

}  // namespace

__global__ void po_gauss_kernel(long n, const double *__restrict__ g7, double lam, double w0, double z0,
                                double power, int mode, double *__restrict__ fields, double *__restrict__ cur)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double kPi = 3.14159265358979323846;
    const double k = 2 * kPi / lam;
    const double zc = k * w0 * w0 / 2.0;
    const double pref = w0 * k * sqrt(power / (8 * kPi));
    const double x = g7[i], y = g7[n + i], zz = g7[2 * n + i];
    const cd Rx = {x, 0.0}, Ry = {y, 0.0}, Rz = {fabs(zz + z0), zc};
    const cd r2 = cadd(cadd(cmul(Rx, Rx), cmul(Ry, Ry)), cmul(Rz, Rz));
    const cd r = csqrt_p(r2);
    // exp(-j k r - k^2 w0^2 / 2)
    const cd ex = cexp_({k * r.i - k * k * w0 * w0 / 2.0, -k * r.r});
    const cd u = cdiv({1.0, 0.0}, cscale(r, k));
    const cd u2 = cmul(u, u), u3 = cmul(u2, u);
    const cd ju = {-u.i, u.r}, ju3 = {-u3.i, u3.r};
    const cd s1 = cadd(csub(cscale(ju, -1.0), u2), ju3);        // -j u - u^2 + j u^3
    const cd s2 = csub(cadd(ju, cscale(u2, 3.0)), cscale(ju3, 3.0));   // j u + 3u^2 - 3j u^3
    const cd s3 = cadd(ju, u2);                                   // j u + u^2
    const cd a = cscale(ex, pref);
    const cd rr = cmul(r, r);
    const cd qxx = cdiv(cmul(Rx, Rx), rr), qxy = cdiv(cmul(Rx, Ry), rr), qyy = cdiv(cmul(Ry, Ry), rr);
    const cd qxz = cdiv(cmul(Rx, Rz), rr), qyz = cdiv(cmul(Ry, Rz), rr);
    const cd pz = cdiv(Rz, r), px = cdiv(Rx, r), py = cdiv(Ry, r);
    cd E[3], H[3];
    E[0] = cmul(a, csub(cadd(s1, cmul(s2, qxx)), cmul(s3, pz)));
    E[1] = cmul(a, cmul(s2, qxy));
    E[2] = cmul(a, csub(cmul(s2, qxz), cmul(s3, px)));
    H[0] = cmul(a, cmul(s2, qxy));
    H[1] = cmul(a, csub(cadd(s1, cmul(s2, qyy)), cmul(s3, pz)));
    H[2] = cmul(a, csub(cmul(s2, qyz), cmul(s3, py)));
    if (zz + z0 < 0.0)
        for (int c = 0; c < 3; ++c) {
            E[c] = cconj(E[c]);
            H[c] = cconj(H[c]);
        }
    if (fields)
        for (int c = 0; c < 3; ++c) {
            fields[(long)c * n + i] = E[c].r;
            fields[(long)(3 + c) * n + i] = E[c].i;
            fields[(long)(6 + c) * n + i] = H[c].r;
            fields[(long)(9 + c) * n + i] = H[c].i;
        }
    if (cur) {
        const double nn[3] = {g7[3 * n + i], g7[4 * n + i], g7[5 * n + i]};
        currents(mode, nn, E, H, cur, n, i);
    }
}

__global__ void po_calc_jm_kernel(long n, const double *__restrict__ g7, const double *__restrict__ fields, int mode,
                                  double *__restrict__ cur)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cd E[3], H[3];
    for (int c = 0; c < 3; ++c) {
        E[c] = {fields[(long)c * n + i], fields[(long)(3 + c) * n + i]};
        H[c] = {fields[(long)(6 + c) * n + i], fields[(long)(9 + c) * n + i]};
    }
    const double nn[3] = {g7[3 * n + i], g7[4 * n + i], g7[5 * n + i]};
    currents(mode, nn, E, H, cur, n, i);
}

static int launch_pts(void *fn, long n, void **args, cudaStream_t s)
{
    if (n == 0) return 0;
    cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)((n + 255) / 256)), dim3(256), args, 0, s);
    if (e != cudaSuccess) return fail(2, std::string("kernel launch: ") + cudaGetErrorString(e));
    note_launches(1);
    return 0;
}

int gauss_beam_dev(long n, const double *g7, double lam, double w0, double z, double power, int mode,
                   double *fields, double *cur, cudaStream_t s)
{
    if (n < 0) return fail(1, "negative point count");
    if (n > 0 && !g7) return fail(1, "null grid");
    if (!(lam > 0.0) || !(w0 > 0.0) || !(power >= 0.0)) return fail(1, "wavelength and waist must be > 0, power >= 0");
    if (mode < 0 || mode > 2) return fail(1, "mode must be 0 (J, M), 1 (PMC: M) or 2 (PEC: J)");
    void *args[] = {&n, &g7, &lam, &w0, &z, &power, &mode, &fields, &cur};
    return launch_pts(reinterpret_cast<void *>(&po_gauss_kernel), n, args, s);
}

int calc_jm_dev(long n, const double *g7, const double *fields, int mode, double *cur, cudaStream_t s)
{
    if (n < 0) return fail(1, "negative point count");
    if (n > 0 && (!g7 || !fields || !cur)) return fail(1, "null buffer");
    if (mode < 0 || mode > 3) return fail(1, "mode must be 0 (J, M), 1 (PMC), 2 (PEC) or 3 (source)");
    void *args[] = {&n, &g7, &fields, &mode, &cur};
    return launch_pts(reinterpret_cast<void *>(&po_calc_jm_kernel), n, args, s);
}

}  // namespace po
