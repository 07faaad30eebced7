// po_grid_dev.cu -- FP64 reflector grid generation on the device.
//
// The same formulas as the host generator po_grid.cpp (reference
// src/common/InterfaceReflector.cpp: paraboloid xy / uv :84-135, :166-244,
// hyperboloid :271-322, :353-434, ellipsoid :460-509, :540-621, plane xy / uv /
// AoE :645-686, :712-768, :794-849, 4x4 transform :35-57), one thread per grid
// point, written straight into the 7-row device layout the propagation entry
// points take (x, y, z, nx, ny, nz, area; index i*ncy + j). The optional
// surface error (:852-866) keeps the reference's random sequence: mt19937
// with a fresh normal distribution per point (Random.h:112-116) is
// sequential, so the deviates are drawn on the host, copied, and applied
// along the normals by a second kernel.
#include <cuda_runtime.h>

#include <random>
#include <string>
#include <vector>

#include "po_internal.h"

namespace po {

// Scalars of a reflparams, by value.
struct GridSpec {
    int type, gmode, ncx, ncy, nfac, spheric, transform;
    double a, b, c;
    double lxu0, lxu1, lyv0, lyv1, gcx, gcy, ecc, rot;
    double m[12];   // first three rows of the 4x4 transform
};

namespace {

constexpr double kPiD = 3.14159265358979323846;

__device__ void quadric_d(int type, double a, double b, double c, double x, double y, double &z, double n[3])
{
    switch (type) {
    case 0:
        z = x * x / (a * a) + y * y / (b * b);
        n[0] = -2 * x / (a * a); n[1] = -2 * y / (b * b); n[2] = 1;
        break;
    case 1:
        z = c * sqrt(x * x / (a * a) + y * y / (b * b) + 1);
        n[0] = -2 * x / (a * a); n[1] = -2 * y / (b * b); n[2] = 2 * z / (c * c);
        break;
    case 2:
        z = c * sqrt(1 - x * x / (a * a) - y * y / (b * b));
        n[0] = 2 * x / (a * a); n[1] = 2 * y / (b * b); n[2] = 2 * z / (c * c);
        break;
    default:
        z = 0;
        n[0] = 0; n[1] = 0; n[2] = 1;
        break;
    }
}

__device__ void slope_d(int type, double a, double b, double c, double x, double y, double z, double &zx, double &zy)
{
    switch (type) {
    case 0: zx = 2 * x / (a * a); zy = 2 * y / (b * b); break;
    case 1: zx = c * c / z * x / (a * a); zy = c * c / z * y / (b * b); break;
    case 2: zx = -c * c / z * x / (a * a); zy = -c * c / z * y / (b * b); break;
    default: zx = 0; zy = 0; break;
    }
}

}  // namespace

__global__ void po_grid_kernel(GridSpec g, double *__restrict__ out)
{
    const long n = (long)g.ncx * g.ncy;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int i = (int)(idx / g.ncy), j = (int)(idx - (long)i * g.ncy);
    double x = 0, y = 0, z = 0, nx = 0, ny = 0, nz = 1, area = 0;
    if (g.gmode == 0) {
        const double dx = (g.lxu1 - g.lxu0) / (g.ncx - 1), dy = (g.lyv1 - g.lyv0) / (g.ncy - 1);
        const bool centred = g.type == 0 || g.type == 1;   // quadrics offset by gcenter; ellipsoids, planes not
        x = i * dx + g.lxu0 + (centred ? g.gcx : 0.0);
        y = j * dy + g.lyv0 + (centred ? g.gcy : 0.0);
        double q[3];
        quadric_d(g.type, g.a, g.b, g.c, x, y, z, q);
        if (g.type == 3) {
            nx = 0; ny = 0; nz = g.nfac;
            area = dx * dy;
        } else {
            const double nrm = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            nx = g.nfac * q[0] / nrm; ny = g.nfac * q[1] / nrm; nz = g.nfac * q[2] / nrm;
            area = nrm * dx * dy;
        }
    } else if (g.gmode == 1) {
        const double du0 = (g.lxu1 - g.lxu0) / (g.ncx - 1), dv = (g.lyv1 - g.lyv0) / g.ncy;
        const double rot = g.rot * kPiD / 180, cr = cos(rot), sr = sin(rot);
        const double v = (j * dv + g.lyv0) * kPiD / 180, sv = sin(v), cv = cos(v);
        const double ef = sqrt(1 - g.ecc * g.ecc * sv * sv);
        const double duv = du0 / ef;
        const double u = i * duv + g.lxu0 / ef;
        const double dudv = u / (ef * ef) * g.ecc * g.ecc * cv * sv;
        x = u * cv * cr - u * sv * sr + g.gcx;
        y = u * cv * sr + u * sv * cr + g.gcy;
        double q[3];
        quadric_d(g.type, g.a, g.b, g.c, x, y, z, q);
        if (g.type == 3) {
            nx = 0; ny = 0; nz = g.nfac;
            area = u * duv * dv * kPiD / 180;
        } else {
            const double nrm = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            nx = g.nfac * q[0] / nrm; ny = g.nfac * q[1] / nrm; nz = g.nfac * q[2] / nrm;
            // |dQ/du x dQ/dv| with Q(u, v) = (x, y, z(x, y))
            const double xu = cv * cr - sv * sr;
            const double xv = cv * cr * dudv - u * sv * cr - sv * sr * dudv - u * cv * sr;
            const double yu = cv * sr + sv * cr;
            const double yv = cv * sr * dudv - u * sv * sr + sv * cr * dudv + u * cv * cr;
            double zx, zy;
            slope_d(g.type, g.a, g.b, g.c, x, y, z, zx, zy);
            const double zu = zx * xu + zy * yu, zv = zx * xv + zy * yv;
            const double cx = yu * zv - zu * yv, cy = zu * xv - xu * zv, cz = xu * yv - yu * xv;
            area = sqrt(cx * cx + cy * cy + cz * cz) * duv * dv * kPiD / 180;
        }
    } else {
        const double dA = (g.lxu1 - g.lxu0) / (g.ncx - 1), dE = (g.lyv1 - g.lyv0) / (g.ncy - 1);
        const double az = i * dA + g.lxu0, el = j * dE + g.lyv0;
        x = az; y = el; z = 0; nx = 0; ny = 0; nz = 1;
        if (g.spheric) {
            x = sqrt(az * az + el * el) * kPiD / 180;
            y = atan2(el, az);
            if (y != y) y = 0;
        }
        area = cos(el * kPiD / 180) * dA * dE * kPiD * kPiD / 180 / 180;
    }
    if (g.transform) {
        const double p[3] = {x, y, z}, q[3] = {nx, ny, nz};
        double po[3], qo[3];
        for (int r = 0; r < 3; ++r) {
            po[r] = g.m[r * 4] * p[0] + g.m[r * 4 + 1] * p[1] + g.m[r * 4 + 2] * p[2] + g.m[r * 4 + 3];
            qo[r] = g.m[r * 4] * q[0] + g.m[r * 4 + 1] * q[1] + g.m[r * 4 + 2] * q[2];
        }
        x = po[0]; y = po[1]; z = po[2];
        nx = qo[0]; ny = qo[1]; nz = qo[2];
    }
    out[idx] = x;
    out[n + idx] = y;
    out[2 * n + idx] = z;
    out[3 * n + idx] = nx;
    out[4 * n + idx] = ny;
    out[5 * n + idx] = nz;
    out[6 * n + idx] = area;
}

// Normal-direction surface error: point += s_i * n_i.
__global__ void po_grid_error_kernel(long n, const double *__restrict__ s, double *__restrict__ out)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const double d = s[idx];
    out[idx] += d * out[3 * n + idx];
    out[n + idx] += d * out[4 * n + idx];
    out[2 * n + idx] += d * out[5 * n + idx];
}

int generate_grid_dev(const reflparams &r, double *out7, bool transform, bool spheric, cudaStream_t s)
{
    if (!r.n_cells || r.n_cells[0] < 1 || r.n_cells[1] < 1) return fail(1, "bad n_cells");
    if (!out7) return fail(1, "null output buffer");
    if (r.gmode < 0 || r.gmode > 2) return fail(1, "gmode must be 0 (xy), 1 (uv) or 2 (AoE)");
    if (!r.coeffs || !r.lxu || !r.lyv || !r.gcenter || (transform && !r.transf)) return fail(1, "null reflparams array");
    GridSpec g{};
    g.type = r.type;
    g.gmode = r.gmode;
    g.ncx = r.n_cells[0];
    g.ncy = r.n_cells[1];
    g.nfac = r.flip ? -1 : 1;
    g.spheric = spheric ? 1 : 0;
    g.transform = transform ? 1 : 0;
    g.a = r.coeffs[0];
    g.b = r.coeffs[1];
    g.c = r.coeffs[2];
    g.lxu0 = r.lxu[0];
    g.lxu1 = r.lxu[1];
    g.lyv0 = r.lyv[0];
    g.lyv1 = r.lyv[1];
    g.gcx = r.gcenter[0];
    g.gcy = r.gcenter[1];
    g.ecc = r.ecc_uv;
    g.rot = r.rot_uv;
    if (transform)
        for (int q = 0; q < 12; ++q) g.m[q] = r.transf[q];
    const long n = (long)g.ncx * g.ncy;
    const unsigned nblk = (unsigned)((n + 255) / 256);
    po_grid_kernel<<<nblk, 256, 0, s>>>(g, out7);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(2, std::string("grid kernel launch: ") + cudaGetErrorString(e));
    note_launches(1);
    if (r.rms > 0) {
        std::vector<double> dev(n);
        std::mt19937 gen(r.rms_seed);
        for (long i = 0; i < n; ++i) {
            std::normal_distribution<double> dist(0.0, r.rms);
            dev[i] = dist(gen);
        }
        double *d = nullptr;
        if (int rc = po::scratch_alloc(reinterpret_cast<void **>(&d), sizeof(double) * n, s)) return rc;
        e = cudaMemcpyAsync(d, dev.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            po_grid_error_kernel<<<nblk, 256, 0, s>>>(n, d, out7);
            e = cudaGetLastError();
            if (e == cudaSuccess) note_launches(1);
        }
        cudaError_t e2 = cudaFreeAsync(d, s);
        // the pageable source of the copy must outlive it
        cudaError_t e3 = cudaStreamSynchronize(s);
        if (e != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
            return fail(2, std::string("surface error: ") +
                               cudaGetErrorString(e != cudaSuccess ? e : (e2 != cudaSuccess ? e2 : e3)));
    }
    return 0;
}

}  // namespace po
