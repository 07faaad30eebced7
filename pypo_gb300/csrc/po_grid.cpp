// po_grid.cpp -- FP64 reflector grid generation (host).
//
// Restates the grid formulas of reference src/common/InterfaceReflector.cpp:
//   paraboloid xy / uv   :84-135, :166-244     hyperboloid xy / uv :271-322, :353-434
//   ellipsoid xy / uv    :460-509, :540-621    plane xy / uv / AoE :645-686, :712-768, :794-849
//   4x4 transform        :35-57 (points get the full affine map, normals the 3x3 part)
//   surface error        :852-866 (normal-direction displacement, mt19937 + a
//                         fresh normal distribution per point, as Random.h:112-116)
// Index order is row-major over (x/u, y/v): idx = i*ncy + j. u-v grids drop
// the upper v end point (dv = range / ncy). AoE grids with `spheric` hold
// (polar angle, azimuth) in radians.
#include <cmath>
#include <random>
#include <vector>

#include "../../include/po_gb300.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Pt {
    double x, y, z, nx, ny, nz, a;
};

inline void put(reflcontainer *c, int idx, const Pt &p)
{
    c->x[idx] = p.x;
    c->y[idx] = p.y;
    c->z[idx] = p.z;
    c->nx[idx] = p.nx;
    c->ny[idx] = p.ny;
    c->nz[idx] = p.nz;
    c->area[idx] = p.a;
}

// Quadric height and unnormalised outward normal for one (x, y).
// type 0: z = x^2/a^2 + y^2/b^2,          n ~ (-2x/a^2, -2y/b^2, 1)
// type 1: z = c sqrt(x^2/a^2 + y^2/b^2 + 1), n ~ (-2x/a^2, -2y/b^2, 2z/c^2)
// type 2: z = c sqrt(1 - x^2/a^2 - y^2/b^2), n ~ ( 2x/a^2,  2y/b^2, 2z/c^2)
// type 3: z = 0,                           n ~ (0, 0, 1)
inline void quadric(int type, double a, double b, double c, double x, double y,
                    double &z, double n[3])
{
    switch (type) {
    case 0:
        z = x * x / (a * a) + y * y / (b * b);
        n[0] = -2 * x / (a * a); n[1] = -2 * y / (b * b); n[2] = 1;
        break;
    case 1:
        z = c * std::sqrt(x * x / (a * a) + y * y / (b * b) + 1);
        n[0] = -2 * x / (a * a); n[1] = -2 * y / (b * b); n[2] = 2 * z / (c * c);
        break;
    case 2:
        z = c * std::sqrt(1 - x * x / (a * a) - y * y / (b * b));
        n[0] = 2 * x / (a * a); n[1] = 2 * y / (b * b); n[2] = 2 * z / (c * c);
        break;
    default:
        z = 0;
        n[0] = 0; n[1] = 0; n[2] = 1;
        break;
    }
}

// dz/dx and dz/dy of the quadric at (x, y, z), for the uv area element.
inline void slope(int type, double a, double b, double c, double x, double y, double z,
                  double &zx, double &zy)
{
    switch (type) {
    case 0: zx = 2 * x / (a * a); zy = 2 * y / (b * b); break;
    case 1: zx = c * c / z * x / (a * a); zy = c * c / z * y / (b * b); break;
    case 2: zx = -c * c / z * x / (a * a); zy = -c * c / z * y / (b * b); break;
    default: zx = 0; zy = 0; break;
    }
}

void grid_xy(const reflparams &r, reflcontainer *c, int nfac)
{
    const int ncx = r.n_cells[0], ncy = r.n_cells[1];
    const double a = r.coeffs[0], b = r.coeffs[1], cc = r.coeffs[2];
    const double dx = (r.lxu[1] - r.lxu[0]) / (ncx - 1);
    const double dy = (r.lyv[1] - r.lyv[0]) / (ncy - 1);
    // Quadrics are offset by gcenter; ellipsoids and planes are not.
    const bool centred = (r.type == 0 || r.type == 1);
    const double xc = centred ? r.gcenter[0] : 0.0, yc = centred ? r.gcenter[1] : 0.0;
    for (int i = 0; i < ncx; ++i) {
        const double x = i * dx + r.lxu[0] + xc;
        for (int j = 0; j < ncy; ++j) {
            const double y = j * dy + r.lyv[0] + yc;
            double z, n[3];
            quadric(r.type, a, b, cc, x, y, z, n);
            Pt p{x, y, z, 0, 0, 0, 0};
            if (r.type == 3) {
                p.nx = 0; p.ny = 0; p.nz = nfac * 1.0;
                p.a = dx * dy;
            } else {
                const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                p.nx = nfac * n[0] / nrm;
                p.ny = nfac * n[1] / nrm;
                p.nz = nfac * n[2] / nrm;
                p.a = nrm * dx * dy;
            }
            put(c, i * ncy + j, p);
        }
    }
}

void grid_uv(const reflparams &r, reflcontainer *c, int nfac)
{
    const int ncx = r.n_cells[0], ncy = r.n_cells[1];
    const double a = r.coeffs[0], b = r.coeffs[1], cc = r.coeffs[2];
    const double du0 = (r.lxu[1] - r.lxu[0]) / (ncx - 1);
    const double dv = (r.lyv[1] - r.lyv[0]) / ncy;
    const double ecc = r.ecc_uv;
    const double rot = r.rot_uv * kPi / 180;
    const double cr = std::cos(rot), sr = std::sin(rot);
    for (int i = 0; i < ncx; ++i) {
        for (int j = 0; j < ncy; ++j) {
            const double v = (j * dv + r.lyv[0]) * kPi / 180;
            const double sv = std::sin(v), cv = std::cos(v);
            const double ef = std::sqrt(1 - ecc * ecc * sv * sv);
            const double duv = du0 / ef;
            const double u = i * duv + r.lxu[0] / ef;
            const double dudv = u / (ef * ef) * ecc * ecc * cv * sv;
            const double x = u * cv * cr - u * sv * sr + r.gcenter[0];
            const double y = u * cv * sr + u * sv * cr + r.gcenter[1];
            double z, n[3];
            quadric(r.type, a, b, cc, x, y, z, n);
            Pt p{x, y, z, 0, 0, 0, 0};
            if (r.type == 3) {
                p.nx = 0; p.ny = 0; p.nz = nfac * 1.0;
                p.a = u * duv * dv * kPi / 180;
            } else {
                const double nrm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                p.nx = nfac * n[0] / nrm;
                p.ny = nfac * n[1] / nrm;
                p.nz = nfac * n[2] / nrm;
                // |dQ/du x dQ/dv| with Q(u, v) = (x, y, z(x, y)).
                const double xu = cv * cr - sv * sr;
                const double xv = cv * cr * dudv - u * sv * cr - sv * sr * dudv - u * cv * sr;
                const double yu = cv * sr + sv * cr;
                const double yv = cv * sr * dudv - u * sv * sr + sv * cr * dudv + u * cv * cr;
                double zx, zy;
                slope(r.type, a, b, cc, x, y, z, zx, zy);
                const double zu = zx * xu + zy * yu;
                const double zv = zx * xv + zy * yv;
                const double cx = yu * zv - zu * yv;
                const double cy = zu * xv - xu * zv;
                const double cz = xu * yv - yu * xv;
                p.a = std::sqrt(cx * cx + cy * cy + cz * cz) * duv * dv * kPi / 180;
            }
            put(c, i * ncy + j, p);
        }
    }
}

void grid_aoe(const reflparams &r, reflcontainer *c, bool spheric)
{
    const int ncx = r.n_cells[0], ncy = r.n_cells[1];
    const double dA = (r.lxu[1] - r.lxu[0]) / (ncx - 1);
    const double dE = (r.lyv[1] - r.lyv[0]) / (ncy - 1);
    for (int i = 0; i < ncx; ++i) {
        const double az = i * dA + r.lxu[0];
        for (int j = 0; j < ncy; ++j) {
            const double el = j * dE + r.lyv[0];
            Pt p{az, el, 0, 0, 0, 1, 0};
            if (spheric) {
                p.x = std::sqrt(az * az + el * el) * kPi / 180;
                p.y = std::atan2(el, az);
                if (p.y != p.y) p.y = 0;
            }
            p.a = std::cos(el * kPi / 180) * dA * dE * kPi * kPi / 180 / 180;
            put(c, i * ncy + j, p);
        }
    }
}

void transform_all(const reflparams &r, reflcontainer *c, int n)
{
    const double *m = r.transf;
    for (int i = 0; i < n; ++i) {
        const double p[3] = {c->x[i], c->y[i], c->z[i]};
        const double q[3] = {c->nx[i], c->ny[i], c->nz[i]};
        double po[3], qo[3];
        for (int row = 0; row < 3; ++row) {
            po[row] = m[row * 4] * p[0] + m[row * 4 + 1] * p[1] + m[row * 4 + 2] * p[2] + m[row * 4 + 3];
            qo[row] = m[row * 4] * q[0] + m[row * 4 + 1] * q[1] + m[row * 4 + 2] * q[2];
        }
        c->x[i] = po[0]; c->y[i] = po[1]; c->z[i] = po[2];
        c->nx[i] = qo[0]; c->ny[i] = qo[1]; c->nz[i] = qo[2];
    }
}

// n deviates N(0, stdev) in the reference's sequence: mt19937 seeded with
// `seed` and a fresh normal distribution per draw (Random.h:112-116).
void normal_deviates(unsigned seed, long n, double stdev, double *out)
{
    std::mt19937 gen(seed);
    for (long i = 0; i < n; ++i) {
        std::normal_distribution<double> dist(0.0, stdev);
        out[i] = dist(gen);
    }
}

void surface_error(const reflparams &r, reflcontainer *c, int n)
{
    std::vector<double> d(n);
    normal_deviates((unsigned)r.rms_seed, n, r.rms, d.data());
    for (int i = 0; i < n; ++i) {
        c->x[i] += d[i] * c->nx[i];
        c->y[i] += d[i] * c->ny[i];
        c->z[i] += d[i] * c->nz[i];
    }
}

}  // namespace

namespace po {

// Correlated surface error on the host, the twin of correlated_error_dev:
// delta_i = rms sqrt(2 / M) sum_m cos(kx_m x_i + ky_m y_i + ph_m) over M
// modes, kx, ky = g0, g1 / corr_len, ph = atan2(g2, g3) from four deviates
// N(0, 1) per mode in the reference's sequence; covariance
// rms^2 exp(-r^2 / (2 corr_len^2)). With `apply`, points move along their
// normals by delta.
int correlated_error_host(long n, double *g7, double rms, double corr_len, unsigned seed, int n_modes, double *delta,
                          int apply)
{
    if (n < 0 || n_modes < 1 || !(corr_len > 0.0) || !(rms >= 0.0) || (n > 0 && !g7)) return 1;
    std::vector<double> g(4 * (size_t)n_modes), kx(n_modes), ky(n_modes), ph(n_modes);
    normal_deviates(seed, 4L * n_modes, 1.0, g.data());
    for (int m = 0; m < n_modes; ++m) {
        kx[m] = g[4 * m] * (1.0 / corr_len);
        ky[m] = g[4 * m + 1] * (1.0 / corr_len);
        ph[m] = std::atan2(g[4 * m + 2], g[4 * m + 3]);
    }
    const double scale = rms * std::sqrt(2.0 / n_modes);
    for (long i = 0; i < n; ++i) {
        double sum = 0.0;
        for (int m = 0; m < n_modes; ++m) sum += std::cos(kx[m] * g7[i] + ky[m] * g7[n + i] + ph[m]);
        const double d = scale * sum;
        if (delta) delta[i] = d;
        if (apply)
            for (int c = 0; c < 3; ++c) g7[c * n + i] += d * g7[(3 + c) * n + i];
    }
    return 0;
}

}  // namespace po

// Host-side grid generation used by the drop-in entry points; the transform
// is applied per point after the surface parametrisation, as the reference does.
int po_grid_fill(const reflparams &r, reflcontainer *c, bool transform, bool spheric)
{
    if (!r.n_cells || r.n_cells[0] < 1 || r.n_cells[1] < 1 || !c || !c->x) return 1;
    const int n = r.n_cells[0] * r.n_cells[1];
    const int nfac = r.flip ? -1 : 1;
    if (r.gmode == 0) grid_xy(r, c, nfac);
    else if (r.gmode == 1) grid_uv(r, c, nfac);
    else if (r.gmode == 2) grid_aoe(r, c, spheric);
    else return 2;
    if (transform) transform_all(r, c, n);
    if (r.rms > 0) surface_error(r, c, n);
    return 0;
}
