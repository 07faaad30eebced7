// po_grid_dev.cu -- FP64 reflector grid generation on the device.
//
// The same formulas as the host generator po_grid.cpp (reference
// src/common/InterfaceReflector.cpp: paraboloid xy / uv :84-135, :166-244,
// hyperboloid :271-322, :353-434, ellipsoid :460-509, :540-621, plane xy / uv /
// AoE :645-686, :712-768, :794-849, 4x4 transform :35-57), one thread per grid
// point, written straight into the 7-row device layout the propagation entry
// points take (x, y, z, nx, ny, nz, area; index i*ncy + j). The optional
// surface error (:852-866) keeps the reference's random sequence, drawn on
// the device (po_mt_normals_kernel): mt19937 seeded with rms_seed and a fresh
// normal distribution per point (src/include/Random.h:112-116), applied along
// the normals by a second kernel.
//
// The correlated surface error (po_correlated_error_dev) is a spectral
// synthesis over random modes drawn from the same generator, evaluated on
// the device at every grid point.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

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
        double *d = nullptr;
        int *err = error_word();
        if (!err) return fail(2, "could not allocate the device error word");
        if (int rc = scratch_alloc(reinterpret_cast<void **>(&d), sizeof(double) * n, s)) return rc;
        int rc = normal_deviates_dev((unsigned)r.rms_seed, n, r.rms, d, err, s);
        if (!rc) {
            po_grid_error_kernel<<<nblk, 256, 0, s>>>(n, d, out7);
            e = cudaGetLastError();
            if (e == cudaSuccess) note_launches(1);
            else rc = fail(2, std::string("surface error: ") + cudaGetErrorString(e));
        }
        scratch_free(d, s);
        return rc;
    }
    return 0;
}

// ------------------------------------------------- mt19937 normal deviates
//
// MT19937 (Matsumoto and Nishimura, 1998) and the reference's draw of one
// normal deviate per fresh distribution: a double in [0, 1) from two
// outputs, low word first, (w0 + w1 2^32) 2^-64 (at most the double below 1);
// Marsaglia's polar method, x, y = 2U - 1 until 0 < r2 = x^2 + y^2 <= 1, then
// y sqrt(-2 ln r2 / r2) stdev, the other deviate of the pair dropped. So each
// attempt takes four outputs, and a block of 624 outputs is exactly 156
// attempts. One CTA: per block, the twist in three phases (each phase reads
// only words that are old or already final), the tempering (thread t holds
// output t), the 156 attempts in parallel, and a warp-ballot scan that
// places the accepted deviates in order.

namespace {

constexpr int kMtN = 624;
constexpr int kMtThreads = 640;

__device__ __forceinline__ uint32_t mt_twist(uint32_t cur, uint32_t next, uint32_t tap)
{
    const uint32_t y = (cur & 0x80000000u) | (next & 0x7fffffffu);
    return tap ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ __forceinline__ double mt_canonical(uint32_t w0, uint32_t w1)
{
    const double u = __dmul_rn(__dadd_rn((double)w0, __dmul_rn((double)w1, 4294967296.0)), 0x1p-64);
    return u < 1.0 ? u : 1.0 - 0x1p-53;
}

}  // namespace

__global__ void __launch_bounds__(kMtThreads)
po_mt_normals_kernel(unsigned seed, long n, double stdev, double *__restrict__ out, int *__restrict__ err)
{
    __shared__ uint32_t mt[kMtN];
    __shared__ int warp_ok[kMtThreads / 32];
    __shared__ int warp_off[kMtThreads / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) {
        uint32_t v = seed;
        mt[0] = v;
        for (int i = 1; i < kMtN; ++i) {
            v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)i;
            mt[i] = v;
        }
    }
    __syncthreads();
    long count = 0;   // block-uniform
    // 156 attempts a block accept about 122.5 deviates on average: the bound
    // is never reached in practice, and ends the loop if it were
    const long max_blocks = n / 100 + 64;
    for (long b = 0; b < max_blocks && count < n; ++b) {
        uint32_t v = 0;
        if (t < 227) v = mt_twist(mt[t], mt[t + 1], mt[t + 397]);
        __syncthreads();
        if (t < 227) mt[t] = v;
        __syncthreads();
        if (t >= 227 && t < 454) v = mt_twist(mt[t], mt[t + 1], mt[t - 227]);
        __syncthreads();
        if (t >= 227 && t < 454) mt[t] = v;
        __syncthreads();
        if (t >= 454 && t < 623) v = mt_twist(mt[t], mt[t + 1], mt[t - 227]);
        else if (t == 623) v = mt_twist(mt[623], mt[0], mt[396]);
        __syncthreads();
        if (t >= 454 && t < kMtN) mt[t] = v;
        __syncthreads();
        uint32_t w = 0;
        if (t < kMtN) {
            w = mt[t];
            w ^= w >> 11;
            w ^= (w << 7) & 0x9d2c5680u;
            w ^= (w << 15) & 0xefc60000u;
            w ^= w >> 18;
        }
        // attempt a = t / 4 takes the outputs of threads 4a .. 4a + 3 (one warp)
        const int base = lane & ~3;
        const uint32_t w0 = __shfl_sync(0xffffffffu, w, base), w1 = __shfl_sync(0xffffffffu, w, base + 1);
        const uint32_t w2 = __shfl_sync(0xffffffffu, w, base + 2), w3 = __shfl_sync(0xffffffffu, w, base + 3);
        bool ok = false;
        double val = 0.0;
        if ((t & 3) == 0 && t < kMtN) {
            const double x = __dsub_rn(__dmul_rn(2.0, mt_canonical(w0, w1)), 1.0);
            const double y = __dsub_rn(__dmul_rn(2.0, mt_canonical(w2, w3)), 1.0);
            const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
            ok = r2 <= 1.0 && r2 != 0.0;
            if (ok) val = __dmul_rn(__dmul_rn(y, __dsqrt_rn(__ddiv_rn(__dmul_rn(-2.0, log(r2)), r2))), stdev);
        }
        const unsigned ball = __ballot_sync(0xffffffffu, ok);
        if (lane == 0) warp_ok[warp] = __popc(ball);
        __syncthreads();
        if (t == 0) {
            int o = 0;
            for (int q = 0; q < kMtThreads / 32; ++q) {
                warp_off[q] = o;
                o += warp_ok[q];
            }
        }
        __syncthreads();
        if (ok) {
            const long at = count + warp_off[warp] + __popc(ball & ((1u << lane) - 1u));
            if (at < n) out[at] = val;
        }
        count += warp_off[kMtThreads / 32 - 1] + warp_ok[kMtThreads / 32 - 1];
        __syncthreads();
    }
    if (t == 0 && count < n) atomicExch(err, kErrRngBound);
}

int normal_deviates_dev(unsigned seed, long n, double stdev, double *out, int *err, cudaStream_t s)
{
    if (n <= 0) return 0;
    po_mt_normals_kernel<<<1, kMtThreads, 0, s>>>(seed, n, stdev, out, err);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(2, std::string("normal deviates: ") + cudaGetErrorString(e));
    note_launches(1);
    return 0;
}

// ------------------------------------------------- correlated surface error

// Modes of the synthesis from four standard normal deviates each:
// (kx, ky) = (g0, g1) / corr_len, phase atan2(g2, g3).
__global__ void po_modes_kernel(int m, const double *__restrict__ g, double inv_len, double *__restrict__ modes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    modes[i] = g[4 * i] * inv_len;
    modes[m + i] = g[4 * i + 1] * inv_len;
    modes[2 * m + i] = atan2(g[4 * i + 2], g[4 * i + 3]);
}

// delta_i = scale sum_m cos(kx_m x_i + ky_m y_i + ph_m), modes in order,
// staged through shared memory 256 at a time; with `apply`, the point also
// moves by delta_i along its normal.
__global__ void __launch_bounds__(256)
po_correlated_kernel(long n, double *__restrict__ g7, int m, const double *__restrict__ modes, double scale,
                     double *__restrict__ delta, int apply)
{
    __shared__ double sk[3][256];
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const double x = i < n ? g7[i] : 0.0, y = i < n ? g7[n + i] : 0.0;
    double sum = 0.0;
    for (int c = 0; c < m; c += 256) {
        const int cnt = min(256, m - c);
        __syncthreads();
        if ((int)threadIdx.x < cnt)
            for (int q = 0; q < 3; ++q) sk[q][threadIdx.x] = modes[q * m + c + threadIdx.x];
        __syncthreads();
        for (int j = 0; j < cnt; ++j) sum += cos(sk[0][j] * x + sk[1][j] * y + sk[2][j]);
    }
    if (i >= n) return;
    const double d = scale * sum;
    if (delta) delta[i] = d;
    if (apply) {
        g7[i] += d * g7[3 * n + i];
        g7[n + i] += d * g7[4 * n + i];
        g7[2 * n + i] += d * g7[5 * n + i];
    }
}

int correlated_error_dev(long n, double *g7, double rms, double corr_len, unsigned seed, int n_modes, double *delta,
                         int apply, cudaStream_t s)
{
    if (n < 0 || n_modes < 1 || !(corr_len > 0.0) || !(rms >= 0.0)) return fail(1, "bad surface-error arguments");
    if (n > 0 && !g7) return fail(1, "null grid");
    if (n == 0) return 0;
    int *err = error_word();
    if (!err) return fail(2, "could not allocate the device error word");
    double *g = nullptr, *modes = nullptr;
    int rc = 0;
    if ((rc = scratch_alloc(reinterpret_cast<void **>(&g), sizeof(double) * 4 * n_modes, s)) ||
        (rc = scratch_alloc(reinterpret_cast<void **>(&modes), sizeof(double) * 3 * n_modes, s))) {
        scratch_free(g, s);
        return rc;
    }
    rc = normal_deviates_dev(seed, 4L * n_modes, 1.0, g, err, s);
    if (!rc) {
        po_modes_kernel<<<(n_modes + 127) / 128, 128, 0, s>>>(n_modes, g, 1.0 / corr_len, modes);
        po_correlated_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
            n, g7, n_modes, modes, rms * sqrt(2.0 / n_modes), delta, apply);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(2, std::string("surface error: ") + cudaGetErrorString(e));
        else note_launches(2);
    }
    scratch_free(g, s);
    scratch_free(modes, s);
    return rc;
}

}  // namespace po
