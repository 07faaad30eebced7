// po_eff_dev.cu -- far-field / aperture efficiency sums on the device (FP64).
//
// The reductions behind the reference's src/PyPO/Efficiencies.py: spillover
// (:90-115), taper (:117-145), cross-polar (:147-159) and main-beam (:161-177)
// efficiencies. One pass over the points accumulates, per thread in FP64 and
// then per block in shared memory, the sums they need; a one-block second
// pass adds the block partials in a fixed order (deterministic). The host
// forms the ratios. The aperture mask is the reference's _generateMask
// (:11-41): an ellipse |p - c|^2 < (o_x cos t)^2 + (o_y sin t)^2 with
// t = atan2(y, x) + pi, or a rectangle; only its outer condition is applied,
// as in the reference.
#include <cuda_runtime.h>

#include <string>

#include "po_internal.h"

namespace po {

constexpr int kEffSums = 10;
constexpr int kEffThreads = 256;
constexpr int kEffBlocks = 152;

struct Aperture {
    int shape;           // 0 none, 1 ellipse, 2 rectangle
    double c[2];         // centre
    double o[2];         // ellipse: outer semi-axes
    double rx[2], ry[2]; // rectangle: x and y bounds relative to the centre
};

__device__ __forceinline__ bool in_aperture(const Aperture &a, double x, double y)
{
    if (a.shape == 0) return true;
    const double dx = x - a.c[0], dy = y - a.c[1];
    if (a.shape == 1) {
        const double t = atan2(y, x) + 3.14159265358979323846;
        const double ox = a.o[0] * cos(t), oy = a.o[1] * sin(t);
        return dx * dx + dy * dy < ox * ox + oy * oy;
    }
    return dx > a.rx[0] && dx < a.rx[1] && dy > a.ry[0] && dy < a.ry[1];
}

// Sums, in order: 0 sum |f|^2 A, 1 sum_m |f|^2 A, 2 sum_m Re f A, 3 sum_m Im f A,
// 4 sum_m A, 5 sum |f|^2, 6 sum |g|^2, 7 max |f|^2, 8 max |g|^2, 9 count_m.
__global__ void __launch_bounds__(kEffThreads)
po_eff_partial_kernel(long n, const double *__restrict__ g7, const double *__restrict__ fr,
                      const double *__restrict__ fi, const double *__restrict__ gr, const double *__restrict__ gi,
                      Aperture ap, double *__restrict__ part)
{
    double s[kEffSums] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double x = g7[i], y = g7[n + i], A = g7[6 * n + i];
        const double re = fr[i], im = fi ? fi[i] : 0.0;
        const double f2 = re * re + im * im;
        s[0] += f2 * A;
        s[5] += f2;
        s[7] = fmax(s[7], f2);
        if (gr) {
            const double gim = gi ? gi[i] : 0.0;
            const double g2 = gr[i] * gr[i] + gim * gim;
            s[6] += g2;
            s[8] = fmax(s[8], g2);
        }
        if (in_aperture(ap, x, y)) {
            s[1] += f2 * A;
            s[2] += re * A;
            s[3] += im * A;
            s[4] += A;
            s[9] += 1.0;
        }
    }
    __shared__ double sh[kEffSums][kEffThreads];
    for (int q = 0; q < kEffSums; ++q) sh[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int w = kEffThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < kEffSums; ++q) {
                const double o = sh[q][threadIdx.x + w];
                sh[q][threadIdx.x] = (q == 7 || q == 8) ? fmax(sh[q][threadIdx.x], o) : sh[q][threadIdx.x] + o;
            }
        __syncthreads();
    }
    if (threadIdx.x < kEffSums) part[(long)blockIdx.x * kEffSums + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void po_eff_final_kernel(int nblk, const double *__restrict__ part, double *__restrict__ sums)
{
    const int q = threadIdx.x;
    if (q >= kEffSums) return;
    double v = 0.0;
    for (int b = 0; b < nblk; ++b) {
        const double o = part[(long)b * kEffSums + q];
        v = (q == 7 || q == 8) ? fmax(v, o) : v + o;
    }
    sums[q] = v;
}

int efficiency_sums_dev(long n, const double *g7, const double *fr, const double *fi, const double *gr,
                        const double *gi, int shape, const double *aper, double *sums, cudaStream_t s)
{
    if (n < 0) return fail(1, "negative point count");
    if (!sums) return fail(1, "null output buffer");
    if (n > 0 && (!g7 || !fr)) return fail(1, "null grid or field");
    if (!gr && gi) return fail(1, "second field: imaginary row without a real row");
    if (shape < 0 || shape > 2) return fail(1, "aperture shape must be 0 (none), 1 (ellipse) or 2 (rectangle)");
    if (shape != 0 && !aper) return fail(1, "null aperture parameters");
    Aperture ap{};
    ap.shape = shape;
    if (shape == 1) {
        ap.c[0] = aper[0]; ap.c[1] = aper[1]; ap.o[0] = aper[2]; ap.o[1] = aper[3];
    } else if (shape == 2) {
        ap.c[0] = aper[0]; ap.c[1] = aper[1];
        ap.rx[0] = aper[2]; ap.rx[1] = aper[3]; ap.ry[0] = aper[4]; ap.ry[1] = aper[5];
    }
    double *part = nullptr;
    if (int rc = po::scratch_alloc(reinterpret_cast<void **>(&part), sizeof(double) * kEffBlocks * kEffSums, s))
        return rc;
    po_eff_partial_kernel<<<kEffBlocks, kEffThreads, 0, s>>>(n, g7, fr, fi, gr, gi, ap, part);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        po_eff_final_kernel<<<1, 32, 0, s>>>(kEffBlocks, part, sums);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(part, s);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(2, std::string("efficiency kernels: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    note_launches(2);
    return 0;
}

}  // namespace po
