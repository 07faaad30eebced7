// po_fitgauss_dev.cu -- Gaussian fit to a beam pattern, on the device.
//
// The reference's fitGaussAbs (src/PyPO/FitGauss.py:67-163), called by
// System.fitGaussAbs and System.calcMainBeam (src/PyPO/System.py:1828-1906):
//
//   1. f = |E_c| / max |E_c|; the fitted pattern is f (LIN) or 20 log10 f
//      (dB), the mask its points at or above the threshold (:88-97);
//   2. from the pattern's peak, the extent of the connected run of masked
//      points along the peak's row and column (MatUtils.py:9-57
//      findConnectedSubsets) bounds a window; masked points strictly inside
//      it are the fit region (:99-120);
//   3. initial parameters from the region's image moments (calcEstimates,
//      FitGauss.py:13-65);
//   4. a downhill-simplex minimisation (po_nm.h, scipy's fmin) of the misfit
//      |1 - (sum f Psi)^2 / (sum f^2 sum Psi^2)| over the region (GaussAbs,
//      :165-195), Psi the rotated elliptical Gaussian of generateGauss
//      (:197-228), in the pattern's scale;
//   5. with a ratio, repeated with the threshold raised by 0.5 dB per round
//      (from the third round on, while below -3 dB) until the fitted
//      Gaussian's power sum over the plain pattern's is below the ratio
//      (:126-161).
//
// The grid is the surface's own (generateGrid without transform; x, y rows
// of the 7-row device layout). Every pass over the points is one kernel with
// FP64 per-thread sums, a block tree, and the block partials added in block
// order by whichever block finishes last (a fixed grid, so each sum is
// deterministic). The host does the window's run lengths, the moment
// algebra and the simplex (po_nm.h, the code of po_fmin): its few hundred
// dependent FP64 operations per step run far faster on the host than on one
// GPU thread (GB300's FP64 units are few, and a lone thread waits out each
// latency). The fit region's points are compacted once per minimisation;
// each launch then evaluates every point the current simplex step may ask
// for (reflection with its expansion and both contractions; all of a
// shrink's vertices; the whole initial simplex), so a step costs one round
// trip. A point's sums do not depend on the batch it is in.
//
// Kept from the reference on purpose, with their effects:
//   * the window's corners are read as x[min(cols), i0], x[max(cols), i0],
//     y[j0, min(rows)], y[j0, max(rows)] with the row and column roles of
//     findConnectedSubsets' result crossed (the reference notes that this
//     assumes xy grids); negative indices wrap and indices past the end are
//     an error, as numpy's are;
//   * an empty window region falls back to an integer array of ones used as
//     an index, which selects grid row 1 (repeated; the repetition cancels
//     in every ratio), so the fit then runs on row 1 (on an xy grid x is
//     constant along a row and that fit is decided by rounding residue);
//   * the first of the ratio rounds uses the plain mask, later ones the
//     windowed one; a pattern whose ratio never drops below the limit loops for
//     ever in the reference; here the call returns an error once a round
//     would only repeat the previous one.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <string>
#include <vector>

#include "po_internal.h"
#include "po_nm.h"

namespace po {

namespace {

constexpr int kFgThreads = 256;
constexpr int kFgBlocks = 152;
constexpr int kFgMaxSums = 6;
constexpr int kScaleLin = 0, kScaleAmp = 1, kScaleDb = 2;

// Gaussian coefficients of a parameter vector (x0, y0, xs, ys, theta, amp),
// in the reference's order of operations (generateGauss, FitGauss.py:213-215).
struct Gauss {
    double a, b, c, xs, ys;
};

Gauss gauss_of(const double *p)
{
    const double x0 = p[0], y0 = p[1], th = p[4];
    const double ct = std::cos(th), st = std::sin(th), s2 = std::sin(2 * th);
    Gauss g;
    g.a = ct * ct / (2 * (x0 * x0)) + st * st / (2 * (y0 * y0));
    g.c = s2 / (4 * (x0 * x0)) - s2 / (4 * (y0 * y0));
    g.b = st * st / (2 * (x0 * x0)) + ct * ct / (2 * (y0 * y0));
    g.xs = p[2];
    g.ys = p[3];
    return g;
}

// Psi at (x, y): exp(-(a dx^2 + 2c dx dy + b dy^2)) (LIN) or 20 log10 of it
// (dB), products and sums rounded one by one as numpy evaluates them.
__device__ __forceinline__ double gauss_at(const Gauss &g, int scale, double x, double y)
{
    const double dx = __dsub_rn(x, g.xs), dy = __dsub_rn(y, g.ys);
    const double t1 = __dmul_rn(g.a, __dmul_rn(dx, dx));
    const double t2 = __dmul_rn(__dmul_rn(__dmul_rn(2.0, g.c), dx), dy);
    const double t3 = __dmul_rn(g.b, __dmul_rn(dy, dy));
    const double e = exp(-__dadd_rn(__dadd_rn(t1, t2), t3));
    return scale == kScaleDb ? __dmul_rn(20.0, log10(e)) : e;
}

// The last block to finish adds the block partials (in block order) into res.
template <int NS>
__device__ void finish_sums(const double (&s)[NS], double *part, double *res, unsigned *count)
{
    __shared__ double sh[NS][kFgThreads];
    __shared__ bool last;
    for (int q = 0; q < NS; ++q) sh[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int w = kFgThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < NS; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int q = 0; q < NS; ++q) part[(long)blockIdx.x * NS + q] = sh[q][0];
        __threadfence();
        last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    if (threadIdx.x < NS) {
        double v = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) v += __ldcg(&part[(long)b * NS + threadIdx.x]);
        res[threadIdx.x] = v;
    }
    if (threadIdx.x == 0) *count = 0u;
}

// (value, index) maximum, first index on ties, NaN above every number (as
// numpy's argmax and max treat them).
__device__ __forceinline__ bool beats(double v, long i, double w, long j)
{
    const bool vn = v != v, wn = w != w;
    if (vn != wn) return vn;
    if (!vn && v != w) return v > w;
    return i < j;
}

__device__ void finish_argmax(double v, long i, double sum, double *part, double *res, unsigned *count)
{
    __shared__ double sv[kFgThreads], ss[kFgThreads];
    __shared__ long si[kFgThreads];
    __shared__ bool last;
    sv[threadIdx.x] = v;
    si[threadIdx.x] = i;
    ss[threadIdx.x] = sum;
    __syncthreads();
    for (int w = kFgThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const int o = threadIdx.x + w;
            if (beats(sv[o], si[o], sv[threadIdx.x], si[threadIdx.x])) {
                sv[threadIdx.x] = sv[o];
                si[threadIdx.x] = si[o];
            }
            ss[threadIdx.x] += ss[o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3L * blockIdx.x] = sv[0];
        part[3L * blockIdx.x + 1] = (double)si[0];
        part[3L * blockIdx.x + 2] = ss[0];
        __threadfence();
        last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    double bv = __ldcg(&part[0]), bs = 0.0;
    long bi = (long)__ldcg(&part[1]);
    for (unsigned b = 0; b < gridDim.x; ++b) {
        const double w = __ldcg(&part[3L * b]);
        const long j = (long)__ldcg(&part[3L * b + 1]);
        if (beats(w, j, bv, bi)) {
            bv = w;
            bi = j;
        }
        bs += __ldcg(&part[3L * b + 2]);
    }
    res[0] = bv;
    res[1] = (double)bi;
    res[2] = bs;
    *count = 0u;
}

// |E_c| into a; res[0] = max |E_c| (NaN if any is NaN).
__global__ void __launch_bounds__(kFgThreads)
fg_abs_kernel(long n, const double *__restrict__ fr, const double *__restrict__ fi, double *__restrict__ a,
              double *part, double *res, unsigned *count)
{
    double m = -1.0;
    long mi = n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = hypot(fr[i], fi ? fi[i] : 0.0);
        a[i] = v;
        if (beats(v, i, m, mi)) {
            m = v;
            mi = i;
        }
    }
    finish_argmax(m, mi, 0.0, part, res, count);
}

// Normalised pattern: nf = a / amax, fit = nf (LIN) or 20 log10 nf (dB).
// res[0] = max fit, res[1] = its first index, res[2] = sum nf^2.
__global__ void __launch_bounds__(kFgThreads)
fg_pattern_kernel(long n, const double *__restrict__ a, const double *__restrict__ amax, int scale,
                  double *__restrict__ fit, double *part, double *res, unsigned *count)
{
    const double m = *amax;
    double best = -CUDART_INF;
    long bi = n;
    double s = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double nf = a[i] / m;
        const double v = scale == kScaleDb ? __dmul_rn(20.0, log10(nf)) : nf;
        fit[i] = v;
        s += __dmul_rn(nf, nf);
        if (beats(v, i, best, bi)) {
            best = v;
            bi = i;
        }
    }
    finish_argmax(best, bi, s, part, res, count);
}

// Selection of the points the sums run over:
//   mode 0: fit >= thr;
//   mode 1: fit >= thr and xlo < x < xhi and ylo < y < yhi;
//   mode 2: grid row 1 (i / ncy == 1).
// res[0] = number of points selected.
struct Window {
    double xlo, xhi, ylo, yhi;
};

__global__ void __launch_bounds__(kFgThreads)
fg_select_kernel(long n, int ncy, const double *__restrict__ g7, const double *__restrict__ fit, double thr,
                 int mode, Window w, unsigned char *__restrict__ sel, double *part, double *res, unsigned *count)
{
    double c[1] = {0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        bool on;
        if (mode == 2) {
            on = i / ncy == 1;
        } else {
            on = fit[i] >= thr;
            if (mode == 1) {
                const double x = g7[i], y = g7[n + i];
                on = on && x > w.xlo && x < w.xhi && y > w.ylo && y < w.yhi;
            }
        }
        sel[i] = on ? 1 : 0;
        c[0] += on ? 1.0 : 0.0;
    }
    finish_sums<1>(c, part, res, count);
}

// Mask values along the peak's row (ncy bytes) and column (ncx bytes).
__global__ void fg_lines_kernel(int ncx, int ncy, long i0, long j0, const double *__restrict__ fit, double thr,
                                unsigned char *__restrict__ out)
{
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ncy) out[k] = fit[i0 * ncy + k] >= thr ? 1 : 0;
    else if (k < (long)ncy + ncx) out[k] = fit[(k - ncy) * ncy + j0] >= thr ? 1 : 0;
}

// Image moments of the selection: sum f, x f, y f, x^2 f, y^2 f, x y f.
__global__ void __launch_bounds__(kFgThreads)
fg_moments_kernel(long n, const double *__restrict__ g7, const double *__restrict__ fit,
                  const unsigned char *__restrict__ sel, double *part, double *res, unsigned *count)
{
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (!sel[i]) continue;
        const double x = g7[i], y = g7[n + i], f = fit[i];
        s[0] += f;
        s[1] += __dmul_rn(x, f);
        s[2] += __dmul_rn(y, f);
        s[3] += __dmul_rn(__dmul_rn(x, x), f);
        s[4] += __dmul_rn(__dmul_rn(y, y), f);
        s[5] += __dmul_rn(__dmul_rn(x, y), f);
    }
    finish_sums<6>(s, part, res, count);
}

// Power of the linear Gaussian over every point: sum Psi^2.
__global__ void __launch_bounds__(kFgThreads)
fg_power_kernel(long n, const double *__restrict__ g7, Gauss g, double *part, double *res, unsigned *count)
{
    double s[1] = {0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double p = gauss_at(g, kScaleLin, g7[i], g7[n + i]);
        s[0] += __dmul_rn(p, p);
    }
    finish_sums<1>(s, part, res, count);
}

// Order-preserving compaction of the selected points into (x, y, pattern)
// arrays; *count = how many. One CTA; thread t takes a contiguous chunk.
constexpr int kCompactThreads = 1024;

__global__ void __launch_bounds__(kCompactThreads)
fg_compact_kernel(long n, const unsigned char *__restrict__ sel, const double *__restrict__ g7,
                  const double *__restrict__ fit, double *__restrict__ cx, double *__restrict__ cy,
                  double *__restrict__ cf, long *__restrict__ count)
{
    __shared__ long offs[kCompactThreads];
    const long per = (n + kCompactThreads - 1) / kCompactThreads;
    const long b = min(n, (long)threadIdx.x * per), e = min(n, b + per);
    long c = 0;
    for (long i = b; i < e; ++i) c += sel[i] ? 1 : 0;
    offs[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        long acc = 0;
        for (int t = 0; t < kCompactThreads; ++t) {
            const long v = offs[t];
            offs[t] = acc;
            acc += v;
        }
        *count = acc;
    }
    __syncthreads();
    long o = offs[threadIdx.x];
    for (long i = b; i < e; ++i)
        if (sel[i]) {
            cx[o] = g7[i];
            cy[o] = g7[n + i];
            cf[o] = fit[i];
            ++o;
        }
}

// Overlap sums of up to kBatch Gaussians over the m compacted points: rows
// (sum f Psi, sum Psi^2, sum f^2) per Gaussian, the block that finishes last
// adding the block partials in block order. Each Gaussian's sums follow the
// same per-thread, per-block and cross-block order whatever else is in the
// batch.
constexpr int kBatch = 8;

struct GaussBatch {
    Gauss g[kBatch];
    int k;
};

__global__ void __launch_bounds__(kFgThreads)
fg_overlap_kernel(const long *__restrict__ count, const double *__restrict__ cx, const double *__restrict__ cy,
                  const double *__restrict__ cf, int scale, GaussBatch b, double *part, double *res,
                  unsigned *done)
{
    constexpr int kWarps = kFgThreads / 32;
    __shared__ double ws[3 * kBatch][kWarps];
    __shared__ bool last;
    const long m = *count;
    const int nq = 3 * b.k, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double s[3 * kBatch];
#pragma unroll
    for (int q = 0; q < 3 * kBatch; ++q) s[q] = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long)gridDim.x * blockDim.x) {
        const double f = cf[i], x = cx[i], y = cy[i];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) {
            if (k < b.k) {
                const double p = gauss_at(b.g[k], scale, x, y);
                s[3 * k] += __dmul_rn(f, p);
                s[3 * k + 1] += __dmul_rn(p, p);
                s[3 * k + 2] += __dmul_rn(f, f);
            }
        }
    }
    // per warp: a fixed shuffle tree; per block: warps in order
#pragma unroll
    for (int q = 0; q < 3 * kBatch; ++q) {
        if (q < nq) {
            double v = s[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) ws[q][wid] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < nq) {
        double v = 0.0;
        for (int w = 0; w < kWarps; ++w) v += ws[threadIdx.x][w];
        part[(long)blockIdx.x * 3 * kBatch + threadIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    if (threadIdx.x < nq) {
        double v = 0.0;
        for (unsigned bb = 0; bb < gridDim.x; ++bb) v += __ldcg(&part[(long)bb * 3 * kBatch + threadIdx.x]);
        res[threadIdx.x] = v;
    }
    if (threadIdx.x == 0) *done = 0u;
}

__global__ void fg_generate_kernel(long n, const double *__restrict__ g7, Gauss g, int scale, double *__restrict__ out)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = gauss_at(g, scale, g7[i], g7[n + i]);
}

// numpy's resolution of an index into an axis of length dim.
bool np_index(long r, long dim, long &out)
{
    if (r < -dim || r >= dim) return false;
    out = r < 0 ? r + dim : r;
    return true;
}

// Scratch of one fit, one allocation.
struct FitScratch {
    double *a = nullptr, *fit = nullptr, *part = nullptr, *res = nullptr;
    double *cx = nullptr, *cy = nullptr, *cf = nullptr, *opart = nullptr, *ores = nullptr;
    long *ncomp = nullptr;
    unsigned char *sel = nullptr, *lines = nullptr;
    unsigned *count = nullptr;
    void *base = nullptr;
};

class Fit {
public:
    Fit(int ncx, int ncy, const double *g7, cudaStream_t s) : ncx_(ncx), ncy_(ncy), n_((long)ncx * ncy), g7_(g7), s_(s) {}
    ~Fit()
    {
        if (sc_.base) cudaFreeAsync(sc_.base, s_);
    }

    int alloc()
    {
        const size_t nd = (size_t)n_ * sizeof(double);
        const size_t parts = sizeof(double) * kFgBlocks * kFgMaxSums;
        const size_t bytes = 5 * (nd + 256) + parts + sizeof(double) * (kFgBlocks + 1) * 3 * kBatch + 8 * 256 +
                             2 * ((size_t)n_ + 256) + (size_t)ncx_ + ncy_ + 256;
        if (int rc = po::scratch_alloc(reinterpret_cast<void **>(&sc_.base), bytes, s_)) return rc;
        char *p = static_cast<char *>(sc_.base);
        auto take = [&](size_t b) {
            char *q = p;
            p += (b + 255) / 256 * 256;
            return q;
        };
        sc_.a = reinterpret_cast<double *>(take(nd));
        sc_.fit = reinterpret_cast<double *>(take(nd));
        sc_.part = reinterpret_cast<double *>(take(parts));
        sc_.res = reinterpret_cast<double *>(take(sizeof(double) * 8));
        sc_.count = reinterpret_cast<unsigned *>(take(sizeof(unsigned)));
        sc_.cx = reinterpret_cast<double *>(take(nd));
        sc_.cy = reinterpret_cast<double *>(take(nd));
        sc_.cf = reinterpret_cast<double *>(take(nd));
        sc_.ncomp = reinterpret_cast<long *>(take(sizeof(long)));
        sc_.opart = reinterpret_cast<double *>(take(sizeof(double) * kFgBlocks * 3 * kBatch));
        sc_.ores = reinterpret_cast<double *>(take(sizeof(double) * 3 * kBatch));
        sc_.sel = reinterpret_cast<unsigned char *>(take((size_t)n_));
        sc_.lines = reinterpret_cast<unsigned char *>(take((size_t)ncx_ + ncy_));
        const cudaError_t e = cudaMemsetAsync(sc_.count, 0, sizeof(unsigned), s_);
        if (e != cudaSuccess) return fail(2, std::string("fit scratch: ") + cudaGetErrorString(e));
        return 0;
    }

    // Launch status, then the first k result words on the host.
    int read(double *h, int k, const char *what)
    {
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, sc_.res, sizeof(double) * k, cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
        if (e != cudaSuccess) return fail(2, std::string(what) + ": " + cudaGetErrorString(e));
        return 0;
    }

    int pattern(const double *fr, const double *fi, int scale, double &fit_max, long &imax, double &nf2)
    {
        double h[3];
        fg_abs_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(n_, fr, fi, sc_.a, sc_.part, sc_.res, sc_.count);
        note_launches(1);
        if (int rc = read(h, 1, "field magnitude")) return rc;
        if (!(h[0] > 0.0) || std::isinf(h[0]))
            return fail(1, "the field component is zero, NaN or infinite: its normalisation is undefined");
        // the maximum stays on the device (res[0]); copy it aside before res is reused
        double *amax = sc_.res + 4;
        cudaError_t e = cudaMemcpyAsync(amax, sc_.res, sizeof(double), cudaMemcpyDeviceToDevice, s_);
        if (e != cudaSuccess) return fail(2, std::string("field maximum: ") + cudaGetErrorString(e));
        fg_pattern_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(n_, sc_.a, amax, scale, sc_.fit, sc_.part, sc_.res,
                                                             sc_.count);
        note_launches(1);
        if (int rc = read(h, 3, "pattern")) return rc;
        fit_max = h[0];
        imax = (long)h[1];
        nf2 = h[2];
        return 0;
    }

    int select(double thr, int mode, const Window &w, double &count)
    {
        fg_select_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(n_, ncy_, g7_, sc_.fit, thr, mode, w, sc_.sel, sc_.part,
                                                            sc_.res, sc_.count);
        note_launches(1);
        return read(&count, 1, "fit region");
    }

    int lines(long i0, long j0, double thr, std::vector<unsigned char> &row, std::vector<unsigned char> &col)
    {
        const long k = (long)ncx_ + ncy_;
        fg_lines_kernel<<<(unsigned)((k + 255) / 256), 256, 0, s_>>>(ncx_, ncy_, i0, j0, sc_.fit, thr, sc_.lines);
        note_launches(1);
        std::vector<unsigned char> h((size_t)k);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), sc_.lines, (size_t)k, cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
        if (e != cudaSuccess) return fail(2, std::string("mask lines: ") + cudaGetErrorString(e));
        row.assign(h.begin(), h.begin() + ncy_);
        col.assign(h.begin() + ncy_, h.end());
        return 0;
    }

    int grid_value(int r, long flat, double &v)
    {
        cudaError_t e = cudaMemcpyAsync(&v, g7_ + (long)r * n_ + flat, sizeof(double), cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
        if (e != cudaSuccess) return fail(2, std::string("grid value: ") + cudaGetErrorString(e));
        return 0;
    }

    int moments(double *m6)
    {
        fg_moments_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(n_, g7_, sc_.fit, sc_.sel, sc_.part, sc_.res, sc_.count);
        note_launches(1);
        return read(m6, 6, "moments");
    }

    // The simplex from p0 over the current selection (fmin(GaussAbs, p0)).
    int fmin(const double *p0, int scale, double *popt)
    {
        fg_compact_kernel<<<1, kCompactThreads, 0, s_>>>(n_, sc_.sel, g7_, sc_.fit, sc_.cx, sc_.cy, sc_.cf, sc_.ncomp);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(2, std::string("fit region compaction: ") + cudaGetErrorString(e));
        NMState st;
        nm_init(st, 6, p0, 1e-4, 1e-4, 0, 0);
        double pts[kBatch][6], val[kBatch];
        int npts = 0;
        while (nm_next(st)) {
            int hit = -1;
            for (int q = 0; q < npts && hit < 0; ++q) {
                bool same = true;
                for (int c = 0; c < 6; ++c) same = same && pts[q][c] == st.x[c];
                if (same) hit = q;
            }
            if (hit < 0) {
                npts = batch(st, pts);
                if (int rc = values(scale, pts, npts, val)) return rc;
                hit = 0;   // the batch starts with the point asked for
            }
            nm_feed(st, val[hit]);
        }
        for (int c = 0; c < 6; ++c) popt[c] = st.sim[c];
        return 0;
    }

    // The point asked for, then the others this step may ask for next.
    static int batch(const NMState &st, double (*pts)[6])
    {
        const int n = st.n;
        int k = 0;
        for (int c = 0; c < n; ++c) pts[k][c] = st.x[c];
        ++k;
        if (st.phase == nm::kInit) {
            // st.k is the vertex asked for; the rest of the initial simplex follows
            for (int v = st.k + 1; v <= n && k < kBatch; ++v, ++k)
                for (int c = 0; c < n; ++c) pts[k][c] = st.sim[v * n + c];
        } else if (st.phase == nm::kReflect) {
            NMState t = st;
            nm::trial(t, 1.0 + 1.0 * 2.0, -(1.0 * 2.0), pts[k++]);
            nm::trial(t, 1.0 + 0.5 * 1.0, -(0.5 * 1.0), pts[k++]);
            nm::trial(t, 1.0 - 0.5, 0.5, pts[k++]);
        } else if (st.phase == nm::kShrink) {
            // st.k is the vertex asked for; later vertices move the same way from their old places
            for (int v = st.k + 1; v <= n && k < kBatch; ++v, ++k)
                for (int c = 0; c < n; ++c)
                    pts[k][c] = nm::add(st.sim[c], nm::mul(0.5, nm::sub(st.sim[v * n + c], st.sim[c])));
        }
        return k;
    }

    // GaussAbs (FitGauss.py:165-195) of each point, one launch.
    int values(int scale, const double (*pts)[6], int k, double *val)
    {
        GaussBatch b{};
        b.k = k;
        for (int q = 0; q < k; ++q) b.g[q] = gauss_of(pts[q]);
        fg_overlap_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(sc_.ncomp, sc_.cx, sc_.cy, sc_.cf, scale, b, sc_.opart,
                                                             sc_.ores, sc_.count);
        note_launches(1);
        double h[3 * kBatch];
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, sc_.ores, sizeof(double) * 3 * k, cudaMemcpyDeviceToHost, s_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
        if (e != cudaSuccess) return fail(2, std::string("overlap sums: ") + cudaGetErrorString(e));
        for (int q = 0; q < k; ++q) {
            const double c00 = h[3 * q] * h[3 * q] / h[3 * q + 2] / h[3 * q + 1];
            val[q] = std::fabs(1 - std::fabs(c00));
        }
        return 0;
    }

    int power(const double *p, double &pw)
    {
        fg_power_kernel<<<kFgBlocks, kFgThreads, 0, s_>>>(n_, g7_, gauss_of(p), sc_.part, sc_.res, sc_.count);
        note_launches(1);
        return read(&pw, 1, "Gaussian power");
    }

private:
    int ncx_, ncy_;
    long n_;
    const double *g7_;
    cudaStream_t s_;
    FitScratch sc_;
};

// calcEstimates (FitGauss.py:13-65) from the six moment sums.
void estimates(const double *m, double &x0, double &y0, double &xm, double &ym, double &theta)
{
    const double M0 = m[0];
    xm = m[1] / M0;
    ym = m[2] / M0;
    const double Mxx = m[3] / M0 - xm * xm;
    const double Myy = m[4] / M0 - ym * ym;
    const double Mxy = m[5] / M0 - xm * ym;
    const double D = 1 / (2 * (Mxx * Myy - Mxy * Mxy));
    const double a = Myy * D, b = Mxx * D, c = -Mxy * D;
    theta = 0.5 * std::atan(2 * c / (a - b));
    if (a - b > 0) theta += 3.14159265358979323846 / 2;
    const double p = std::sqrt((a - b) * (a - b) + 4 * (c * c));
    double X = 1 / (a + b - p), Y = 1 / (a + b + p);
    if (X <= 0 && Y > 0) {
        X = Y;
    } else if (Y <= 0 && X > 0) {
        Y = X;
    } else if (Y <= 0 && X <= 0) {
        X *= -1;
        Y *= -1;
    }
    x0 = std::sqrt(X);
    y0 = std::sqrt(Y);
}

// Length of the run of set values starting next to `at` and walking by `dir`.
long run_length(const std::vector<unsigned char> &v, long at, int dir)
{
    long k = 0;
    for (long i = at + dir; i >= 0 && i < (long)v.size() && v[i]; i += dir) ++k;
    return k;
}

}  // namespace

int fit_gauss_abs_dev(int ncx, int ncy, const double *g7, const double *fr, const double *fi, double thres, int scale,
                      int use_ratio, double ratio, double *popt, double *p0_out, cudaStream_t s)
{
    if (ncx < 1 || ncy < 1) return fail(1, "fit: grid must have at least one point per axis");
    if (!g7 || !fr || !popt) return fail(1, "fit: null grid, field or output");
    if (scale == kScaleAmp)
        return fail(1, "fit: scale AMP defines no Gaussian (the reference's generateGauss leaves Psi unset for it)");
    if (scale != kScaleLin && scale != kScaleDb) return fail(1, "fit: scale must be 0 (LIN) or 2 (dB)");
    if (use_ratio && std::isnan(ratio)) return fail(1, "fit: NaN ratio (the reference's loop never runs)");
    if (std::isnan(thres)) return fail(1, "fit: NaN threshold");

    Fit F(ncx, ncy, g7, s);
    if (int rc = F.alloc()) return rc;
    auto thr_of = [&](double t) { return scale == kScaleDb ? t : std::pow(10.0, t / 20); };

    double fit_max = 0.0, nf2 = 0.0;
    long imax = 0;
    if (int rc = F.pattern(fr, fi, scale, fit_max, imax, nf2)) return rc;
    const long i0 = imax / ncy, j0 = imax % ncy;

    // connected runs through the peak (findConnectedSubsets) and the window
    std::vector<unsigned char> row, col;
    if (int rc = F.lines(i0, j0, thr_of(thres), row, col)) return rc;
    const long nr_up = run_length(row, j0, +1), nr_lo = run_length(row, j0, -1);
    const long nc_up = run_length(col, i0, +1), nc_lo = run_length(col, i0, -1);
    const long rows_min = i0 - nr_lo, rows_max = i0 + nr_up;    // lims_row
    const long cols_min = j0 - nc_lo, cols_max = j0 + nc_up;    // lims_col
    long r0, r1, c0, c1, q0, q1, s0, s1;
    if (!np_index(cols_min, ncx, r0) || !np_index(cols_max, ncx, r1) || !np_index(i0, ncy, c0) ||
        !np_index(j0, ncx, q0) || !np_index(rows_min, ncy, s0) || !np_index(rows_max, ncy, s1))
        return fail(1, "fit: the window corners index past the grid (the reference raises IndexError here)");
    c1 = c0;
    q1 = q0;
    Window w{};
    if (int rc = F.grid_value(0, r0 * ncy + c0, w.xlo)) return rc;
    if (int rc = F.grid_value(0, r1 * ncy + c1, w.xhi)) return rc;
    if (int rc = F.grid_value(1, q0 * ncy + s0, w.ylo)) return rc;
    if (int rc = F.grid_value(1, q1 * ncy + s1, w.yhi)) return rc;

    double count;
    if (int rc = F.select(thr_of(thres), 1, w, count)) return rc;
    if (count == 0) {
        if (ncx < 2) return fail(1, "fit: empty fit region on a grid without row 1 (the reference raises IndexError)");
        if (int rc = F.select(0.0, 2, w, count)) return rc;
    }
    double m6[6];
    if (int rc = F.moments(m6)) return rc;
    double p0[6];
    estimates(m6, p0[0], p0[1], p0[2], p0[3], p0[4]);
    p0[5] = fit_max;
    if (p0_out)
        for (int q = 0; q < 6; ++q) p0_out[q] = p0[q];

    auto fmin = [&](double *out) { return F.fmin(p0, scale, out); };
    if (!use_ratio) return fmin(popt);

    // ratio rounds (FitGauss.py:126-161)
    double t = thres, cur = ratio;
    int num = 0;
    double last_thr = NAN;
    int last_mode = -1;
    double last_ratio = 0.0;
    while (cur >= ratio) {
        const double thr = thr_of(t);
        const int mode = num >= 1 ? 1 : 0;
        if (!(mode == last_mode && thr == last_thr)) {
            // a round with new inputs
            if (int rc = F.select(thr, mode, w, count)) return rc;
            if (int rc = fmin(popt)) return rc;
            double pw;
            if (int rc = F.power(popt, pw)) return rc;
            last_ratio = pw / nf2;
            last_mode = mode;
            last_thr = thr;
        } else if (num > 2) {
            return fail(4, "fit: the power ratio stays at or above the limit with the threshold at -3 dB "
                           "(the reference loops for ever here)");
        }
        cur = last_ratio;
        if (num > 1 && t < -3) t += 0.5;
        ++num;
    }
    return 0;
}

int generate_gauss_dev(long n, const double *g7, const double *popt, int scale, double *out, cudaStream_t s)
{
    if (n < 0) return fail(1, "negative point count");
    if (n > 0 && (!g7 || !out)) return fail(1, "null grid or output");
    if (!popt) return fail(1, "null parameters");
    if (scale != kScaleLin && scale != kScaleDb) return fail(1, "scale must be 0 (LIN) or 2 (dB)");
    if (n == 0) return 0;
    fg_generate_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, g7, gauss_of(popt), scale, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(2, std::string("Gaussian kernel: ") + cudaGetErrorString(e));
    note_launches(1);
    return 0;
}

}  // namespace po
