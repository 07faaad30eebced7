// po_capi.cu -- the extern "C" entry points of libpo_gb300 (include/po_gb300.h).
#include <cuda_runtime.h>

#include <cstdio>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "po_internal.h"

namespace {

using po::fail;

std::mutex g_stream_mu;
cudaStream_t g_streams[64] = {};

// Frame half-extent (wavelengths) of this thread's last mixed-precision
// host-buffer call; 0 after any other call.
thread_local double t_extent = 0.0;
thread_local unsigned long long t_band = 0;

// Private non-blocking stream of the host-buffer entry points, one per device.
// The message of a device error code of the kernels (kErr* in po_kernels.cuh).
std::string device_error_text(int code)
{
    const char *what = code == po::kErrWaitTimeout     ? "a kernel gave up waiting for a tile copy"
                       : code == po::kErrBandOverflow ? "more near-tangent pairs than the band list holds"
                       : code == po::kErrRngBound     ? "the device normal generator ran past its bound"
                                                      : "a kernel reported an error";
    return std::string(what) + " (device error " + std::to_string(code) + "); results are invalid";
}

int lib_stream(cudaStream_t *s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(2, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(2, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_stream_mu);
    if (!g_streams[dev]) {
        e = cudaStreamCreateWithFlags(&g_streams[dev], cudaStreamNonBlocking);
        if (e != cudaSuccess) return fail(2, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    *s = g_streams[dev];
    return 0;
}

// *flag = 1 where any of the n values is non-zero (-0.0 counts as zero, NaN
// as non-zero). Every writer stores the same value.
__global__ void po_any_nonzero_kernel(const double *__restrict__ p, long n, int *__restrict__ flag)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        if (p[i] != 0.0) *flag = 1;
}

// Whether the magnetic currents (rows 6-11 of a device copy of 12 x ns
// currents) are all zero, which selects the M = 0 kernels. Checked on the
// device after the copy: a host scan of the rows would leave the GPU idle.
int device_m_is_zero(const double *d_cur, long ns, cudaStream_t s, bool &zero)
{
    int *flag = nullptr, h = 0;
    if (int rc = po::scratch_alloc(reinterpret_cast<void **>(&flag), sizeof(int), s)) return rc;
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        po_any_nonzero_kernel<<<2 * 152, 256, 0, s>>>(d_cur + 6 * ns, 6 * ns, flag);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (flag) cudaFreeAsync(flag, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(2, std::string("checking the magnetic currents: ") + cudaGetErrorString(e));
    po::note_launches(1);
    zero = h == 0;
    return 0;
}

// Whether the magnetic currents of a host-buffer call are all zero. A
// non-zero among the first kMPrefix values of the caller's host rows settles
// it at once (no device round trip: currents with M, the common case of a
// feed); otherwise the device checks all of them (device_m_is_zero), which
// keeps the host from scanning a large M = 0 block.
constexpr long kMPrefix = 4096;
int m_is_zero(const double *h_cur, const double *d_cur, long ns, cudaStream_t s, bool &zero)
{
    const double *m = h_cur + 6 * ns;
    const long n = std::min(6 * ns, kMPrefix);
    for (long i = 0; i < n; ++i)
        if (m[i] != 0.0) {   // -0.0 counts as zero, NaN as non-zero, as on the device
            zero = false;
            return 0;
        }
    return device_m_is_zero(d_cur, ns, s, zero);
}

#define CK(expr)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            rc = fail(2, std::string(#expr) + ": " + cudaGetErrorString(e_));             \
            goto done;                                                                    \
        }                                                                                 \
    } while (0)

// Stream-ordered scratch of a host-buffer call, from the library's own pool.
#define PO_SCRATCH(ptr, bytes)                                                            \
    do {                                                                                  \
        if ((rc = po::scratch_alloc(reinterpret_cast<void **>(&ptr), (bytes), s))) goto done; \
    } while (0)

// Host slots read back by a host-buffer call: the frame's half-extent and
// the number of near-tangent pairs. They are page-locked so that the copies
// stay asynchronous: a device-to-host copy into pageable memory makes the
// host wait for all of the call's kernels before it can queue the output
// copies. Pageable (the caller's slots) if pinning fails. One small
// page-locked block per calling thread, kept.
struct HostSlots {
    double extent;
    unsigned band;
};

HostSlots *host_slots(HostSlots *pageable)
{
    thread_local HostSlots *pinned = nullptr;
    thread_local bool tried = false;
    if (!tried) {
        tried = true;
        if (cudaMallocHost(&pinned, sizeof(HostSlots)) != cudaSuccess) {
            pinned = nullptr;
            (void)cudaGetLastError();
        }
    }
    HostSlots *h = pinned ? pinned : pageable;
    h->extent = 0.0;
    h->band = 0;
    return h;
}

// Host buffers in, host buffers out; synchronous.
int run_host(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
             const double *tgt7, double k, double eps, double t, int precision, double *out)
{
    po::clear_error();
    t_extent = 0.0;
    t_band = 0;
    {
        po::RunArgs v;
        v.mode = mode;
        v.ns = ns;
        v.src7 = src7;
        v.gmode = gmode;
        v.ncx = ncx;
        v.ncy = ncy;
        v.cur = cur;
        v.nt = nt;
        v.tgt7 = tgt7;
        v.k = k;
        v.epsilon = eps;
        v.t_dir = t;
        v.precision = precision;
        v.out = out;
        if (int rc = po::validate(v)) return rc;
    }
    if (nt == 0) return 0;
    const int ncur = mode == po::kScalar ? 2 : 12;
    const int nout = po::n_out(mode);
    cudaStream_t s = nullptr;
    if (int rc = lib_stream(&s)) return rc;
    double *d_src = nullptr, *d_cur = nullptr, *d_tgt = nullptr, *d_out = nullptr;
    int rc = 0, code = 0;
    HostSlots local{};
    HostSlots *hs = host_slots(&local);
    po::RunArgs a;
    PO_SCRATCH(d_src, sizeof(double) * 7 * std::max(ns, 1L));
    PO_SCRATCH(d_cur, sizeof(double) * ncur * std::max(ns, 1L));
    PO_SCRATCH(d_tgt, sizeof(double) * 7 * nt);
    PO_SCRATCH(d_out, sizeof(double) * nout * nt);
    if (ns > 0) {
        CK(cudaMemcpyAsync(d_src, src7, sizeof(double) * 7 * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_cur, cur, sizeof(double) * ncur * ns, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(d_tgt, tgt7, sizeof(double) * 7 * nt, cudaMemcpyHostToDevice, s));
    a.mode = mode;
    a.ns = ns;
    a.src7 = d_src;
    a.gmode = gmode;
    a.ncx = ncx;
    a.ncy = ncy;
    a.cur = d_cur;
    a.nt = nt;
    a.tgt7 = d_tgt;
    a.k = k;
    a.epsilon = eps;
    a.t_dir = t;
    a.precision = precision;
    a.m_zero = false;
    if (mode != po::kScalar && ns > 0) {
        bool mz = false;
        if ((rc = m_is_zero(cur, d_cur, ns, s, mz))) goto done;
        a.m_zero = mz;
    }
    a.extent_host = &hs->extent;
    a.band_host = &hs->band;
    a.out = d_out;
    a.stream = s;
    rc = po::run_device(a);
    if (rc) goto done;
    CK(cudaMemcpyAsync(out, d_out, sizeof(double) * nout * nt, cudaMemcpyDeviceToHost, s));
    rc = po::read_device_error(s, &code);   // the call's one synchronisation
    if (!rc && precision == 0) {
        t_extent = hs->extent;
        t_band = hs->band;
    }
    if (!rc && code) rc = fail(4, device_error_text(code));
done:
    if (d_src) cudaFreeAsync(d_src, s);
    if (d_cur) cudaFreeAsync(d_cur, s);
    if (d_tgt) cudaFreeAsync(d_tgt, s);
    if (d_out) cudaFreeAsync(d_out, s);
    if (s && rc) cudaStreamSynchronize(s);   // copies from the caller's buffers may still be in flight
    return rc;
}

// reflparamsf -> reflparams with owned double arrays.
struct Widened {
    double coeffs[3], lxu[2], lyv[2], gcenter[2], transf[16];
    reflparams r;
};

void widen(const reflparamsf &f, Widened &w)
{
    for (int i = 0; i < 3; ++i) w.coeffs[i] = f.coeffs ? f.coeffs[i] : 0.0;
    for (int i = 0; i < 2; ++i) {
        w.lxu[i] = f.lxu[i];
        w.lyv[i] = f.lyv[i];
        w.gcenter[i] = f.gcenter ? f.gcenter[i] : 0.0;
    }
    for (int i = 0; i < 16; ++i) w.transf[i] = f.transf ? f.transf[i] : (i % 5 == 0 ? 1.0 : 0.0);
    w.r.coeffs = w.coeffs;
    w.r.lxu = w.lxu;
    w.r.lyv = w.lyv;
    w.r.n_cells = f.n_cells;
    w.r.flip = f.flip;
    w.r.gmode = f.gmode;
    w.r.gcenter = w.gcenter;
    w.r.ecc_uv = f.ecc_uv;
    w.r.rot_uv = f.rot_uv;
    w.r.type = f.type;
    w.r.transf = w.transf;
    w.r.rms = f.rms;
    w.r.rms_seed = f.rms_seed;
}

// Shared body of the callKernelf_* drop-ins. Both grids are generated in
// FP64 on the device from the widened reflparams (the reference generates
// them on the host); the float currents are copied as they are and widened
// on the device; after the mixed-precision run and the call's one
// synchronisation of its kernels, the outputs and the two grids are narrowed
// to float on the device and copied into the caller's bundle rows and
// containers cs / ct, as the reference leaves them.
int drop_in(int mode, float *const *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
            reflcontainerf *ct, float *const *inp, float k, float epsilon, float t)
{
    po::clear_error();
    t_extent = 0.0;
    t_band = 0;
    if (!source.n_cells || !source.lxu || !source.lyv || !target.n_cells || !target.lxu || !target.lyv)
        return fail(1, "reflparamsf has null arrays");
    const long ns = (long)source.n_cells[0] * source.n_cells[1];
    const long nt = (long)target.n_cells[0] * target.n_cells[1];
    if (ns <= 0 || nt <= 0) return fail(1, "empty grid");
    const int nout = po::n_out(mode);
    if (nout < 0) return fail(1, "mode must be 0..5 (JM EH JMEH EHP FF scalar)");
    const int ncur = mode == po::kScalar ? 2 : 12;
    for (int r = 0; r < ncur; ++r)
        if (!inp[r]) return fail(1, "null current array");
    for (int r = 0; r < nout; ++r)
        if (!res[r]) return fail(1, "null result array");
    Widened ws, wt;
    widen(source, ws);
    widen(target, wt);
    cudaStream_t s = nullptr;
    if (int rc = lib_stream(&s)) return rc;
    double *d_src = nullptr, *d_cur = nullptr, *d_tgt = nullptr, *d_out = nullptr;
    float *d_f = nullptr;   // float staging: the currents in, then the outputs and grids out
    const long nf = std::max({(long)ncur * ns, (long)nout * nt, 7L * std::max(ns, nt)});
    int rc = 0, code = 0;
    HostSlots local{};
    HostSlots *hs = host_slots(&local);
    po::RunArgs a;
    const unsigned cblk = 608;   // 152 SMs x 4, grid-stride
    PO_SCRATCH(d_src, sizeof(double) * 7 * ns);
    PO_SCRATCH(d_cur, sizeof(double) * ncur * ns);
    PO_SCRATCH(d_tgt, sizeof(double) * 7 * nt);
    PO_SCRATCH(d_out, sizeof(double) * nout * nt);
    PO_SCRATCH(d_f, sizeof(float) * nf);
    if ((rc = po::generate_grid_dev(ws.r, d_src, true, true, s)) ||
        (rc = po::generate_grid_dev(wt.r, d_tgt, true, true, s)))
        goto done;
    for (int r = 0; r < ncur; ++r)
        CK(cudaMemcpyAsync(d_f + (size_t)r * ns, inp[r], sizeof(float) * ns, cudaMemcpyHostToDevice, s));
    {
        long n = (long)ncur * ns;
        void *args[] = {&d_f, &d_cur, &n};
        CK(cudaLaunchKernel(po::f2d_kernel(), dim3(cblk), dim3(256), args, 0, s));
    }
    a.mode = mode;
    a.ns = ns;
    a.src7 = d_src;
    a.gmode = source.gmode;
    a.ncx = source.n_cells[0];
    a.ncy = source.n_cells[1];
    a.cur = d_cur;
    a.nt = nt;
    a.tgt7 = d_tgt;
    a.k = (double)k;
    a.epsilon = (double)epsilon;
    a.t_dir = (double)t;
    a.precision = 0;
    a.m_zero = false;
    if (mode != po::kScalar) {
        bool mz = false;
        if ((rc = device_m_is_zero(d_cur, ns, s, mz))) goto done;
        a.m_zero = mz;
    }
    a.extent_host = &hs->extent;
    a.band_host = &hs->band;
    a.out = d_out;
    a.stream = s;
    rc = po::run_device(a);
    if (rc) goto done;
    {
        long n = (long)nout * nt;
        void *args[] = {&d_out, &d_f, &n};
        CK(cudaLaunchKernel(po::d2f_kernel(), dim3(cblk), dim3(256), args, 0, s));
    }
    for (int r = 0; r < nout; ++r)
        CK(cudaMemcpyAsync(res[r], d_f + (size_t)r * nt, sizeof(float) * nt, cudaMemcpyDeviceToHost, s));
    rc = po::read_device_error(s, &code);   // the kernels' one synchronisation
    if (!rc && code) rc = fail(4, device_error_text(code));
    if (rc) goto done;
    t_extent = hs->extent;
    t_band = hs->band;
    // the grids, as the reference leaves them in cs and ct
    for (int w = 0; w < 2; ++w) {
        reflcontainerf *cf = w == 0 ? cs : ct;
        if (!cf || !cf->x) continue;
        long n = 7L * (w == 0 ? ns : nt);
        double *g = w == 0 ? d_src : d_tgt;
        void *args[] = {&g, &d_f, &n};
        CK(cudaLaunchKernel(po::d2f_kernel(), dim3(cblk), dim3(256), args, 0, s));
        float *dst[7] = {cf->x, cf->y, cf->z, cf->nx, cf->ny, cf->nz, cf->area};
        const long np = n / 7;
        for (int r = 0; r < 7; ++r)
            if (dst[r]) CK(cudaMemcpyAsync(dst[r], d_f + (size_t)r * np, sizeof(float) * np, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
done:
    if (d_src) cudaFreeAsync(d_src, s);
    if (d_cur) cudaFreeAsync(d_cur, s);
    if (d_tgt) cudaFreeAsync(d_tgt, s);
    if (d_out) cudaFreeAsync(d_out, s);
    if (d_f) cudaFreeAsync(d_f, s);
    if (s && rc) cudaStreamSynchronize(s);
    return rc;
}

}  // namespace

extern "C" {

const char *po_last_error(void) { return po::last_error(); }

int po_n_out(int mode) { return po::n_out(mode); }

int po_last_launches(void) { return po::last_launches(); }

int po_generate_grid(reflparams refl, reflcontainer *container, int transform, int spheric)
{
    po::clear_error();
    if (po_grid_fill(refl, container, transform != 0, spheric != 0))
        return fail(1, "grid generation failed (bad gmode, sizes or null container)");
    return 0;
}

int po_generate_grid_dev(reflparams refl, double *out7, int transform, int spheric, void *stream)
{
    po::clear_error();
    return po::generate_grid_dev(refl, out7, transform != 0, spheric != 0, static_cast<cudaStream_t>(stream));
}

int po_correlated_error(long n, double *grid7, double rms, double corr_len, unsigned seed, int n_modes,
                        double *delta, int apply)
{
    po::clear_error();
    if (po::correlated_error_host(n, grid7, rms, corr_len, seed, n_modes, delta, apply))
        return fail(1, "po_correlated_error: bad arguments (n >= 0, n_modes >= 1, corr_len > 0, rms >= 0, grid)");
    return 0;
}

int po_correlated_error_dev(long n, double *grid7, double rms, double corr_len, unsigned seed, int n_modes,
                            double *delta, int apply, void *stream)
{
    po::clear_error();
    return po::correlated_error_dev(n, grid7, rms, corr_len, seed, n_modes, delta, apply,
                                    static_cast<cudaStream_t>(stream));
}

int po_gauss_beam_dev(long n, const double *grid7, double lam, double w0, double z, double power, int mode,
                      double *fields, double *currents, void *stream)
{
    po::clear_error();
    return po::gauss_beam_dev(n, grid7, lam, w0, z, power, mode, fields, currents,
                              static_cast<cudaStream_t>(stream));
}

int po_calc_jm_dev(long n, const double *grid7, const double *fields, int mode, double *currents, void *stream)
{
    po::clear_error();
    return po::calc_jm_dev(n, grid7, fields, mode, currents, static_cast<cudaStream_t>(stream));
}

int po_efficiency_sums_dev(long n, const double *grid7, const double *f_re, const double *f_im, const double *g_re,
                           const double *g_im, int shape, const double *aperture, double *sums, void *stream)
{
    po::clear_error();
    return po::efficiency_sums_dev(n, grid7, f_re, f_im, g_re, g_im, shape, aperture, sums,
                                   static_cast<cudaStream_t>(stream));
}

int po_fit_gauss_abs_dev(int ncx, int ncy, const double *grid7, const double *f_re, const double *f_im, double thres,
                         int scale, int use_ratio, double ratio, double *popt, double *p0, void *stream)
{
    po::clear_error();
    return po::fit_gauss_abs_dev(ncx, ncy, grid7, f_re, f_im, thres, scale, use_ratio, ratio, popt, p0,
                                 static_cast<cudaStream_t>(stream));
}

int po_generate_gauss_dev(long n, const double *grid7, const double *popt, int scale, double *out, void *stream)
{
    po::clear_error();
    return po::generate_gauss_dev(n, grid7, popt, scale, out, static_cast<cudaStream_t>(stream));
}

int po_fmin(int n, const double *x0, double xtol, double ftol, long maxiter, long maxfun, po_objective f, void *ctx,
            double *xopt, double *fopt, long *iterations, long *fcalls)
{
    po::clear_error();
    if (!f) return po::fail(1, "fmin: null objective");
    const po::Objective obj = [&](const double *x, double *fx) {
        const int rc = f(x, fx, ctx);
        return rc == 0 ? 0 : po::fail(rc, "fmin: the objective returned a non-zero status");
    };
    return po::fmin_nm(n, x0, xtol, ftol, maxiter, maxfun, obj, xopt, fopt, iterations, fcalls);
}

int po_run_d(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
             const double *tgt7, double k, double epsilon, double t_direction, int precision, double *out)
{
    return run_host(mode, ns, src7, gmode, ncx, ncy, cur, nt, tgt7, k, epsilon, t_direction, precision, out);
}

int po_run_dev(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
               const double *tgt7, double k, double epsilon, double t_direction, int precision, int flags,
               double *out, void *stream)
{
    po::clear_error();
    po::RunArgs a;
    a.mode = mode;
    a.ns = ns;
    a.src7 = src7;
    a.gmode = gmode;
    a.ncx = ncx;
    a.ncy = ncy;
    a.cur = cur;
    a.nt = nt;
    a.tgt7 = tgt7;
    a.k = k;
    a.epsilon = epsilon;
    a.t_dir = t_direction;
    a.precision = precision;
    a.m_zero = (flags & 1) != 0;
    a.out = out;
    a.stream = static_cast<cudaStream_t>(stream);
    return po::run_device(a);
}

namespace {

int adjoint_dev(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
                const double *tgt7, double k, double epsilon, double t_direction, int precision, int flags,
                const double *cot, double *grad_cur, double *grad_ds, double *grad_dt, cudaStream_t stream,
                HostSlots *slots)
{
    po::AdjArgs a;
    a.mode = mode;
    a.ns = ns;
    a.src7 = src7;
    a.gmode = gmode;
    a.ncx = ncx;
    a.ncy = ncy;
    a.cur = cur;
    a.nt = nt;
    a.tgt7 = tgt7;
    a.k = k;
    a.epsilon = epsilon;
    a.t_dir = t_direction;
    a.precision = precision;
    a.m_zero = (flags & 1) != 0;
    a.out = grad_cur ? grad_cur : (grad_ds ? grad_ds : grad_dt);   // validate() wants an output
    a.cot = cot;
    a.grad_cur = grad_cur;
    a.grad_ds = grad_ds;
    a.grad_dt = grad_dt;
    a.stream = stream;
    a.extent_host = slots ? &slots->extent : nullptr;
    a.band_host = slots ? &slots->band : nullptr;
    if (!grad_cur && !grad_ds && !grad_dt) return fail(1, "no gradient requested");
    return po::run_adjoint(a);
}

}  // namespace

int po_adjoint_dev(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
                   const double *tgt7, double k, double epsilon, double t_direction, int precision, int flags,
                   const double *cot, double *grad_cur, double *grad_ds, double *grad_dt, void *stream)
{
    po::clear_error();
    return adjoint_dev(mode, ns, src7, gmode, ncx, ncy, cur, nt, tgt7, k, epsilon, t_direction, precision, flags, cot,
                       grad_cur, grad_ds, grad_dt, static_cast<cudaStream_t>(stream), nullptr);
}

double po_last_extent(void) { return t_extent; }
unsigned long long po_last_band_pairs(void) { return t_band; }

int po_adjoint_d(int mode, long ns, const double *src7, int gmode, int ncx, int ncy, const double *cur, long nt,
                 const double *tgt7, double k, double epsilon, double t_direction, int precision, const double *cot,
                 double *grad_cur, double *grad_ds, double *grad_dt)
{
    po::clear_error();
    t_extent = 0.0;
    t_band = 0;
    if (mode < 0 || mode > 5) return fail(1, "mode must be 0..5");
    if (ns < 0 || nt < 0) return fail(1, "negative size");
    const int nout = po::n_out(mode);
    cudaStream_t s = nullptr;
    if (int rc = lib_stream(&s)) return rc;
    double *d_src = nullptr, *d_cur = nullptr, *d_tgt = nullptr, *d_cot = nullptr;
    double *d_gc = nullptr, *d_gs = nullptr, *d_gt = nullptr;
    int rc = 0, code = 0;
    HostSlots local{};
    HostSlots *hs = host_slots(&local);
    const size_t ns1 = std::max(ns, 1L), nt1 = std::max(nt, 1L);
    const int ncur = mode == po::kScalar ? 2 : 12;
    PO_SCRATCH(d_src, sizeof(double) * 7 * ns1);
    PO_SCRATCH(d_cur, sizeof(double) * ncur * ns1);
    PO_SCRATCH(d_tgt, sizeof(double) * 7 * nt1);
    PO_SCRATCH(d_cot, sizeof(double) * nout * nt1);
    if (grad_cur) PO_SCRATCH(d_gc, sizeof(double) * ncur * ns1);
    if (grad_ds) PO_SCRATCH(d_gs, sizeof(double) * ns1);
    if (grad_dt) PO_SCRATCH(d_gt, sizeof(double) * nt1);
    if (ns > 0) {
        CK(cudaMemcpyAsync(d_src, src7, sizeof(double) * 7 * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_cur, cur, sizeof(double) * ncur * ns, cudaMemcpyHostToDevice, s));
    }
    if (nt > 0) {
        CK(cudaMemcpyAsync(d_tgt, tgt7, sizeof(double) * 7 * nt, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_cot, cot, sizeof(double) * nout * nt, cudaMemcpyHostToDevice, s));
    }
    {
        bool mz = false;
        if (ns > 0 && mode != po::kScalar && (rc = m_is_zero(cur, d_cur, ns, s, mz))) goto done;
        rc = adjoint_dev(mode, ns, d_src, gmode, ncx, ncy, d_cur, nt, d_tgt, k, epsilon, t_direction, precision,
                         mz ? 1 : 0, d_cot, d_gc, d_gs, d_gt, s, hs);
    }
    if (rc) goto done;
    if (grad_cur && ns > 0)
        CK(cudaMemcpyAsync(grad_cur, d_gc, sizeof(double) * ncur * ns, cudaMemcpyDeviceToHost, s));
    if (grad_ds && ns > 0) CK(cudaMemcpyAsync(grad_ds, d_gs, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
    if (grad_dt && nt > 0) CK(cudaMemcpyAsync(grad_dt, d_gt, sizeof(double) * nt, cudaMemcpyDeviceToHost, s));
    rc = po::read_device_error(s, &code);   // the call's one synchronisation
    if (!rc && precision == 0) {
        t_extent = hs->extent;
        t_band = hs->band;
    }
    if (!rc && code) rc = fail(4, device_error_text(code));
done:
    for (double *p : {d_src, d_cur, d_tgt, d_cot, d_gc, d_gs, d_gt})
        if (p) cudaFreeAsync(p, s);
    if (s && rc) cudaStreamSynchronize(s);   // copies from the caller's buffers may still be in flight
    return rc;
}

int po_timing_enable(int slots)
{
    po::clear_error();
    return po::timing_enable(slots);
}

int po_timing_collect(float *ms, int max) { return po::timing_collect(ms, max); }

int po_fp32_probe(int blocks, int iters, float *out, void *stream)
{
    po::clear_error();
    if (blocks < 1 || iters < 1 || !out) return fail(1, "po_fp32_probe: bad arguments");
    void *args[] = {&iters, nullptr, &out};
    float seed = 1.0f;
    args[1] = &seed;
    cudaError_t e = cudaLaunchKernel(po::fp32_probe_kernel(), dim3(blocks), dim3(256), args, 0,
                                     static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(2, std::string("po_fp32_probe: ") + cudaGetErrorString(e));
    po::note_launches(1);
    return 0;
}

int po_device_error(void *stream, int *code)
{
    po::clear_error();
    if (!code) return fail(1, "po_device_error: null code");
    return po::read_device_error(static_cast<cudaStream_t>(stream), code);
}

int po_wait_selftest(unsigned limit, int *err, int word, void *stream)
{
    po::clear_error();
    int *w = err;
    if (!w) {
        if (word == 0) {
            w = po::error_word();
            if (!w) return fail(2, "po_wait_selftest: no device error word");
        } else if (word == 1) {
            w = po::static_status_word();
            if (!w) return fail(3, "po_wait_selftest: po_run_dev_static has not run on this device");
        } else {
            return fail(1, "po_wait_selftest: word must be 0 (allocating entries) or 1 (po_run_dev_static)");
        }
    }
    void *args[] = {&limit, &w};
    cudaError_t e = cudaLaunchKernel(po::wait_selftest_kernel(), dim3(1), dim3(64), args, 0,
                                     static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(2, std::string("po_wait_selftest: ") + cudaGetErrorString(e));
    po::note_launches(1);
    return 0;
}

int po_scratch_in_use(unsigned long long *bytes)
{
    po::clear_error();
    if (!bytes) return fail(1, "po_scratch_in_use: null argument");
    return po::scratch_used(bytes);
}

#define ROWS12(b) {b->r1x, b->r1y, b->r1z, b->i1x, b->i1y, b->i1z, b->r2x, b->r2y, b->r2z, b->i2x, b->i2y, b->i2z}

int callKernelf_JM(c2Bundlef *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                   reflcontainerf *ct, c2Bundlef *currents, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !currents) return fail(1, "null bundle");
    float *r[12] = ROWS12(res);
    float *c[12] = ROWS12(currents);
    return drop_in(po::kJM, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callKernelf_EH(c2Bundlef *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                   reflcontainerf *ct, c2Bundlef *currents, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !currents) return fail(1, "null bundle");
    float *r[12] = ROWS12(res);
    float *c[12] = ROWS12(currents);
    return drop_in(po::kEH, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callKernelf_JMEH(c4Bundlef *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                     reflcontainerf *ct, c2Bundlef *currents, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !currents) return fail(1, "null bundle");
    float *r[24] = {res->r1x, res->r1y, res->r1z, res->i1x, res->i1y, res->i1z, res->r2x, res->r2y,
                    res->r2z, res->i2x, res->i2y, res->i2z, res->r3x, res->r3y, res->r3z, res->i3x,
                    res->i3y, res->i3z, res->r4x, res->r4y, res->r4z, res->i4x, res->i4y, res->i4z};
    float *c[12] = ROWS12(currents);
    return drop_in(po::kJMEH, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callKernelf_EHP(c2rBundlef *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                    reflcontainerf *ct, c2Bundlef *currents, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !currents) return fail(1, "null bundle");
    float *r[15] = {res->r1x, res->r1y, res->r1z, res->i1x, res->i1y, res->i1z, res->r2x, res->r2y,
                    res->r2z, res->i2x, res->i2y, res->i2z, res->r3x, res->r3y, res->r3z};
    float *c[12] = ROWS12(currents);
    return drop_in(po::kEHP, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callKernelf_FF(c2Bundlef *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                   reflcontainerf *ct, c2Bundlef *currents, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !currents) return fail(1, "null bundle");
    float *r[12] = ROWS12(res);
    float *c[12] = ROWS12(currents);
    return drop_in(po::kFF, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callKernelf_scalar(arrC1f *res, reflparamsf source, reflparamsf target, reflcontainerf *cs,
                       reflcontainerf *ct, arrC1f *inp, float k, float epsilon, float t_direction, int, int)
{
    if (!res || !inp) return fail(1, "null array");
    float *r[2] = {res->x, res->y};
    float *c[2] = {inp->x, inp->y};
    return drop_in(po::kScalar, r, source, target, cs, ct, c, k, epsilon, t_direction);
}

int callRTKernel(reflparamsf, cframef *, cframef *, float, float, int, int)
{
    static const char msg[] =
        "callRTKernel: the GPU ray tracer is not part of libpo_gb300; bind callRTKernel from libpypogpu";
    std::fprintf(stderr, "libpo_gb300: %s\n", msg);
    return fail(6, msg);
}

}  // extern "C"
