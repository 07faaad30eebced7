// po_internal.h -- shared declarations of libpo_gb300's host code.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <string>

#include "../../include/po_gb300.h"
#include "po_kernels.cuh"

namespace po {

// One propagation on device buffers. All pointers are device memory.
struct RunArgs {
    int mode = kEH;
    long ns = 0;
    const double *src7 = nullptr;  // 7 rows x ns
    int gmode = 0, ncx = 0, ncy = 0;
    const double *cur = nullptr;   // 12 rows (or 2 for scalar) x ns
    long nt = 0;
    const double *tgt7 = nullptr;  // 7 rows x nt
    double k = 1.0, epsilon = 1.0, t_dir = -1.0;
    int precision = 0;             // 0 mixed, 1 plain FP64
    bool m_zero = false;           // M == 0 on the source
    double *out = nullptr;         // n_out(mode) rows x nt
    cudaStream_t stream = nullptr;
    double *extent_host = nullptr; // mixed path: host slot for the frame's half-extent (wavelengths),
                                   // written by a copy queued on `stream`
    unsigned *band_host = nullptr; // mixed path: host slot for the number of near-tangent pairs the
                                   // call met (decided in FP64), written the same way
};

// Adjoint of one propagation: cotangents of the outputs in, gradients with
// respect to the source currents and the normal displacements out.
struct AdjArgs : RunArgs {
    const double *cot = nullptr;   // n_out(mode) rows x nt
    double *grad_cur = nullptr;    // 12 rows x ns, or null
    double *grad_ds = nullptr;     // ns, or null
    double *grad_dt = nullptr;     // nt, or null (near field only)
};

int n_out(int mode);
int run_adjoint(const AdjArgs &a);
int validate(const RunArgs &a);   // argument checks only, no CUDA calls
int run_device(const RunArgs &a);

// Thread-local error reporting.
int fail(int code, const std::string &msg);
void clear_error();
void note_launches(int n);

const char *last_error();
int last_launches();

// Measurement hook: CUDA event pairs recorded on the launching stream around
// every main-kernel launch, read back (synchronising) by timing_collect.
int timing_enable(int slots);
int timing_collect(float *ms, int max);

// Synchronises `s`, returns and clears the device error words (wait
// timeouts): the allocating paths' word and, once the allocation-free entry
// has set up on this device, its static status word. Allocates nothing.
int read_device_error(cudaStream_t s, int *code);
// The allocating paths' error word of the current device (allocated once).
int *error_word();
// The allocation-free entry's status word on the current device, or null
// before its first call there (po_noalloc.cu).
int *static_status_word();

// Stream-ordered scratch from the library's own memory pool (one per device,
// created on first use; the device's default pool is left as it is).
int scratch_alloc(void **p, size_t bytes, cudaStream_t s);
void scratch_free(void *p, cudaStream_t s);
// Bytes of the library's pool on the current device in use by scratch that
// has not been freed (0 before the pool exists).
int scratch_used(unsigned long long *bytes);

// Where one mixed-precision propagation takes its scratch. Every buffer is
// taken before the first launch, so a source that runs out fails before any
// device work. take() gives 256-byte aligned memory; room() is what is left.
class Scratch {
public:
    virtual ~Scratch() = default;
    virtual int take(void **p, size_t bytes) = 0;
    virtual size_t room() const = 0;
    // entries of the list of near-tangent pairs a call of ns x nt pairs takes (BandList)
    virtual unsigned band_cap(long ns, long nt) const { return band_cap_for(ns, nt); }
    template <typename T>
    int get(T **p, size_t count)
    {
        void *q = nullptr;
        const int rc = take(&q, count * sizeof(T));
        *p = static_cast<T *>(q);
        return rc;
    }
};

// The mixed-precision forward of run_device on a given scratch source and
// error word (run_device: the library's pool and error word; the
// allocation-free entry: its static array and status word). In two steps:
// mixed_prepare takes every buffer (no device work), mixed_launch queues the
// kernels on a.stream.
// Constants, buffers and launch shape of one mixed-precision propagation.
struct MixedPlan {
    int kind = 0, nacc = 0, ts = -1;
    bool far = false, has_m = false;
    double kappa = 0, fac_re = 0, fac_im = 0, zeta_inv = 0;
    long tiles = 0, ntb = 0, nsplit = 1, chunk = 0;
    double *bbox = nullptr, *part = nullptr;
    Frame *frame = nullptr;
    float4 *srcpk = nullptr, *tgtpk = nullptr;
    unsigned long long *keys = nullptr;
    int *order = nullptr;
    void *sort_tmp = nullptr;
    size_t sort_bytes = 0;
    BandList band{nullptr, nullptr, 0};   // near-tangent pairs (not the scalar kind)
};
int mixed_prepare(const RunArgs &a, Scratch &sc, MixedPlan &p);
int mixed_launch(const RunArgs &a, MixedPlan &p, int *err);
int run_mixed(const RunArgs &a, Scratch &sc, int *err);

// Radix sort of (key, index) pairs for the far field's source order
// (po_farfield.cu); with temp == nullptr it only sets *temp_bytes, on the
// host, with no device work.
cudaError_t ff_sort(void *temp, size_t *temp_bytes, const unsigned long long *key_in, unsigned long long *key_out,
                    const int *idx_in, int *idx_out, long n, cudaStream_t s);

// Number of chunks of a streamed axis (ns items in tiles of `tile`) for a
// grid of `nb` owning blocks on `slots` resident CTAs: minimises waves times
// chunk length, with a small cost per extra chunk; at most max_chunks.
long choose_split(long nb, long ns, long slots, long max_chunks, long tile);

// FP64 grid generation on the device into a 7-row layout (po_grid_dev.cu).
int generate_grid_dev(const reflparams &r, double *out7, bool transform, bool spheric, cudaStream_t s);
// n normal deviates N(0, stdev) in the reference's sequence (mt19937 seeded
// with `seed`, a fresh distribution per draw), on the device.
int normal_deviates_dev(unsigned seed, long n, double stdev, double *out, int *err, cudaStream_t s);
// Correlated surface error at the n points of a 7-row device grid (delta
// and/or the points moved along their normals), and its host twin (po_grid.cpp).
int correlated_error_dev(long n, double *g7, double rms, double corr_len, unsigned seed, int n_modes, double *delta,
                         int apply, cudaStream_t s);
int correlated_error_host(long n, double *g7, double rms, double corr_len, unsigned seed, int n_modes, double *delta,
                          int apply);

// Source producers on the device (po_sources_dev.cu).
int gauss_beam_dev(long n, const double *g7, double lam, double w0, double z, double power, int mode,
                   double *fields, double *cur, cudaStream_t s);
int calc_jm_dev(long n, const double *g7, const double *fields, int mode, double *cur, cudaStream_t s);

// Efficiency sums on the device (po_eff_dev.cu).
int efficiency_sums_dev(long n, const double *g7, const double *fr, const double *fi, const double *gr,
                        const double *gi, int shape, const double *aper, double *sums, cudaStream_t s);

// Downhill-simplex minimiser (po_fmin.cpp). The objective writes f(x) and
// returns 0, or a non-zero status that aborts the minimisation.
using Objective = std::function<int(const double *x, double *fx)>;
int fmin_nm(int n, const double *x0, double xatol, double fatol, long maxiter, long maxfun, const Objective &func,
            double *xopt, double *fopt, long *nit, long *nfev);

// Gaussian beam fit on the device (po_fitgauss_dev.cu).
int fit_gauss_abs_dev(int ncx, int ncy, const double *g7, const double *fr, const double *fi, double thres,
                      int scale, int use_ratio, double ratio, double *popt, double *p0, cudaStream_t s);
int generate_gauss_dev(long n, const double *g7, const double *popt, int scale, double *out, cudaStream_t s);

}  // namespace po

int po_grid_fill(const reflparams &r, reflcontainer *c, bool transform, bool spheric);
