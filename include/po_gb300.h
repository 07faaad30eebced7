/*
 * po_gb300.h -- C-ABI of libpo_gb300.so, the GB300 (sm_103a) physical-optics
 * surface-current integrator.
 *
 * The struct layouts below are identical to PyPO's (reference
 * src/include/Structs.h:42-147, :243-348) so that the reference's ctypes
 * structs (src/PyPO/Structs.py) bind to these entry points unchanged.
 *
 * Every entry point returns an int status: 0 on success, non-zero on error,
 * with a message available from po_last_error() on the calling thread. No
 * entry point calls exit() or cudaDeviceReset(); the CUDA context is shared
 * with the caller (for example PyTorch).
 *
 * Mode numbers: 0 JM, 1 EH, 2 JMEH, 3 EHP, 4 FF, 5 scalar. The semantics are
 * those of the reference's FP64 CPU path (src/CPU/Propagation.h): PEC
 * currents J = 2 n x H, M = 0 for JM and JMEH; reflected H scaled by the
 * medium conductance in EHP; exp(-t j k r) in scalar mode; the illumination
 * test n_s . R_hat >= 0 for both time directions.
 */
#ifndef PO_GB300_H
#define PO_GB300_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- ABI structs (same layout as the reference's) ---------------------- */

typedef struct arrC1 { double *x, *y; } arrC1;
typedef struct arrC1f { float *x, *y; } arrC1f;

typedef struct c2Bundle {
    double *r1x, *r1y, *r1z, *i1x, *i1y, *i1z;
    double *r2x, *r2y, *r2z, *i2x, *i2y, *i2z;
} c2Bundle;
typedef struct c2Bundlef {
    float *r1x, *r1y, *r1z, *i1x, *i1y, *i1z;
    float *r2x, *r2y, *r2z, *i2x, *i2y, *i2z;
} c2Bundlef;

typedef struct c4Bundlef {
    float *r1x, *r1y, *r1z, *i1x, *i1y, *i1z;
    float *r2x, *r2y, *r2z, *i2x, *i2y, *i2z;
    float *r3x, *r3y, *r3z, *i3x, *i3y, *i3z;
    float *r4x, *r4y, *r4z, *i4x, *i4y, *i4z;
} c4Bundlef;

typedef struct c2rBundlef {
    float *r1x, *r1y, *r1z, *i1x, *i1y, *i1z;
    float *r2x, *r2y, *r2z, *i2x, *i2y, *i2z;
    float *r3x, *r3y, *r3z;
} c2rBundlef;

typedef struct reflparams {
    double *coeffs;
    double *lxu;
    double *lyv;
    int *n_cells;
    bool flip;
    int gmode;
    double *gcenter;
    double ecc_uv;
    double rot_uv;
    int type;
    double *transf;
    double rms;
    unsigned int rms_seed;
} reflparams;

typedef struct reflparamsf {
    float *coeffs;
    float *lxu;
    float *lyv;
    int *n_cells;
    bool flip;
    int gmode;
    float *gcenter;
    float ecc_uv;
    float rot_uv;
    int type;
    float *transf;
    float rms;
    unsigned int rms_seed;
} reflparamsf;

typedef struct reflcontainer {
    int size;
    double *x, *y, *z, *nx, *ny, *nz, *area;
} reflcontainer;

typedef struct reflcontainerf {
    int size;
    float *x, *y, *z, *nx, *ny, *nz, *area;
} reflcontainerf;

/* Ray-trace frame (reference Structs.h:352-362); only callRTKernel takes it. */
typedef struct cframef {
    int size;
    float *x, *y, *z, *dx, *dy, *dz;
} cframef;

/* ---- errors ------------------------------------------------------------- */

/* Message of the last failed call on this thread ("" when none). */
const char *po_last_error(void);

/* ---- drop-in replacements for the reference's libpypogpu ----------------
 * Same signatures as reference src/CUDA/InterfaceCUDA.h:31-64 (ctypes
 * argtypes src/PyPO/BindGPU.py:34-74), called from BindGPU.PyPO_GPUf
 * (src/PyPO/BindGPU.py:83-224). Like the reference they generate the source
 * and target grids from the reflparamsf into cs / ct (here in FP64 on the
 * device, then stored as float; the reference generates them on the host),
 * and fill res. nBlocks / nThreads are accepted and
 * ignored: the engine picks its own tiling. Computation is mixed precision
 * (FP32 bulk, split hi/lo separation and phase). The reference returns void;
 * these return the status (ctypes restype None ignores it).
 */
int callKernelf_JM(c2Bundlef *res, reflparamsf source, reflparamsf target,
                   reflcontainerf *cs, reflcontainerf *ct, c2Bundlef *currents,
                   float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:1636-1706 */
int callKernelf_EH(c2Bundlef *res, reflparamsf source, reflparamsf target,
                   reflcontainerf *cs, reflcontainerf *ct, c2Bundlef *currents,
                   float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:1729-1797 */
int callKernelf_JMEH(c4Bundlef *res, reflparamsf source, reflparamsf target,
                     reflcontainerf *cs, reflcontainerf *ct, c2Bundlef *currents,
                     float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:1821-1895 */
int callKernelf_EHP(c2rBundlef *res, reflparamsf source, reflparamsf target,
                    reflcontainerf *cs, reflcontainerf *ct, c2Bundlef *currents,
                    float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:1919-2000 */
int callKernelf_FF(c2Bundlef *res, reflparamsf source, reflparamsf target,
                   reflcontainerf *cs, reflcontainerf *ct, c2Bundlef *currents,
                   float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:2023-2090 */
int callKernelf_scalar(arrC1f *res, reflparamsf source, reflparamsf target,
                       reflcontainerf *cs, reflcontainerf *ct, arrC1f *inp,
                       float k, float epsilon, float t_direction, int nBlocks, int nThreads);
    /* replaces Kernelsf.cu:2113-2175 */

/* The reference's loadGPUlib (src/PyPO/BindGPU.py:18-81) also binds its GPU
 * ray tracer, callRTKernel (InterfaceCUDA.h:66-68), so the library must
 * export that name for the unmodified loader to bind. The ray tracer is not
 * part of this library: the call writes nothing to fr_out, returns 6, sets
 * po_last_error() and prints one line on stderr (the reference's binding
 * ignores the status). Bind callRTKernel from libpypogpu to keep GPU ray
 * tracing. */
int callRTKernel(reflparamsf ctp, cframef *fr_in, cframef *fr_out, float epsilon, float t0,
                 int nBlocks, int nThreads);

/* ---- FP64 grid generation ------------------------------------------------
 * Same contract as the reference's generateGrid (src/common/InterfaceReflector.h:24-25,
 * src/common/InterfaceReflector.cpp:882-972): fills container (size
 * n_cells[0]*n_cells[1], row-major over (x/u, y/v)) with points, unit
 * normals and area elements, applies the 4x4 transform when `transform`,
 * maps AoE grids to (polar, azimuth) radians when `spheric`, and adds the
 * uncorrelated normal-direction surface error when rms > 0.
 */
int po_generate_grid(reflparams refl, reflcontainer *container, int transform, int spheric);

/* The same FP64 grid, generated on the device into `out7`: a device buffer
 * of 7 rows x n_cells[0]*n_cells[1] doubles (x, y, z, nx, ny, nz, area), the
 * layout po_run_dev takes, queued on `stream`. The reflparams arrays are host
 * memory, read during the call. With rms > 0 the surface-error deviates are
 * drawn on the device in the reference's sequence (mt19937 seeded with
 * rms_seed, a fresh normal distribution per point, Random.h:112-116,
 * InterfaceReflector.cpp:852-866). Replaces the host loops of
 * InterfaceReflector.cpp:882-1081 when the grid is only needed on the GPU. */
int po_generate_grid_dev(reflparams refl, double *out7, int transform, int spheric, void *stream);

/* Correlated surface error (no counterpart in the reference, whose surface
 * error is uncorrelated, InterfaceReflector.cpp:852-866): a Gaussian random
 * surface with covariance rms^2 exp(-r^2 / (2 corr_len^2)) over the points'
 * (x, y), by spectral synthesis
 *   delta_i = rms sqrt(2 / M) sum_m cos(kx_m x_i + ky_m y_i + ph_m),
 * M = n_modes, with the modes from the reference's generator (mt19937 seeded
 * with `seed`, a fresh normal deviate per draw): four deviates g per mode,
 * (kx, ky) = (g0, g1) / corr_len, ph = atan2(g2, g3). grid7 is a 7-row grid
 * (x, y, z, nx, ny, nz, area) of n points; delta (n, or NULL) receives the
 * displacement; with apply != 0 the points also move by it along their
 * normals. po_correlated_error works on host memory, po_correlated_error_dev
 * on device memory, queued on `stream`; both give the same numbers to
 * rounding. */
int po_correlated_error(long n, double *grid7, double rms, double corr_len, unsigned seed, int n_modes,
                        double *delta, int apply);
int po_correlated_error_dev(long n, double *grid7, double rms, double corr_len, unsigned seed, int n_modes,
                            double *delta, int apply, void *stream);

/* ---- source producers on the device --------------------------------------
 * po_gauss_beam_dev: the vector Gaussian feed of makeGaussBeam
 * (BeamInit.h:407-596 initGaussBeam, BindBeam.py:160-199) on the n points of
 * a device grid (7 rows, the layout above): fields E, H and equivalent
 * currents J, M as 12 rows x n (c2Bundle order); either output may be NULL.
 * lam, w0, z (waist position), power as the reference's GPODict; mode 0
 * J = n x H, M = -n x E; 1 (PMC) M only, doubled; 2 (PEC) J only, doubled.
 * po_calc_jm_dev: the equivalent currents of given fields (12 x n) on a
 * device grid, calcCurrents (BeamInit.h:660-843, BindBeam.py:236-280), modes
 * 0-2 as above and 3: J = 2 n x E. Both queue on `stream`. */
int po_gauss_beam_dev(long n, const double *grid7, double lam, double w0, double z, double power, int mode,
                      double *fields, double *currents, void *stream);
int po_calc_jm_dev(long n, const double *grid7, const double *fields, int mode, double *currents, void *stream);

/* ---- efficiencies on the device --------------------------------------------
 * The sums behind Efficiencies.py calcSpillover / calcTaper / calcXpol /
 * calcMainBeam (Efficiencies.py:90-177) over the n points of a device grid
 * (7 rows; x, y and area are read), for one field component f (device rows
 * f_re, f_im; f_im NULL for a real f) and an optional second one g (cross-polar or fitted Gaussian;
 * NULL, NULL if unused; g_im NULL alone for a real g such as a fitted
 * Gaussian). Aperture (_generateMask, Efficiencies.py:11-41):
 * shape 0 none, 1 ellipse (aperture = cx, cy, outer_x, outer_y), 2 rectangle
 * (cx, cy, x_lo, x_hi, y_lo, y_hi relative to the centre); host memory.
 * Writes 10 doubles to the device buffer `sums`: sum |f|^2 A, then over the
 * aperture sum |f|^2 A, sum Re f A, sum Im f A, sum A; then sum |f|^2,
 * sum |g|^2, max |f|^2, max |g|^2, aperture point count. Queued on `stream`,
 * deterministic. */
int po_efficiency_sums_dev(long n, const double *grid7, const double *f_re, const double *f_im, const double *g_re,
                           const double *g_im, int shape, const double *aperture, double *sums, void *stream);

/* ---- Gaussian beam fit on the device ---------------------------------------
 * po_fit_gauss_abs_dev: FitGauss.py fitGaussAbs (:67-163) as System.fitGaussAbs
 * and System.calcMainBeam call it (System.py:1828-1906), on the ncx x ncy
 * points of a device grid made without transform or spherical mapping (7
 * rows as above; x and y are read) and the field component f (device rows
 * f_re, f_im; f_im NULL for a real amplitude). thres in dB (the reference's
 * default is -11), scale as the reference's Scales (0 LIN, 2 dB; 1 AMP has
 * no Gaussian in the reference and is rejected). use_ratio = 0 is ratio
 * None; otherwise the fit is repeated with a rising threshold until the
 * fitted power over the pattern's falls below `ratio` (FitGauss.py:126-161).
 * Writes the 6 parameters (x0, y0, xs, ys, theta, amp) to host memory
 * `popt`, and where p0 is not NULL the simplex's starting point there (the
 * image-moment estimates of calcEstimates, FitGauss.py:13-65, and the
 * pattern's maximum as amp). Synchronises `stream` once per objective value. Status 4: the
 * ratio rounds would repeat for ever (the reference never returns there).
 * po_generate_gauss_dev: generateGauss (FitGauss.py:197-228) of host
 * parameters popt on the n points of a device grid into the device buffer
 * out (n doubles), scale 0 LIN or 2 dB; queued on `stream`.
 * po_fmin: the downhill-simplex minimiser behind both, scipy.optimize.fmin's
 * method (FitGauss.py:128, :150), with a host objective f(x, &fx, ctx)
 * returning 0 (a non-zero return aborts with that status). maxiter or maxfun
 * <= 0 stands for None (the default 200 n). Writes xopt (n), and fopt,
 * iterations and function calls where those pointers are not NULL. */
typedef int (*po_objective)(const double *x, double *fx, void *ctx);
int po_fit_gauss_abs_dev(int ncx, int ncy, const double *grid7, const double *f_re, const double *f_im, double thres,
                         int scale, int use_ratio, double ratio, double *popt, double *p0, void *stream);
int po_generate_gauss_dev(long n, const double *grid7, const double *popt, int scale, double *out, void *stream);
int po_fmin(int n, const double *x0, double xtol, double ftol, long maxiter, long maxfun, po_objective f, void *ctx,
            double *xopt, double *fopt, long *iterations, long *fcalls);

/* Frame half-extent, in wavelengths, of this thread's last mixed-precision
 * host-buffer call (po_run_d, po_adjoint_d); 0 after any other call. It sets
 * the mixed path's hi/lo quantum, so its error grows with it (the path holds
 * 1e-5 relative L2 up to about 5e4); the library computes it on the device
 * and reads it back with the call's results. */
double po_last_extent(void);

/* Number of near-tangent (source, target) pairs (|n . R_hat| < 1e-6) that
 * this thread's last mixed-precision host-buffer call (po_run_d,
 * po_adjoint_d) left out of its FP32 sums and decided, and summed if lit, in
 * FP64 with the reference's rounding; 0 after any other call. A count above
 * the call's list capacity came with device error 103. */
unsigned long long po_last_band_pairs(void);

/* ---- explicit-grid, double-precision entry (host buffers) ---------------
 * New; the reference has no equivalent (its C-ABI regenerates grids inside
 * every call, Kernelsf.cu:1643-1644, so it cannot take perturbed surfaces or
 * target subsets, and its float ABI rounds positions, BindUtils.py:277-328).
 *
 *   src7  7*ns doubles, rows x y z nx ny nz area (row-major over (ncx, ncy))
 *   cur   12*ns doubles in c2Bundle row order (r1x r1y r1z i1x i1y i1z
 *         r2x ... i2z: J then M), or 2*ns (re, im) for scalar mode
 *   tgt7  7*nt doubles, rows x y z nx ny nz area; for FF x is the polar
 *         angle and y the azimuth (radians), as the reference's AoE grid
 *   out   po_n_out(mode)*nt doubles in bundle row order
 *   precision  0 mixed (FP32 bulk + split hi/lo phase), 1 plain FP64
 *   ns, nt     0 .. 2^31 - 1 (device indices are 32-bit; larger is status 1)
 *
 * Whether M == 0 (which selects the kernels without magnetic terms) is
 * settled from the first 4096 magnetic values on the host when one of them
 * is non-zero, else by a device check of all of them. The call synchronises
 * once, on a private stream; page-locked buffers make its copies fastest.
 */
int po_n_out(int mode);
int po_run_d(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
             const double *cur, long nt, const double *tgt7,
             double k, double epsilon, double t_direction, int precision, double *out);

/* ---- device-pointer entry ------------------------------------------------
 * As po_run_d, but every array is device memory and the work is queued on
 * `stream` (a cudaStream_t; NULL = legacy default stream). The call returns
 * once the work is queued; device scratch is stream-ordered.
 * flags bit 0: caller guarantees M == 0 (JM outputs, PEC chains), which
 * selects the kernel variant that skips the magnetic-current terms.
 */
int po_run_dev(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
               const double *cur, long nt, const double *tgt7,
               double k, double epsilon, double t_direction, int precision, int flags,
               double *out, void *stream);

/* ---- allocation-free device entry ------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory: a framework that reserves the GPU's memory for its own pool (an
 * allocation from inside it fails or fragments that pool), or a
 * latency-critical loop that cannot take the device-wide synchronisation of
 * cudaFree. Same arguments and results as po_run_dev in mixed precision, plus
 * `status`: an optional device int, cleared at the start of the call and set
 * to a device error code (101 a kernel gave up a bounded wait, 103 more than
 * 16,384 near-tangent pairs; see po_device_error). With status == NULL the
 * code goes to an internal word inside the array instead, which stays set across calls
 * until po_device_error reads and clears it (po_device_error allocates
 * nothing).
 * The scratch is a fixed 64 MiB device array inside the library, held by
 * every GPU that loads it until the process exits; problems needing more
 * (about 88*ns + 128*nt bytes, plus 96*nt per extra source chunk) are
 * rejected with status 5 and a message. The first call on a device looks up
 * that array's address: make it before any stream capture. All calls share
 * the array, so calls that overlap on the GPU race; the caller serialises
 * them. Calls no cudaMalloc/cudaFree or other allocating routine. */
int po_run_dev_static(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
                      const double *cur, long nt, const double *tgt7,
                      double k, double epsilon, double t_direction, int flags,
                      double *out, int *status, void *stream);

/* ---- adjoint (vector-Jacobian product) ----------------------------------
 * New; the reference has no derivatives. For a real loss L of one
 * propagation's outputs, `cot` holds dL/d(output) in the output's row layout
 * (po_n_out(mode) rows x nt, real and imaginary parts as separate rows).
 * Returns, for any non-NULL destination:
 *   grad_cur  dL/d(cur), 12 rows x ns (c2Bundle order, real rows); for the
 *             scalar mode 2 rows (re, im) of the source field
 *   grad_ds   dL/d(delta_s), ns: displacement of each source point along its
 *             normal, normals and areas frozen (the reference's surface-error
 *             convention, InterfaceReflector.cpp:852-866)
 *   grad_dt   dL/d(delta_t), nt: the same for target points (near field and
 *             scalar)
 * Every mode. EHP is nonlinear in the target's fields: its adjoint runs the
 * EH forward again and maps the cotangents through the EHP reflection's
 * Jacobian there (forward-mode dual numbers) before the EH adjoint. The
 * Green's function is recomputed, nothing of size ns*nt is stored.
 * precision 0 mixed, 1 plain FP64. flags bit 0: M == 0 on the source.
 * po_adjoint_dev queues on `stream` (device pointers); po_adjoint_d takes host
 * buffers and synchronises. */
int po_adjoint_dev(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
                   const double *cur, long nt, const double *tgt7,
                   double k, double epsilon, double t_direction, int precision, int flags,
                   const double *cot, double *grad_cur, double *grad_ds, double *grad_dt, void *stream);
int po_adjoint_d(int mode, long ns, const double *src7, int gmode, int ncx, int ncy,
                 const double *cur, long nt, const double *tgt7,
                 double k, double epsilon, double t_direction, int precision,
                 const double *cot, double *grad_cur, double *grad_ds, double *grad_dt);

/* Number of kernel launches the last call on this thread queued. */
int po_last_launches(void);

/* Synchronises `stream`, then returns (and clears) the device error words in
 * *code: 0 when every kernel finished normally, 101 when a kernel gave up a
 * bounded wait for a tile copy, 103 when a call met more near-tangent
 * (source, target) pairs than its list holds (every pair of a call of up
 * to 2^22 pairs, else one entry per 65,536 pairs, between 2^22 and 2^24;
 * 16,384 for po_run_dev_static), 102 when the device normal generator overran its
 * bound; the results of such a call are invalid. It reads the
 * word of the allocating entries and the internal word of po_run_dev_static
 * (calls made with status == NULL); it allocates nothing. */
int po_device_error(void *stream, int *code);

/* Self-test of the failure detection (no counterpart in the reference, whose
 * CUDA error path calls exit(), src/include/MemUtils.h:27-34). One CTA waits
 * on an mbarrier that nothing arrives on, with `limit` bounded polls (the
 * kernels' own wait), gives up, and sets 101 in: `err` (a device int) when
 * non-NULL, else the allocating entries' word (word == 0) or the internal
 * word of po_run_dev_static (word == 1; 3 if that entry has not run on this
 * device yet). No copy is in flight while it waits, so giving up is clean.
 * Queued on `stream`. */
int po_wait_selftest(unsigned limit, int *err, int word, void *stream);

/* Bytes of the library's own scratch pool on the current device that are in
 * use (allocated and not yet freed in stream order); 0 before the pool
 * exists. The pool is private: the device's default pool is not changed. */
int po_scratch_in_use(unsigned long long *bytes);

/* ---- measurement support --------------------------------------------------
 * po_timing_enable(n) arms n CUDA event pairs, recorded on the launching
 * stream around each subsequent main-kernel launch (mixed or FP64);
 * po_timing_collect copies up to `max` durations in ms (in launch order,
 * synchronising on the events) and re-arms. n = 0 disables. */
int po_timing_enable(int slots);
int po_timing_collect(float *ms, int max);

/* FP32 FFMA throughput probe: `blocks` x 256 threads, each running 8
 * independent FMA chains for `iters` steps (16 flops per thread-step); out
 * holds blocks*256 floats (device). Queued on `stream`. */
int po_fp32_probe(int blocks, int iters, float *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PO_GB300_H */
