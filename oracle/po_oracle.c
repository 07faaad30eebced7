/*
 * po_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of PyPO's CPU physical-optics integrator. It is
 * the checker that the CUDA engine in pypo_gb300/ is compared against. Only
 * tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
 * bench.py may load this library. The product path never calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py compares this file's output
 * with golden vectors produced by the reference's own CPU library, compiled
 * from its sources by oracle/build_ref.sh (tests/golden/make_golden.py).
 *
 * What it restates (reference file:line, paths inside PyPO):
 *   - near-field kernel  fieldAtPoint        src/CPU/Propagation.h:977-1144
 *   - JM  (PEC)          propagateBeam_JM_PEC src/CPU/Propagation.h:269-323
 *   - EH                 propagateBeam_EH     src/CPU/Propagation.h:574-617
 *   - JMEH (PEC)         propagateBeam_JMEH_PEC src/CPU/Propagation.h:482-555
 *   - EHP                propagateBeam_EHP    src/CPU/Propagation.h:805-914
 *   - FF                 propagateToFarField + farfieldAtPoint
 *                                            src/CPU/Propagation.h:1581-1781
 *   - scalar             propagateScalarBeam + fieldScalarAtPoint
 *                                            src/CPU/Propagation.h:933-956, 1279-1331
 *   - constants          Propagation ctor    src/CPU/Propagation.h:193-249
 *   - target split       parallelProp_*      src/CPU/Propagation.h:1348-1562
 *
 * Conventions kept from the reference:
 *   - trapezoid weights: the x/u end rows always get 1/2; the y/v end columns
 *     get 1/2 unless gmode == 1 (uv grids are periodic in v);
 *   - the y/v sum is formed first and then weighted into the x/u sum;
 *   - a source is skipped when n_s . R_hat < 0 (near field) or n_s . r_hat < 0
 *     (far field), for both time directions; scalar mode has no such test;
 *   - the physical constants are float literals widened to double.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define OR_JM 0
#define OR_EH 1
#define OR_JMEH 2
#define OR_EHP 3
#define OR_FF 4
#define OR_SCALAR 5

typedef double complex cplx;

typedef struct {
    int mode;
    long ns;
    const double *src;  /* 7*ns: x, y, z, nx, ny, nz, area */
    const double *cur;  /* 12*ns in c2Bundle order, or 2*ns (re, im) for scalar */
    int gmode, ncx, ncy;
    int unit_w;         /* gmode < 0: explicit point cloud, unit weights */
    long nt;
    const double *tgt;  /* 7*nt: x, y, z, nx, ny, nz, area */
    const long *tidx;   /* optional subset of target indices */
    long nout_pts;      /* number of points written */
    double k, t_dir;
    double pref;        /* k^2 / (4 pi) with the float-literal pi */
    double pif;
    double zeta_inv;
    double *out;
    long begin, end;    /* range over output points */
} or_job;

static double or_half_weight(int gmode, int ncx, int ncy, int xu, int yv, int *yhalf)
{
    *yhalf = (gmode >= 0) && (gmode != 1) && (yv == 0 || yv == ncy - 1);
    return (gmode >= 0 && (xu == 0 || xu == ncx - 1)) ? 0.5 : 1.0;
}

static double or_x_weight(const void *job, int xu);

/* Near-field E and H at one target point. Propagation.h:977-1144. */
static void or_field_at_point(const or_job *jb, const double pt[3], cplx e[3], cplx h[3])
{
    const double *sx = jb->src, *sy = jb->src + jb->ns, *sz = jb->src + 2 * jb->ns;
    const double *snx = jb->src + 3 * jb->ns, *sny = jb->src + 4 * jb->ns, *snz = jb->src + 5 * jb->ns;
    const double *sa = jb->src + 6 * jb->ns;
    const double *c = jb->cur;
    const long n = jb->ns;
    const double k = jb->k, t = jb->t_dir;
    for (int q = 0; q < 3; ++q) { e[q] = 0; h[q] = 0; }

    for (int xu = 0; xu < jb->ncx; ++xu) {
        cplx ye[3] = {0, 0, 0}, yh[3] = {0, 0, 0};
        for (int yv = 0; yv < jb->ncy; ++yv) {
            long i = (long)xu * jb->ncy + yv;
            cplx js[3], ms[3];
            for (int q = 0; q < 3; ++q) {
                js[q] = c[q * n + i] + I * c[(3 + q) * n + i];
                ms[q] = c[(6 + q) * n + i] + I * c[(9 + q) * n + i];
            }
            double rv[3] = {pt[0] - sx[i], pt[1] - sy[i], pt[2] - sz[i]};
            double R = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
            double R_inv = 1.0 / R;
            double kR = k * R;
            double u = 1.0 / kR;
            double rh[3] = {rv[0] * R_inv, rv[1] * R_inv, rv[2] * R_inv};
            double ndr = snx[i] * rh[0] + sny[i] * rh[1] + snz[i] * rh[2];
            if (ndr < 0) continue;

            cplx s1 = u * (-I + t * u + I * u * u);
            cplx s2 = u * (I - t * 3.0 * u - 3.0 * I * u * u);
            cplx s3 = t * (I * u - t * u * u);

            cplx jdr = js[0] * rh[0] + js[1] * rh[1] + js[2] * rh[2];
            cplx mdr = ms[0] * rh[0] + ms[1] * rh[1] + ms[2] * rh[2];
            cplx mxr[3] = {ms[1] * rh[2] - ms[2] * rh[1], ms[2] * rh[0] - ms[0] * rh[2],
                           ms[0] * rh[1] - ms[1] * rh[0]};
            cplx jxr[3] = {js[1] * rh[2] - js[2] * rh[1], js[2] * rh[0] - js[0] * rh[2],
                           js[0] * rh[1] - js[1] * rh[0]};
            cplx green = jb->pref * cexp(t * I * k * R) * sa[i];

            int yhalf;
            (void)or_half_weight(jb->gmode, jb->ncx, jb->ncy, xu, yv, &yhalf);
            double w = yhalf ? 0.5 : 1.0;
            for (int q = 0; q < 3; ++q) {
                ye[q] += w * (js[q] * s1 + jdr * rh[q] * s2 + mxr[q] * s3) * green;
                yh[q] += w * (ms[q] * s1 + mdr * rh[q] * s2 - jxr[q] * s3) * green;
            }
        }
        double wx = or_x_weight(jb, xu);
        for (int q = 0; q < 3; ++q) { e[q] += wx * ye[q]; h[q] += wx * yh[q]; }
    }
}

/* Far-field E and H in direction r_hat. Propagation.h:1656-1781. */
static void or_farfield_at_point(const or_job *jb, const double rh[3], cplx e[3], cplx h[3])
{
    const double *sx = jb->src, *sy = jb->src + jb->ns, *sz = jb->src + 2 * jb->ns;
    const double *snx = jb->src + 3 * jb->ns, *sny = jb->src + 4 * jb->ns, *snz = jb->src + 5 * jb->ns;
    const double *sa = jb->src + 6 * jb->ns;
    const double *c = jb->cur;
    const long n = jb->ns;
    const double k = jb->k, t = jb->t_dir;
    for (int q = 0; q < 3; ++q) { e[q] = 0; h[q] = 0; }

    for (int xu = 0; xu < jb->ncx; ++xu) {
        cplx ye[3] = {0, 0, 0}, yh[3] = {0, 0, 0};
        for (int yv = 0; yv < jb->ncy; ++yv) {
            long i = (long)xu * jb->ncy + yv;
            double ndr = snx[i] * rh[0] + sny[i] * rh[1] + snz[i] * rh[2];
            if (ndr < 0) continue;
            cplx js[3], ms[3];
            for (int q = 0; q < 3; ++q) {
                js[q] = c[q * n + i] + I * c[(3 + q) * n + i];
                ms[q] = c[(6 + q) * n + i] + I * c[(9 + q) * n + i];
            }
            cplx jdr = js[0] * rh[0] + js[1] * rh[1] + js[2] * rh[2];
            cplx mdr = ms[0] * rh[0] + ms[1] * rh[1] + ms[2] * rh[2];
            cplx rxm[3] = {rh[1] * ms[2] - rh[2] * ms[1], rh[2] * ms[0] - rh[0] * ms[2],
                           rh[0] * ms[1] - rh[1] * ms[0]};
            cplx rxj[3] = {rh[1] * js[2] - rh[2] * js[1], rh[2] * js[0] - rh[0] * js[2],
                           rh[0] * js[1] - rh[1] * js[0]};
            double rpr = sx[i] * rh[0] + sy[i] * rh[1] + sz[i] * rh[2];
            cplx green = -jb->pref * I * cexp(-t * I * k * rpr) * sa[i];
            int yhalf;
            (void)or_half_weight(jb->gmode, jb->ncx, jb->ncy, xu, yv, &yhalf);
            double w = yhalf ? 0.5 : 1.0;
            for (int q = 0; q < 3; ++q) {
                ye[q] += w * (js[q] - jdr * rh[q] + t * rxm[q]) * green;
                yh[q] += w * (ms[q] - mdr * rh[q] - t * rxj[q]) * green;
            }
        }
        double wx = or_x_weight(jb, xu);
        for (int q = 0; q < 3; ++q) { e[q] += wx * ye[q]; h[q] += wx * yh[q]; }
    }
}

/* Scalar Green's-function sum. Propagation.h:1279-1331 (CPU phase sign). */
static cplx or_scalar_at_point(const or_job *jb, const double pt[3])
{
    const double *sx = jb->src, *sy = jb->src + jb->ns, *sz = jb->src + 2 * jb->ns;
    const double *sa = jb->src + 6 * jb->ns;
    const double *fre = jb->cur, *fim = jb->cur + jb->ns;
    const double k = jb->k, t = jb->t_dir;
    cplx out = 0;
    for (int xu = 0; xu < jb->ncx; ++xu) {
        cplx yf = 0;
        for (int yv = 0; yv < jb->ncy; ++yv) {
            long i = (long)xu * jb->ncy + yv;
            cplx f = fre[i] + I * fim[i];
            double rv[3] = {pt[0] - sx[i], pt[1] - sy[i], pt[2] - sz[i]};
            double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
            cplx term = -k * k * f * cexp(t * -I * k * r) / (4 * jb->pif * r) * sa[i];
            int yhalf;
            (void)or_half_weight(jb->gmode, jb->ncx, jb->ncy, xu, yv, &yhalf);
            yf += yhalf ? 0.5 * term : term;
        }
        out += or_x_weight(jb, xu) * yf;
    }
    return out;
}

static double or_x_weight(const void *job, int xu)
{
    const or_job *jb = (const or_job *)job;
    if (jb->unit_w) return 1.0;
    return (xu == 0 || xu == jb->ncx - 1) ? 0.5 : 1.0;
}

static void or_norm(const double v[3], double o[3])
{
    double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (nrm <= DBL_TRUE_MIN) nrm = DBL_TRUE_MIN;
    for (int q = 0; q < 3; ++q) o[q] = v[q] / nrm;
}

static void or_cross(const double a[3], const double b[3], double o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Reflection epilogue of EHP. Propagation.h:840-913; snell Utils.h:421-432. */
static void or_ehp(const cplx e[3], const cplx h[3], const double n[3], double zeta_inv,
                   cplx er[3], cplx hr[3], double sr[3])
{
    double s[3], si[3], tmp[3], pip[3], pia[3], prp[3], pra[3];
    cplx hc[3] = {conj(h[0]), conj(h[1]), conj(h[2])};
    cplx exh[3] = {e[1] * hc[2] - e[2] * hc[1], e[2] * hc[0] - e[0] * hc[2],
                   e[0] * hc[1] - e[1] * hc[0]};
    for (int q = 0; q < 3; ++q) s[q] = creal(exh[q]);
    or_norm(s, si);
    or_cross(si, n, tmp);
    or_norm(tmp, pip);
    or_cross(pip, si, pia);
    double f = 2.0 * (si[0] * n[0] + si[1] * n[1] + si[2] * n[2]);
    for (int q = 0; q < 3; ++q) sr[q] = si[q] - n[q] * f;
    or_cross(sr, n, tmp);
    or_norm(tmp, prp);
    or_cross(sr, prp, pra);
    cplx ep = e[0] * prp[0] + e[1] * prp[1] + e[2] * prp[2];
    cplx ea = e[0] * pra[0] + e[1] * pra[1] + e[2] * pra[2];
    for (int q = 0; q < 3; ++q) er[q] = -ep * pip[q] - ea * pia[q];
    cplx t[3] = {sr[1] * er[2] - sr[2] * er[1], sr[2] * er[0] - sr[0] * er[2],
                 sr[0] * er[1] - sr[1] * er[0]};
    for (int q = 0; q < 3; ++q) hr[q] = t[q] * zeta_inv;
}

static void *or_worker(void *arg)
{
    const or_job *jb = (const or_job *)arg;
    const long nt = jb->nt, np = jb->nout_pts;
    const double *tx = jb->tgt, *ty = jb->tgt + nt, *tz = jb->tgt + 2 * nt;
    const double *tnx = jb->tgt + 3 * nt, *tny = jb->tgt + 4 * nt, *tnz = jb->tgt + 5 * nt;
    double *o = jb->out;
    for (long p = jb->begin; p < jb->end; ++p) {
        long i = jb->tidx ? jb->tidx[p] : p;
        double pt[3] = {tx[i], ty[i], tz[i]};
        double nn[3] = {tnx[i], tny[i], tnz[i]};
        cplx e[3], h[3];
        if (jb->mode == OR_SCALAR) {
            cplx v = or_scalar_at_point(jb, pt);
            o[p] = creal(v);
            o[np + p] = cimag(v);
            continue;
        }
        if (jb->mode == OR_FF) {
            /* x = polar angle, y = azimuth. Propagation.h:1605-1615. */
            double ph = pt[0], th = pt[1];
            double rh[3] = {cos(th) * sin(ph), sin(th) * sin(ph), cos(ph)};
            or_farfield_at_point(jb, rh, e, h);
        } else {
            or_field_at_point(jb, pt, e, h);
        }
        cplx a[3], b[3];
        int base = 0;
        switch (jb->mode) {
        case OR_EH:
        case OR_FF:
            for (int q = 0; q < 3; ++q) { a[q] = e[q]; b[q] = h[q]; }
            break;
        case OR_JM:
        case OR_JMEH: {
            cplx jt[3] = {nn[1] * h[2] - nn[2] * h[1], nn[2] * h[0] - nn[0] * h[2],
                          nn[0] * h[1] - nn[1] * h[0]};
            for (int q = 0; q < 3; ++q) { a[q] = 2.0 * jt[q]; b[q] = 0; }
            if (jb->mode == OR_JMEH) {
                for (int q = 0; q < 3; ++q) {
                    o[(12 + q) * np + p] = creal(e[q]);
                    o[(15 + q) * np + p] = cimag(e[q]);
                    o[(18 + q) * np + p] = creal(h[q]);
                    o[(21 + q) * np + p] = cimag(h[q]);
                }
            }
            break;
        }
        case OR_EHP: {
            double sr[3];
            or_ehp(e, h, nn, jb->zeta_inv, a, b, sr);
            for (int q = 0; q < 3; ++q) o[(12 + q) * np + p] = sr[q];
            break;
        }
        default:
            break;
        }
        for (int q = 0; q < 3; ++q) {
            o[(base + q) * np + p] = creal(a[q]);
            o[(base + 3 + q) * np + p] = cimag(a[q]);
            o[(base + 6 + q) * np + p] = creal(b[q]);
            o[(base + 9 + q) * np + p] = cimag(b[q]);
        }
    }
    return NULL;
}

/* Number of output arrays per mode (c2Bundle 12, c4Bundle 24, c2rBundle 15, arrC1 2). */
int po_oracle_nout(int mode)
{
    static const int n[6] = {12, 12, 24, 15, 12, 2};
    return (mode >= 0 && mode < 6) ? n[mode] : -1;
}

/*
 * Run one propagation. src/tgt are 7-row SoA (x, y, z, nx, ny, nz, area);
 * cur is 12-row c2Bundle order (r1x r1y r1z i1x i1y i1z r2x ... i2z) or 2-row
 * (re, im) for scalar mode. Writes po_oracle_nout(mode) rows of length
 * (tidx ? nidx : nt) into out. Returns 0 on success.
 */
int po_oracle_run(int mode, long ns, const double *src, const double *cur,
                  int gmode, int ncx, int ncy,
                  long nt, const double *tgt, const long *tidx, long nidx,
                  double k, double epsilon, double t_dir, int nthreads, double *out)
{
    if (mode < 0 || mode > 5 || ns < 0 || nt < 0) return 1;
    int unit_w = 0;
    if (gmode < 0) {   /* point cloud: one row of ns points, unit weights (not a reference mode) */
        unit_w = 1;
        ncx = ns > 0 ? 1 : 0;
        ncy = (int)ns;
    } else if ((long)ncx * ncy != ns) {
        return 1;
    }
    if (nthreads < 1) nthreads = 1;
    /* Constants: float literals widened to double, Propagation.h:196-203. */
    const double pif = (double)3.14159265359f;
    const double c_l = (double)2.99792458e8f;
    const double mu0 = (double)1.2566370614e-6f;
    const double eps_vac = 1.0 / (mu0 * c_l * c_l);
    const double eps = epsilon * eps_vac;
    const double zeta = sqrt(mu0 / eps);

    or_job base;
    memset(&base, 0, sizeof(base));
    base.mode = mode;
    base.ns = ns;
    base.src = src;
    base.cur = cur;
    base.gmode = gmode;
    base.ncx = ncx;
    base.ncy = ncy;
    base.unit_w = unit_w;
    base.nt = nt;
    base.tgt = tgt;
    base.tidx = tidx;
    base.nout_pts = tidx ? nidx : nt;
    base.k = k;
    base.t_dir = t_dir;
    base.pref = k * k / (4. * pif);
    base.pif = pif;
    base.zeta_inv = 1.0 / zeta;
    base.out = out;

    const long np = base.nout_pts;
    if (np == 0) return 0;
    if (nthreads > np) nthreads = (int)np;
    or_job *jobs = (or_job *)malloc(sizeof(or_job) * nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    char *live = (char *)calloc(nthreads, 1);
    if (!jobs || !th || !live) { free(jobs); free(th); free(live); return 2; }
    long step = (np + nthreads - 1) / nthreads;
    for (int w = 0; w < nthreads; ++w) {
        jobs[w] = base;
        jobs[w].begin = w * step;
        jobs[w].end = (w + 1) * step < np ? (w + 1) * step : np;
        if (jobs[w].begin >= jobs[w].end) continue;
        if (nthreads == 1 || pthread_create(&th[w], NULL, or_worker, &jobs[w]) != 0)
            or_worker(&jobs[w]);
        else
            live[w] = 1;
    }
    for (int w = 0; w < nthreads; ++w)
        if (live[w]) pthread_join(th[w], NULL);
    free(live);
    free(jobs);
    free(th);
    return 0;
}

/* ------------------------------------------------------------------ adjoint
 *
 * FP64 vector-Jacobian product of po_oracle_run for modes JM, EH, JMEH, FF and
 * scalar. The reference has no derivatives; this is the CPU statement of the
 * engine's adjoint (the formulas of pypo_gb300/csrc/po_adjoint.cu, written
 * here from the forward above), used as a checker and as the CPU baseline's
 * adjoint leg. For a real loss L = sum(cot * out):
 *   - the cotangent rows map onto (gE, gH) per target: EH, FF direct; JM
 *     J = 2 n x H gives gH += 2 gJ x n; JMEH adds its E, H rows; FF then
 *     becomes gS_J = P gE + t r x gH, gS_M = P gH - t r x gE (P = I - r r^T);
 *   - currents: Jbar' = sum_t conj(c1) gE + conj(c2)(gE.d)d + conj(c3)(gH x d),
 *     Mbar' = sum_t conj(c1) gH + conj(c2)(gH.d)d - conj(c3)(gE x d), with
 *     c1 = G s1, c2 = G s2 / R^2, c3 = G s3 / R (s1..s3 and G = e^{t j k R} as
 *     in or_field_at_point); far field Jbar' = sum_t conj(G) gS_J (and M);
 *     the gradient with respect to the caller's currents is
 *     conj(prefactor * weight * area) times these;
 *   - displacement of a point along its frozen normal (areas frozen, the
 *     reference's surface-error convention, InterfaceReflector.cpp:852-866):
 *     phi(d) = Re[a.E + b.H] for one pair, a = conj gE, b = conj gH, d = r_t - r_s;
 *     grad phi = Re[sigma d + c2 grad(beta) + c3 W] with alpha = a.J + b.M,
 *     beta = (J.d)(a.d) + (M.d)(b.d), W = a x M - b x J,
 *     sigma = d1 alpha + d2 beta + d3 (W.d) and the radial derivatives
 *     d1 = G/R^2 [t(1-3u^2) + j(2u-3u^3)], d2 = G/R^4 [-t(1-15u^2) + j(-6u+15u^3)],
 *     d3 = G/R^3 [-(1-3u^2) - 3jtu]; dL/d delta_s = -n_s . sum_t grad phi,
 *     dL/d delta_t = n_t . sum_s grad phi; far field
 *     dL/d delta_s = t k (n_s . r) Im[G (conj(gS_J).J' + conj(gS_M).M')];
 *     scalar: out = sum c f with c = -k^2 e^{-t j k r} w A / (4 pi r),
 *     dc/dr = c (-t j k - 1/r);
 *   - the illumination mask is piecewise constant: its derivative is dropped.
 */

typedef struct {
    int mode, side;          /* side 0: one source per item; 1: one target per item */
    long ns, nt;
    const double *src, *tgt;
    const cplx *Jp, *Mp;     /* folded currents, 3 per source (scalar: Jp[0] = f') */
    const cplx *gE, *gH;     /* mapped cotangents, 3 per target (scalar: gE[0]) */
    const double *dir;       /* far field: r_hat, 3 per target */
    double k, t;
    double *acc;             /* side 0: 13 per source (Jbar' re/im 6, Mbar' 6, displacement) */
    double *gdt;             /* side 1: one per target */
    long begin, end;
} oa_job;

static cplx oa_dot_r(const cplx *v, const double *x) { return v[0] * x[0] + v[1] * x[1] + v[2] * x[2]; }
static cplx oa_dot_c(const cplx *a, const cplx *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void oa_cross_r(const cplx *v, const double *x, cplx *o)
{
    o[0] = v[1] * x[2] - v[2] * x[1];
    o[1] = v[2] * x[0] - v[0] * x[2];
    o[2] = v[0] * x[1] - v[1] * x[0];
}

/* Near-field pair: c2, c3 and the gradient of phi along `nv`, the caller's
 * normal (n . grad phi). Lit test and rounding as or_field_at_point. */
static int oa_nf_pair(const oa_job *jb, long s, long ti, double d[3], double *R_out, cplx *c1, cplx *c2, cplx *c3,
                      cplx *d1, cplx *d2, cplx *d3)
{
    const double *sp = jb->src, *tp = jb->tgt;
    const long ns = jb->ns, nt = jb->nt;
    d[0] = tp[ti] - sp[s];
    d[1] = tp[nt + ti] - sp[ns + s];
    d[2] = tp[2 * nt + ti] - sp[2 * ns + s];
    const double R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double rinv = 1.0 / R;
    const double rh[3] = {d[0] * rinv, d[1] * rinv, d[2] * rinv};
    const double ndr = sp[3 * ns + s] * rh[0] + sp[4 * ns + s] * rh[1] + sp[5 * ns + s] * rh[2];
    if (ndr < 0) return 0;
    const double t = jb->t, u = 1.0 / (jb->k * R), u2 = u * u, u3 = u2 * u;
    const double rinv2 = rinv * rinv;
    const cplx G = cexp(t * I * jb->k * R);
    *c1 = G * (t * u2 + I * (u3 - u));
    *c2 = (-3.0 * *c1 - 2.0 * I * u * G) * rinv2;
    *c3 = G * (-u2 * rinv + I * t * u * rinv);
    *d1 = G * (t * (1 - 3 * u2) + I * (2 * u - 3 * u3)) * rinv2;
    *d2 = G * (-t * (1 - 15 * u2) + I * (-6 * u + 15 * u3)) * rinv2 * rinv2;
    *d3 = G * (-(1 - 3 * u2) - 3 * I * t * u) * rinv2 * rinv;
    *R_out = R;
    return 1;
}

/* n . grad_d phi for one near-field pair (J, M the folded currents of the
 * source; a, b the conjugated cotangents of the target). */
static double oa_nf_grad(const double d[3], const double n[3], cplx c2, cplx c3, cplx d1, cplx d2, cplx d3,
                         const cplx *J, const cplx *M, const cplx *a, const cplx *b)
{
    const cplx Jd = oa_dot_r(J, d), Md = oa_dot_r(M, d), ad = oa_dot_r(a, d), bd = oa_dot_r(b, d);
    const cplx alpha = oa_dot_c(a, J) + oa_dot_c(b, M);
    const cplx beta = Jd * ad + Md * bd;
    cplx Mxd[3], Jxd[3], Mxn[3], Jxn[3];
    oa_cross_r(M, d, Mxd);
    oa_cross_r(J, d, Jxd);
    oa_cross_r(M, n, Mxn);
    oa_cross_r(J, n, Jxn);
    const cplx Wd = oa_dot_c(a, Mxd) - oa_dot_c(b, Jxd);
    const cplx Wn = oa_dot_c(a, Mxn) - oa_dot_c(b, Jxn);
    const cplx gbn = ad * oa_dot_r(J, n) + Jd * oa_dot_r(a, n) + bd * oa_dot_r(M, n) + Md * oa_dot_r(b, n);
    const cplx sig = d1 * alpha + d2 * beta + d3 * Wd;
    const double ndd = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
    return creal(sig) * ndd + creal(c2 * gbn) + creal(c3 * Wn);
}

static void *oa_worker(void *arg)
{
    const oa_job *jb = (const oa_job *)arg;
    const long ns = jb->ns, nt = jb->nt;
    const double *sp = jb->src, *tp = jb->tgt;
    const double k = jb->k, t = jb->t;
    for (long it = jb->begin; it < jb->end; ++it) {
        if (jb->side == 1) {   /* target displacement (near field) */
            const long ti = it;
            const double n[3] = {tp[3 * nt + ti], tp[4 * nt + ti], tp[5 * nt + ti]};
            cplx a[3], b[3];
            for (int q = 0; q < 3; ++q) { a[q] = conj(jb->gE[3 * ti + q]); b[q] = conj(jb->gH[3 * ti + q]); }
            double acc = 0;
            for (long s = 0; s < ns; ++s) {
                double d[3], R;
                cplx c1, c2, c3, d1, d2, d3;
                if (jb->mode == OR_SCALAR) {
                    d[0] = tp[ti] - sp[s]; d[1] = tp[nt + ti] - sp[ns + s]; d[2] = tp[2 * nt + ti] - sp[2 * ns + s];
                    R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    const cplx c = cexp(-t * I * k * R) / R;
                    const cplx dcdr = c * (-t * I * k - 1.0 / R);
                    const double ndd = (n[0] * d[0] + n[1] * d[1] + n[2] * d[2]) / R;
                    acc += creal(a[0] * jb->Jp[3 * s] * dcdr) * ndd;
                    continue;
                }
                if (!oa_nf_pair(jb, s, ti, d, &R, &c1, &c2, &c3, &d1, &d2, &d3)) continue;
                acc += oa_nf_grad(d, n, c2, c3, d1, d2, d3, jb->Jp + 3 * s, jb->Mp + 3 * s, a, b);
            }
            jb->gdt[ti] = acc;
            continue;
        }
        const long s = it;
        const double n[3] = {sp[3 * ns + s], sp[4 * ns + s], sp[5 * ns + s]};
        const cplx *J = jb->Jp + 3 * s, *M = jb->Mp + 3 * s;
        cplx jb_[3] = {0, 0, 0}, mb_[3] = {0, 0, 0};
        double dsum = 0;
        for (long ti = 0; ti < nt; ++ti) {
            const cplx *gE = jb->gE + 3 * ti, *gH = jb->gH + 3 * ti;
            if (jb->mode == OR_SCALAR) {
                double d[3] = {tp[ti] - sp[s], tp[nt + ti] - sp[ns + s], tp[2 * nt + ti] - sp[2 * ns + s]};
                const double R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const cplx c = cexp(-t * I * k * R) / R;
                jb_[0] += conj(c) * gE[0];
                const cplx dcdr = c * (-t * I * k - 1.0 / R);
                const double ndd = (n[0] * d[0] + n[1] * d[1] + n[2] * d[2]) / R;
                dsum -= creal(conj(gE[0]) * J[0] * dcdr) * ndd;
                continue;
            }
            if (jb->mode == OR_FF) {
                const double *r = jb->dir + 3 * ti;
                const double ndr = n[0] * r[0] + n[1] * r[1] + n[2] * r[2];
                if (ndr < 0) continue;
                const double rpr = sp[s] * r[0] + sp[ns + s] * r[1] + sp[2 * ns + s] * r[2];
                const cplx G = cexp(-t * I * k * rpr);
                cplx Z = 0;
                for (int q = 0; q < 3; ++q) {
                    jb_[q] += conj(G) * gE[q];
                    mb_[q] += conj(G) * gH[q];
                    Z += conj(gE[q]) * J[q] + conj(gH[q]) * M[q];
                }
                dsum += t * k * cimag(G * Z) * ndr;
                continue;
            }
            double d[3], R;
            cplx c1, c2, c3, d1, d2, d3;
            if (!oa_nf_pair(jb, s, ti, d, &R, &c1, &c2, &c3, &d1, &d2, &d3)) continue;
            const cplx ged = oa_dot_r(gE, d), ghd = oa_dot_r(gH, d);
            cplx ghxd[3], gexd[3];
            oa_cross_r(gH, d, ghxd);
            oa_cross_r(gE, d, gexd);
            for (int q = 0; q < 3; ++q) {
                jb_[q] += conj(c1) * gE[q] + conj(c2) * ged * d[q] + conj(c3) * ghxd[q];
                mb_[q] += conj(c1) * gH[q] + conj(c2) * ghd * d[q] - conj(c3) * gexd[q];
            }
            cplx a[3], b[3];
            for (int q = 0; q < 3; ++q) { a[q] = conj(gE[q]); b[q] = conj(gH[q]); }
            dsum -= oa_nf_grad(d, n, c2, c3, d1, d2, d3, J, M, a, b);
        }
        double *o = jb->acc + 13 * s;
        for (int q = 0; q < 3; ++q) {
            o[q] = creal(jb_[q]);
            o[3 + q] = cimag(jb_[q]);
            o[6 + q] = creal(mb_[q]);
            o[9 + q] = cimag(mb_[q]);
        }
        o[12] = dsum;
    }
    return NULL;
}

static void oa_run(oa_job *base, long n, int nthreads)
{
    if (n <= 0) return;
    if (nthreads > n) nthreads = (int)n;
    if (nthreads < 1) nthreads = 1;
    oa_job *jobs = (oa_job *)malloc(sizeof(oa_job) * nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    char *live = (char *)calloc(nthreads, 1);
    if (!jobs || !th || !live) {   /* run serially */
        base->begin = 0;
        base->end = n;
        oa_worker(base);
        free(jobs); free(th); free(live);
        return;
    }
    long step = (n + nthreads - 1) / nthreads;
    for (int w = 0; w < nthreads; ++w) {
        jobs[w] = *base;
        jobs[w].begin = w * step;
        jobs[w].end = (w + 1) * step < n ? (w + 1) * step : n;
        if (jobs[w].begin >= jobs[w].end) continue;
        if (nthreads == 1 || pthread_create(&th[w], NULL, oa_worker, &jobs[w]) != 0)
            oa_worker(&jobs[w]);
        else
            live[w] = 1;
    }
    for (int w = 0; w < nthreads; ++w)
        if (live[w]) pthread_join(th[w], NULL);
    free(live);
    free(jobs);
    free(th);
}

/*
 * Adjoint of po_oracle_run. cot: po_oracle_nout(mode) rows of nt. Outputs
 * (each may be NULL): grad_cur (12, ns) rows in c2Bundle order (2 rows for
 * scalar), grad_ds (ns), grad_dt (nt; near field and scalar). Returns 0 on
 * success, 1 for a mode without an adjoint (EHP) or bad sizes, 2 on memory.
 */
int po_oracle_adjoint(int mode, long ns, const double *src, const double *cur,
                      int gmode, int ncx, int ncy, long nt, const double *tgt,
                      const double *cot, double k, double epsilon, double t_dir, int nthreads,
                      double *grad_cur, double *grad_ds, double *grad_dt)
{
    (void)epsilon;
    if (mode < 0 || mode > 5 || mode == OR_EHP || ns < 0 || nt < 0) return 1;
    if (mode == OR_FF) grad_dt = NULL;
    int unit_w = gmode < 0;
    if (unit_w) { ncx = ns > 0 ? 1 : 0; ncy = (int)ns; }
    else if ((long)ncx * ncy != ns) return 1;
    const int sc = mode == OR_SCALAR;
    const int ncur = sc ? 2 : 12;
    if (ns == 0 || nt == 0) {
        if (grad_cur) memset(grad_cur, 0, sizeof(double) * ncur * ns);
        if (grad_ds) memset(grad_ds, 0, sizeof(double) * ns);
        if (grad_dt) memset(grad_dt, 0, sizeof(double) * nt);
        return 0;
    }
    const double pif = (double)3.14159265359f;
    const double pref = k * k / (4. * pif);
    /* folded prefactor: near field pref, far field -j pref, scalar -k^2/(4 pi) */
    const cplx fac = sc ? -k * k / (4 * pif) : (mode == OR_FF ? -I * pref : pref);
    cplx *Jp = (cplx *)malloc(sizeof(cplx) * 3 * ns), *Mp = (cplx *)malloc(sizeof(cplx) * 3 * ns);
    cplx *fw = (cplx *)malloc(sizeof(cplx) * ns);
    cplx *gE = (cplx *)calloc(3 * nt, sizeof(cplx)), *gH = (cplx *)calloc(3 * nt, sizeof(cplx));
    double *dir = (double *)malloc(sizeof(double) * 3 * nt);
    double *acc = (double *)calloc(13 * ns, sizeof(double));
    if (!Jp || !Mp || !fw || !gE || !gH || !dir || !acc) {
        free(Jp); free(Mp); free(fw); free(gE); free(gH); free(dir); free(acc);
        return 2;
    }
    for (long s = 0; s < ns; ++s) {
        const int xu = unit_w ? 0 : (int)(s / ncy), yv = unit_w ? 0 : (int)(s % ncy);
        double w = 1.0;
        if (!unit_w) {
            int yhalf;
            w = or_half_weight(gmode, ncx, ncy, xu, yv, &yhalf);
            if (yhalf) w *= 0.5;
        }
        fw[s] = fac * w * src[6 * ns + s];
        if (sc) {
            Jp[3 * s] = fw[s] * (cur[s] + I * cur[ns + s]);
            Jp[3 * s + 1] = Jp[3 * s + 2] = 0;
            Mp[3 * s] = Mp[3 * s + 1] = Mp[3 * s + 2] = 0;
            continue;
        }
        for (int q = 0; q < 3; ++q) {
            Jp[3 * s + q] = fw[s] * (cur[q * ns + s] + I * cur[(3 + q) * ns + s]);
            Mp[3 * s + q] = fw[s] * (cur[(6 + q) * ns + s] + I * cur[(9 + q) * ns + s]);
        }
    }
    for (long i = 0; i < nt; ++i) {
        cplx *e = gE + 3 * i, *h = gH + 3 * i;
        if (sc) { e[0] = cot[i] + I * cot[nt + i]; continue; }
        if (mode == OR_EH || mode == OR_FF)
            for (int q = 0; q < 3; ++q) {
                e[q] = cot[q * nt + i] + I * cot[(3 + q) * nt + i];
                h[q] = cot[(6 + q) * nt + i] + I * cot[(9 + q) * nt + i];
            }
        if (mode == OR_JMEH)
            for (int q = 0; q < 3; ++q) {
                e[q] = cot[(12 + q) * nt + i] + I * cot[(15 + q) * nt + i];
                h[q] = cot[(18 + q) * nt + i] + I * cot[(21 + q) * nt + i];
            }
        if (mode == OR_JM || mode == OR_JMEH) {   /* J = 2 n x H: gH += 2 gJ x n */
            const double n[3] = {tgt[3 * nt + i], tgt[4 * nt + i], tgt[5 * nt + i]};
            cplx g[3], gxn[3];
            for (int q = 0; q < 3; ++q) g[q] = cot[q * nt + i] + I * cot[(3 + q) * nt + i];
            oa_cross_r(g, n, gxn);
            for (int q = 0; q < 3; ++q) h[q] += 2.0 * gxn[q];
        }
        if (mode == OR_FF) {
            const double th = tgt[i], ph = tgt[nt + i];
            double *r = dir + 3 * i;
            r[0] = cos(ph) * sin(th); r[1] = sin(ph) * sin(th); r[2] = cos(th);
            const cplx ed = oa_dot_r(e, r), hd = oa_dot_r(h, r);
            cplx hxr[3], exr[3], sj[3], sm[3];
            /* r x v = -(v x r) */
            oa_cross_r(h, r, hxr);
            oa_cross_r(e, r, exr);
            for (int q = 0; q < 3; ++q) {
                sj[q] = e[q] - ed * r[q] - t_dir * hxr[q];
                sm[q] = h[q] - hd * r[q] + t_dir * exr[q];
            }
            for (int q = 0; q < 3; ++q) { e[q] = sj[q]; h[q] = sm[q]; }
        }
    }
    oa_job base;
    memset(&base, 0, sizeof(base));
    base.mode = mode;
    base.ns = ns;
    base.nt = nt;
    base.src = src;
    base.tgt = tgt;
    base.Jp = Jp;
    base.Mp = Mp;
    base.gE = gE;
    base.gH = gH;
    base.dir = dir;
    base.k = k;
    base.t = t_dir;
    base.acc = acc;
    base.gdt = grad_dt;
    if (grad_cur || grad_ds) {
        base.side = 0;
        oa_run(&base, ns, nthreads);
    }
    if (grad_dt) {
        base.side = 1;
        oa_run(&base, nt, nthreads);
    }
    for (long s = 0; s < ns; ++s) {
        const double *a = acc + 13 * s;
        const cplx f = conj(fw[s]);
        if (grad_cur) {
            if (sc) {
                const cplx g = f * (a[0] + I * a[3]);
                grad_cur[s] = creal(g);
                grad_cur[ns + s] = cimag(g);
            } else {
                for (int g = 0; g < 2; ++g)
                    for (int q = 0; q < 3; ++q) {
                        const cplx v = f * (a[6 * g + q] + I * a[6 * g + 3 + q]);
                        grad_cur[(6 * g + q) * ns + s] = creal(v);
                        grad_cur[(6 * g + 3 + q) * ns + s] = cimag(v);
                    }
            }
        }
        if (grad_ds) grad_ds[s] = a[12];
    }
    free(Jp); free(Mp); free(fw); free(gE); free(gH); free(dir); free(acc);
    return 0;
}
