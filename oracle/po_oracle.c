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
