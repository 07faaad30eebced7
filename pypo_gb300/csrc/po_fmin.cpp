// po_fmin.cpp -- downhill-simplex minimiser for the Gaussian beam fit.
//
// The reference fits its Gaussian with scipy.optimize.fmin (reference
// src/PyPO/FitGauss.py:128, :150): the Nelder-Mead method (Nelder & Mead,
// Computer Journal 7, 1965) in the form scipy 1.x publishes in
// scipy/optimize/_optimize.py (_minimize_neldermead), non-adaptive, without
// bounds. This is a restatement of that method with the same constants and
// the same order of decisions, so that, given bit-identical objective values,
// it visits the same points and returns the same vertex:
//
//   * coefficients: reflection rho = 1, expansion chi = 2, contraction
//     psi = 1/2, shrink sigma = 1/2;
//   * initial simplex: x0, and x0 with coordinate k scaled by 1.05 (or set to
//     2.5e-4 where it is zero), k = 0..N-1;
//   * stop when max |x_i - x_0| <= xatol and max |f_0 - f_i| <= fatol over the
//     simplex (checked before each iteration), or after maxiter iterations or
//     maxfun calls (default 200 N each);
//   * a call past maxfun aborts the step it is in (the simplex keeps the
//     vertices already replaced), and the simplex is re-sorted after every
//     step, by value, stably, NaN last.
//
// Host arithmetic only; the library is built with -ffp-contract=off so that
// a*b - c*d rounds each product as numpy does.
#include <cmath>
#include <limits>
#include <vector>

#include "po_internal.h"

namespace po {

namespace {

bool before(double a, double b)
{
    return a < b || (!std::isnan(a) && std::isnan(b));
}

// Stable sort of the simplex rows by value (insertion sort: N + 1 is small).
void sort_simplex(int n, std::vector<double> &sim, std::vector<double> &fs)
{
    std::vector<double> row(n);
    for (int i = 1; i <= n; ++i) {
        const double f = fs[i];
        for (int c = 0; c < n; ++c) row[c] = sim[(size_t)i * n + c];
        int j = i - 1;
        while (j >= 0 && before(f, fs[j])) {
            fs[j + 1] = fs[j];
            for (int c = 0; c < n; ++c) sim[(size_t)(j + 1) * n + c] = sim[(size_t)j * n + c];
            --j;
        }
        fs[j + 1] = f;
        for (int c = 0; c < n; ++c) sim[(size_t)(j + 1) * n + c] = row[c];
    }
}

}  // namespace

int fmin_nm(int n, const double *x0, double xatol, double fatol, long maxiter, long maxfun, const Objective &func,
            double *xopt, double *fopt, long *nit, long *nfev)
{
    if (n < 1) return fail(1, "fmin: need at least one parameter");
    if (!x0 || !xopt) return fail(1, "fmin: null x0 or xopt");
    const long dflt = 200L * n;
    const long inf = std::numeric_limits<long>::max();
    // maxiter / maxfun <= 0 stand for None; scipy's resolution of the two
    if (maxiter <= 0 && maxfun <= 0) {
        maxiter = dflt;
        maxfun = dflt;
    } else if (maxiter <= 0) {
        maxiter = inf;
    } else if (maxfun <= 0) {
        maxfun = inf;
    }
    const double rho = 1.0, chi = 2.0, psi = 0.5, sigma = 0.5;
    const double nonzdelt = 0.05, zdelt = 0.00025;

    const int np1 = n + 1;
    std::vector<double> sim((size_t)np1 * n), fs(np1, std::numeric_limits<double>::infinity());
    for (int c = 0; c < n; ++c) sim[c] = x0[c];
    for (int k = 0; k < n; ++k) {
        double *y = &sim[(size_t)(k + 1) * n];
        for (int c = 0; c < n; ++c) y[c] = x0[c];
        y[k] = y[k] != 0.0 ? (1.0 + nonzdelt) * y[k] : zdelt;
    }

    long fcalls = 0;
    int err = 0;
    // 0 = value in *fx, 1 = maxfun reached (the step is abandoned), -1 = error
    auto call = [&](const double *x, double *fx) -> int {
        if (fcalls >= maxfun) return 1;
        ++fcalls;
        const int rc = func(x, fx);
        if (rc != 0) {
            err = rc;
            return -1;
        }
        return 0;
    };

    for (int k = 0; k < np1; ++k) {
        const int rc = call(&sim[(size_t)k * n], &fs[k]);
        if (rc < 0) return err;
        if (rc > 0) break;
    }
    sort_simplex(n, sim, fs);

    std::vector<double> xbar(n), xr(n), xe(n), xc(n), xcc(n);
    long iterations = 1;
    while (fcalls < maxfun && iterations < maxiter) {
        // one step; rc > 0 abandons it, as scipy's _MaxFuncCallError does
        int rc = 0;
        bool converged = false;
        {
            double dx = 0.0, df = 0.0;
            for (int i = 1; i < np1; ++i) {
                for (int c = 0; c < n; ++c) {
                    const double d = std::fabs(sim[(size_t)i * n + c] - sim[c]);
                    if (d > dx || std::isnan(d)) dx = std::isnan(dx) ? dx : d;
                }
                const double d = std::fabs(fs[0] - fs[i]);
                if (d > df || std::isnan(d)) df = std::isnan(df) ? df : d;
            }
            converged = dx <= xatol && df <= fatol;
        }
        if (!converged) {
            for (int c = 0; c < n; ++c) {
                double s = sim[c];
                for (int i = 1; i < n; ++i) s += sim[(size_t)i * n + c];
                xbar[c] = s / n;
            }
            const double *worst = &sim[(size_t)n * n];
            for (int c = 0; c < n; ++c) xr[c] = (1.0 + rho) * xbar[c] - rho * worst[c];
            double fxr = 0.0;
            rc = call(xr.data(), &fxr);
            bool shrink = false;
            if (rc == 0) {
                if (fxr < fs[0]) {
                    for (int c = 0; c < n; ++c) xe[c] = (1.0 + rho * chi) * xbar[c] - rho * chi * worst[c];
                    double fxe = 0.0;
                    rc = call(xe.data(), &fxe);
                    if (rc == 0) {
                        const bool take_e = fxe < fxr;
                        for (int c = 0; c < n; ++c) sim[(size_t)n * n + c] = take_e ? xe[c] : xr[c];
                        fs[n] = take_e ? fxe : fxr;
                    }
                } else if (fxr < fs[n - 1]) {
                    for (int c = 0; c < n; ++c) sim[(size_t)n * n + c] = xr[c];
                    fs[n] = fxr;
                } else if (fxr < fs[n]) {
                    // outside contraction
                    for (int c = 0; c < n; ++c) xc[c] = (1.0 + psi * rho) * xbar[c] - psi * rho * worst[c];
                    double fxc = 0.0;
                    rc = call(xc.data(), &fxc);
                    if (rc == 0) {
                        if (fxc <= fxr) {
                            for (int c = 0; c < n; ++c) sim[(size_t)n * n + c] = xc[c];
                            fs[n] = fxc;
                        } else {
                            shrink = true;
                        }
                    }
                } else {
                    // inside contraction
                    for (int c = 0; c < n; ++c) xcc[c] = (1.0 - psi) * xbar[c] + psi * worst[c];
                    double fxcc = 0.0;
                    rc = call(xcc.data(), &fxcc);
                    if (rc == 0) {
                        if (fxcc < fs[n]) {
                            for (int c = 0; c < n; ++c) sim[(size_t)n * n + c] = xcc[c];
                            fs[n] = fxcc;
                        } else {
                            shrink = true;
                        }
                    }
                }
            }
            if (rc == 0 && shrink) {
                for (int j = 1; j < np1 && rc == 0; ++j) {
                    double *v = &sim[(size_t)j * n];
                    for (int c = 0; c < n; ++c) v[c] = sim[c] + sigma * (v[c] - sim[c]);
                    rc = call(v, &fs[j]);
                }
            }
            if (rc < 0) return err;
            if (rc == 0) ++iterations;
        }
        sort_simplex(n, sim, fs);
        if (converged) break;
    }

    for (int c = 0; c < n; ++c) xopt[c] = sim[c];
    if (fopt) {
        double m = fs[0];
        for (int i = 0; i < np1; ++i)
            if (std::isnan(fs[i])) m = fs[i];
            else if (!std::isnan(m) && fs[i] < m) m = fs[i];
        *fopt = m;
    }
    if (nit) *nit = iterations;
    if (nfev) *nfev = fcalls;
    return 0;
}

}  // namespace po
