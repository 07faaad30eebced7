// po_nm.h -- the downhill simplex as a state machine (host code).
//
// scipy.optimize.fmin's Nelder-Mead (scipy/optimize/_optimize.py,
// _minimize_neldermead, non-adaptive, no bounds), which the reference's
// Gaussian fit calls (src/PyPO/FitGauss.py:128, :150), restated so that the
// objective is evaluated outside it: nm_next() yields the next point to
// evaluate (false when the minimisation is over) and nm_feed() takes its
// value. The host minimiser (po_fmin.cpp) and the Gaussian fit's driver
// (po_fitgauss_dev.cu, whose objective values come from the GPU, several
// per launch) drive the same code. Given the same values it visits scipy's
// points in scipy's order:
//
//   * coefficients rho = 1, chi = 2, psi = 1/2, sigma = 1/2; initial simplex
//     x0 and x0 with coordinate k scaled by 1.05 (2.5e-4 where it is zero);
//   * before each step: stop when max |x_i - x_0| <= xatol and
//     max |f_0 - f_i| <= fatol, or after maxiter steps / maxfun values
//     (200 n each by default; <= 0 stands for None, as in scipy);
//   * a value requested past maxfun abandons the step it is in (vertices
//     already replaced stay), as scipy's _MaxFuncCallError does;
//   * the simplex is re-sorted after every step, by value, stably, NaN last.
//
// Arithmetic: every product and sum is rounded on its own (the library is
// built with -ffp-contract=off), in numpy's order.
#pragma once

namespace po {

constexpr int kNMMax = 8;   // parameters

struct NMState {
    int n;
    double sim[(kNMMax + 1) * kNMMax], fs[kNMMax + 1];
    double xbar[kNMMax];
    double x[kNMMax];    // the point whose value is wanted
    double xr[kNMMax];   // the step's reflection, kept while its expansion is tried
    double fxr;
    double xatol, fatol;
    long maxiter, maxfun, fcalls, iterations;
    int phase, k;
};

namespace nm {

// kWant*: a trial point is in x, to be requested (or the step abandoned);
// kReflect .. kContractIn, kInit, kShrink: waiting for the value of x.
enum Phase { kInit, kCheck, kReflect, kWantExpand, kExpand, kWantContractOut, kContractOut, kWantContractIn,
             kContractIn, kShrink, kDone };

inline double mul(double a, double b) { return a * b; }
inline double add(double a, double b) { return a + b; }
inline double sub(double a, double b) { return a - b; }
inline bool isnan_(double a) { return a != a; }
inline double inf_() { return __builtin_huge_val(); }

// a sorts before b: smaller, and NaN after every number
inline bool before(double a, double b) { return a < b || (!isnan_(a) && isnan_(b)); }

// stable insertion sort of the vertices by value
inline void sort(NMState &s)
{
    const int n = s.n;
    for (int i = 1; i <= n; ++i) {
        const double f = s.fs[i];
        double row[kNMMax];
        for (int c = 0; c < n; ++c) row[c] = s.sim[i * n + c];
        int j = i - 1;
        while (j >= 0 && before(f, s.fs[j])) {
            s.fs[j + 1] = s.fs[j];
            for (int c = 0; c < n; ++c) s.sim[(j + 1) * n + c] = s.sim[j * n + c];
            --j;
        }
        s.fs[j + 1] = f;
        for (int c = 0; c < n; ++c) s.sim[(j + 1) * n + c] = row[c];
    }
}

// running max of |d| as numpy's max computes it: NaN, once seen, stays
inline double max_abs(double m, double d)
{
    const double a = d < 0 ? -d : d;
    if (isnan_(m)) return m;
    if (isnan_(a)) return a;
    return a > m ? a : m;
}

inline bool converged(const NMState &s)
{
    const int n = s.n;
    double dx = 0.0, df = 0.0;
    for (int i = 1; i <= n; ++i) {
        for (int c = 0; c < n; ++c) dx = max_abs(dx, sub(s.sim[i * n + c], s.sim[c]));
        df = max_abs(df, sub(s.fs[0], s.fs[i]));
    }
    return dx <= s.xatol && df <= s.fatol;
}

// out = a * xbar + b * worst, coordinate by coordinate
inline void trial(NMState &s, double a, double b, double *out)
{
    const double *w = &s.sim[s.n * s.n];
    for (int c = 0; c < s.n; ++c) out[c] = add(mul(a, s.xbar[c]), mul(b, w[c]));
}

inline void end_step(NMState &s)
{
    ++s.iterations;
    sort(s);
    s.phase = kCheck;
}

inline void replace_worst(NMState &s, const double *v, double f)
{
    for (int c = 0; c < s.n; ++c) s.sim[s.n * s.n + c] = v[c];
    s.fs[s.n] = f;
}

}  // namespace nm

inline void nm_init(NMState &s, int n, const double *x0, double xatol, double fatol, long maxiter, long maxfun)
{
    s.n = n;
    const long dflt = 200L * n, inf = 0x7fffffffffffffffL;
    if (maxiter <= 0 && maxfun <= 0) {
        maxiter = dflt;
        maxfun = dflt;
    } else if (maxiter <= 0) {
        maxiter = inf;
    } else if (maxfun <= 0) {
        maxfun = inf;
    }
    s.maxiter = maxiter;
    s.maxfun = maxfun;
    s.xatol = xatol;
    s.fatol = fatol;
    for (int c = 0; c < n; ++c) s.sim[c] = x0[c];
    for (int k = 0; k < n; ++k) {
        double *y = &s.sim[(k + 1) * n];
        for (int c = 0; c < n; ++c) y[c] = x0[c];
        y[k] = y[k] != 0.0 ? nm::mul(1.0 + 0.05, y[k]) : 0.00025;
    }
    for (int i = 0; i <= n; ++i) s.fs[i] = nm::inf_();
    s.fcalls = 0;
    s.iterations = 1;
    s.phase = nm::kInit;
    s.k = 0;
}

// Next point to evaluate, into s.x; false when the minimisation is over.
inline bool nm_next(NMState &s)
{
    using namespace nm;
    const int n = s.n;
    for (;;) {
        switch (s.phase) {
        case kInit:
            if (s.k <= n && s.fcalls < s.maxfun) {
                for (int c = 0; c < n; ++c) s.x[c] = s.sim[s.k * n + c];
                ++s.fcalls;
                return true;
            }
            sort(s);
            s.phase = kCheck;
            break;
        case kCheck:
            if (!(s.fcalls < s.maxfun && s.iterations < s.maxiter) || converged(s)) {
                s.phase = kDone;
                return false;
            }
            for (int c = 0; c < n; ++c) {
                double t = s.sim[c];
                for (int i = 1; i < n; ++i) t = add(t, s.sim[i * n + c]);
                s.xbar[c] = t / n;
            }
            trial(s, 1.0 + 1.0, -1.0, s.x);   // (1 + rho) xbar - rho w
            ++s.fcalls;                       // fcalls < maxfun here
            s.phase = kReflect;
            return true;
        case kWantExpand:
        case kWantContractOut:
        case kWantContractIn:
            if (s.fcalls >= s.maxfun) {       // the step is abandoned
                sort(s);
                s.phase = kCheck;
                break;
            }
            ++s.fcalls;
            s.phase = s.phase == kWantExpand ? kExpand : (s.phase == kWantContractOut ? kContractOut : kContractIn);
            return true;
        case kShrink:
            if (s.k <= n) {
                double *v = &s.sim[s.k * n];
                for (int c = 0; c < n; ++c) v[c] = add(s.sim[c], mul(0.5, sub(v[c], s.sim[c])));
                if (s.fcalls >= s.maxfun) {   // abandoned with this vertex moved
                    sort(s);
                    s.phase = kCheck;
                    break;
                }
                for (int c = 0; c < n; ++c) s.x[c] = v[c];
                ++s.fcalls;
                return true;
            }
            end_step(s);
            break;
        default:
            return false;
        }
    }
}

// Value of the point nm_next returned.
inline void nm_feed(NMState &s, double fx)
{
    using namespace nm;
    const int n = s.n;
    switch (s.phase) {
    case kInit:
        s.fs[s.k++] = fx;
        break;
    case kReflect:
        s.fxr = fx;
        if (fx < s.fs[0]) {
            for (int c = 0; c < n; ++c) s.xr[c] = s.x[c];
            trial(s, 1.0 + 1.0 * 2.0, -(1.0 * 2.0), s.x);    // (1 + rho chi) xbar - rho chi w
            s.phase = kWantExpand;
        } else if (fx < s.fs[n - 1]) {
            replace_worst(s, s.x, fx);
            end_step(s);
        } else if (fx < s.fs[n]) {
            trial(s, 1.0 + 0.5 * 1.0, -(0.5 * 1.0), s.x);    // (1 + psi rho) xbar - psi rho w
            s.phase = kWantContractOut;
        } else {
            trial(s, 1.0 - 0.5, 0.5, s.x);                   // (1 - psi) xbar + psi w
            s.phase = kWantContractIn;
        }
        break;
    case kExpand:
        if (fx < s.fxr) replace_worst(s, s.x, fx);
        else replace_worst(s, s.xr, s.fxr);
        end_step(s);
        break;
    case kContractOut:
        if (fx <= s.fxr) {
            replace_worst(s, s.x, fx);
            end_step(s);
        } else {
            s.phase = kShrink;
            s.k = 1;
        }
        break;
    case kContractIn:
        if (fx < s.fs[n]) {
            replace_worst(s, s.x, fx);
            end_step(s);
        } else {
            s.phase = kShrink;
            s.k = 1;
        }
        break;
    case kShrink:
        s.fs[s.k++] = fx;
        break;
    default:
        break;
    }
}

// Lowest value as numpy's min reports it (NaN if any value is NaN).
inline double nm_fmin(const NMState &s)
{
    double m = s.fs[0];
    for (int i = 0; i <= s.n; ++i) {
        if (nm::isnan_(s.fs[i])) return s.fs[i];
        if (s.fs[i] < m) m = s.fs[i];
    }
    return m;
}

}  // namespace po
