// po_fmin.cpp -- host downhill-simplex minimiser (po_fmin).
//
// The reference fits its Gaussian with scipy.optimize.fmin (reference
// src/PyPO/FitGauss.py:128, :150). This drives the simplex of po_nm.h, the
// restatement of scipy's Nelder-Mead shared with the device fit, with a host
// objective: given bit-identical values it visits scipy's points in scipy's
// order and returns the same vertex, value and counts.
#include "po_internal.h"
#include "po_nm.h"

namespace po {

int fmin_nm(int n, const double *x0, double xatol, double fatol, long maxiter, long maxfun, const Objective &func,
            double *xopt, double *fopt, long *nit, long *nfev)
{
    if (n < 1 || n > kNMMax) return fail(1, "fmin: between 1 and 8 parameters");
    if (!x0 || !xopt) return fail(1, "fmin: null x0 or xopt");
    NMState s;
    nm_init(s, n, x0, xatol, fatol, maxiter, maxfun);
    while (nm_next(s)) {
        double fx = 0.0;
        if (int rc = func(s.x, &fx)) return rc;
        nm_feed(s, fx);
    }
    for (int c = 0; c < n; ++c) xopt[c] = s.sim[c];
    if (fopt) *fopt = nm_fmin(s);
    if (nit) *nit = s.iterations;
    if (nfev) *nfev = s.fcalls;
    return 0;
}

}  // namespace po
