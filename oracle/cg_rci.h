/*
 * Reverse-communication conjugate gradient shared by the oracle's MKL-API
 * shim (mkl_shim/mkl_shim.c, which backs the reference's solverCG) and the
 * CPU restatement (lpm_oracle.c), so both run the identical arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY (oracle).  Behaviour follows the published
 * contract of MKL's RCI ISS dcg family as the reference uses it
 * (src/solver.c:188-270):
 *   tmp[0:n]   vector to multiply      tmp[n:2n]  product A*tmp[0:n]
 *   tmp[2n:3n] residual r              tmp[3n:4n] (preconditioned residual, unused)
 *   ipar[0]=n ipar[2]=stage ipar[3]=iterations ipar[4]=max iterations
 *   ipar[7] max-iteration test, ipar[8] residual test, ipar[9] user test,
 *   ipar[10] preconditioner (not supported here)
 *   dpar[0] relative tol, dpar[1] absolute tol, dpar[2]=|r0|^2,
 *   dpar[3]=dpar[0]*dpar[2]+dpar[1], dpar[4]=|r|^2, dpar[5]=previous |r|^2,
 *   dpar[6]=alpha, dpar[7]=beta.
 * Residual stopping test: dpar[4] <= dpar[3] (squared norms).
 * rci_request: 1 = compute tmp[n:2n] = A*tmp[0:n] and call again,
 *              2 = user stopping test, 0 = converged,
 *              -1 = maximum iterations reached, -2 = division by zero,
 *              -10000 = unsupported option.
 * Dot products are plain left-to-right sums so results are reproducible.
 */
#ifndef LPM_CG_RCI_H
#define LPM_CG_RCI_H

#include <string.h>
#include <math.h>

static double lpm_rci_dot(int n, const double *a, const double *b)
{
    double s = 0.0;
    for (int i = 0; i < n; i++)
        s += a[i] * b[i];
    return s;
}

static void lpm_rci_init(int n, int *rci, int *ipar, double *dpar)
{
    memset(ipar, 0, 128 * sizeof(int));
    memset(dpar, 0, 128 * sizeof(double));
    ipar[0] = n;
    ipar[1] = 6;
    ipar[2] = 1;
    ipar[3] = 0;
    ipar[4] = n < 150 ? n : 150;
    ipar[5] = 1;
    ipar[6] = 1;
    ipar[7] = 1;
    ipar[8] = 0;
    ipar[9] = 1;
    ipar[10] = 0;
    dpar[0] = 1.0e-6;
    dpar[1] = 0.0;
    *rci = 0;
}

static void lpm_rci_check(int n, int *rci, const int *ipar, const double *dpar)
{
    if (ipar[0] != n || ipar[4] <= 0 || dpar[0] < 0.0 || dpar[1] < 0.0 || ipar[10] != 0)
        *rci = -1100;
    else
        *rci = 0;
}

/* One reverse-communication step.  x and b are the caller's arrays. */
static void lpm_rci_step(int n, double *x, const double *b, int *rci, int *ipar,
                         double *dpar, double *tmp)
{
    double *p = tmp, *q = tmp + n, *r = tmp + 2 * (size_t)n;
    if (ipar[10] != 0) {
        *rci = -10000;
        return;
    }
    switch (ipar[2]) {
    case 1: /* request A*x0 */
        memcpy(p, x, (size_t)n * sizeof(double));
        ipar[2] = 2;
        *rci = 1;
        return;
    case 2: /* r0 = b - A*x0, p = r0 */
        for (int i = 0; i < n; i++)
            r[i] = b[i] - q[i];
        dpar[2] = lpm_rci_dot(n, r, r);
        dpar[4] = dpar[2];
        dpar[3] = dpar[0] * dpar[2] + dpar[1];
        if (ipar[8] && dpar[4] <= dpar[3]) {
            ipar[2] = 4;
            *rci = 0;
            return;
        }
        memcpy(p, r, (size_t)n * sizeof(double));
        ipar[2] = 3;
        *rci = 1;
        return;
    case 3: { /* q = A*p available */
        double pq = lpm_rci_dot(n, p, q);
        if (pq == 0.0) {
            ipar[2] = 4;
            *rci = -2;
            return;
        }
        double alpha = dpar[4] / pq;
        for (int i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        dpar[6] = alpha;
        dpar[5] = dpar[4];
        dpar[4] = lpm_rci_dot(n, r, r);
        ipar[3] += 1;
        if (ipar[8] && dpar[4] <= dpar[3]) {
            ipar[2] = 4;
            *rci = 0;
            return;
        }
        if (ipar[7] && ipar[3] >= ipar[4]) {
            ipar[2] = 4;
            *rci = -1;
            return;
        }
        double beta = dpar[4] / dpar[5];
        dpar[7] = beta;
        for (int i = 0; i < n; i++)
            p[i] = r[i] + beta * p[i];
        if (ipar[9]) {
            ipar[2] = 5;
            *rci = 2;
            return;
        }
        *rci = 1;
        return;
    }
    case 5: /* resume after a user stopping test */
        ipar[2] = 3;
        *rci = 1;
        return;
    default:
        *rci = 0;
        return;
    }
}

#endif
