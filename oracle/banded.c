/*
 * Test infrastructure (oracle only; never linked into the product library).
 *
 * Direct FP64 solve of a symmetric positive definite sparse system by an
 * LDL^T factorisation in band storage.  The reference factorises the nonlocal
 * fluidity matrix with CXSparse's LU (materialsrc/g_nonlocal_mu2.c:510-519,
 * cs_lusol(order=1, tol=1e-12)); CXSparse is not available here, and any exact
 * direct method returns the same solution up to rounding (a few ulps times the
 * condition number), so the oracle uses this band solver instead.
 *
 * The fluidity matrix couples only nodes that share an element, and the
 * reference numbers its unknowns in ascending node order
 * (g_nonlocal_mu2.c:365-381), so the lower bandwidth is at most the node row
 * length plus one.  Cost is O(n * w^2) for n unknowns and bandwidth w.
 */
#include <stdlib.h>
#include <math.h>

#include "banded.h"

/* band[i * (w + 1) + (j - i + w)] holds row i, column j, for i - w <= j <= i. */
#define BAND(i, j) band[(size_t)(i) * (size_t)(w + 1) + (size_t)((j) - (i) + w)]

int oracle_band_ldlt_solve(long n, long w, double *band, double *b)
{
    double *diag = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (diag == NULL || n <= 0) {
        free(diag);
        return 0;
    }

    /* Row-oriented LDL^T: L is unit lower triangular, stored over A. */
    int ok = 1;
    for (long i = 0; i < n && ok; i++) {
        long j0 = (i - w > 0) ? i - w : 0;
        for (long j = j0; j < i; j++) {
            double s = BAND(i, j);
            long k0 = (j - w > j0) ? j - w : j0;
            for (long k = k0; k < j; k++) {
                s -= BAND(i, k) * diag[k] * BAND(j, k);
            }
            BAND(i, j) = s / diag[j];
        }
        double d = BAND(i, i);
        for (long k = j0; k < i; k++) {
            double lik = BAND(i, k);
            d -= lik * lik * diag[k];
        }
        if (!(d != 0.0) || !isfinite(d)) {
            ok = 0;
            break;
        }
        diag[i] = d;
    }

    if (ok) {
        /* L y = b */
        for (long i = 0; i < n; i++) {
            long j0 = (i - w > 0) ? i - w : 0;
            double s = b[i];
            for (long j = j0; j < i; j++) {
                s -= BAND(i, j) * b[j];
            }
            b[i] = s;
        }
        /* D z = y */
        for (long i = 0; i < n; i++) {
            b[i] /= diag[i];
        }
        /* L^T x = z */
        for (long i = n - 1; i >= 0; i--) {
            long i1 = (i + w < n - 1) ? i + w : n - 1;
            double s = b[i];
            for (long r = i + 1; r <= i1; r++) {
                s -= BAND(r, i) * b[r];
            }
            b[i] = s;
        }
    }

    free(diag);
    return ok;
}

int oracle_band_ldlt_solve_csc(long n, const long *colptr, const long *rowidx,
                               const double *val, double *b)
{
    long w = 0;
    if (n <= 0) {
        return 0;
    }
    for (long j = 0; j < n; j++) {
        for (long k = colptr[j]; k < colptr[j + 1]; k++) {
            long i = rowidx[k];
            if (i > j && i - j > w) {
                w = i - j;
            }
        }
    }
    double *band = (double *)calloc((size_t)n * (size_t)(w + 1), sizeof(double));
    if (band == NULL) {
        return 0;
    }
    /* Scatter the lower triangle (row >= column). */
    for (long j = 0; j < n; j++) {
        for (long k = colptr[j]; k < colptr[j + 1]; k++) {
            long i = rowidx[k];
            if (i >= j) {
                BAND(i, j) += val[k];
            }
        }
    }
    int ok = oracle_band_ldlt_solve(n, w, band, b);
    free(band);
    return ok;
}
