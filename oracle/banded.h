/*
 * Test infrastructure (oracle only): banded LDL^T direct solve used in place
 * of CXSparse's cs_lusol for the nonlocal fluidity system.
 */
#ifndef ORACLE_BANDED_H
#define ORACLE_BANDED_H

/* Band storage: band[i * (w + 1) + (j - i + w)] holds A(i, j) for
   i - w <= j <= i.  Factorises in place and solves A x = b (b <- x).
   Returns 1 on success, 0 on a zero or non-finite pivot. */
int oracle_band_ldlt_solve(long n, long w, double *band, double *b);

/* Solves A x = b in place (b <- x) for SPD A given in compressed-sparse-column
   form (n columns, colptr[n+1], rowidx/val of colptr[n] entries, duplicates
   already summed).  Returns 1 on success, 0 on a zero or non-finite pivot. */
int oracle_band_ldlt_solve_csc(long n, const long *colptr, const long *rowidx,
                               const double *val, double *b);

#endif
