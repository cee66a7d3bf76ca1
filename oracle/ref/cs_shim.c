/*
 * Test infrastructure (oracle only): the subset of the CXSparse API that the
 * reference's nonlocal materials call, written from CXSparse's published
 * interface (triplet assembly, compression to CSC, duplicate summation, and a
 * direct solve).  CXSparse itself is absent from this machine and its version
 * is unpinned by the reference (cmake/FindCXSparse.cmake searches system
 * paths; CMakeLists.txt:18 requires it without a version).
 *
 * cs_lusol here factorises with the banded LDL^T of oracle/banded.c instead
 * of an LU with fill-reducing ordering: the fluidity matrix assembled by
 * materialsrc/g_nonlocal_mu2.c:455-507 is symmetric positive definite, so both
 * give the same solution up to rounding.  cs_qrsol reuses the same solve.
 */
#include <stdlib.h>
#include <string.h>

#include "suitesparse/cs.h"
#include "../banded.h"

cs *cs_spalloc(long m, long n, long nzmax, long values, long triplet)
{
    cs *A = (cs *)calloc(1, sizeof(cs));
    if (A == NULL) {
        return NULL;
    }
    if (nzmax < 1) {
        nzmax = 1;
    }
    A->m = m;
    A->n = n;
    A->nzmax = nzmax;
    A->nz = triplet ? 0 : -1;
    A->p = (long *)malloc(sizeof(long) * (size_t)(triplet ? nzmax : n + 1));
    A->i = (long *)malloc(sizeof(long) * (size_t)nzmax);
    A->x = values ? (double *)malloc(sizeof(double) * (size_t)nzmax) : NULL;
    if (A->p == NULL || A->i == NULL || (values && A->x == NULL)) {
        return cs_spfree(A);
    }
    return A;
}

static int grow(cs *A, long nzmax)
{
    long *p = (long *)realloc(A->p, sizeof(long) * (size_t)nzmax);
    if (p == NULL) {
        return 0;
    }
    A->p = p;
    long *ii = (long *)realloc(A->i, sizeof(long) * (size_t)nzmax);
    if (ii == NULL) {
        return 0;
    }
    A->i = ii;
    if (A->x != NULL) {
        double *x = (double *)realloc(A->x, sizeof(double) * (size_t)nzmax);
        if (x == NULL) {
            return 0;
        }
        A->x = x;
    }
    A->nzmax = nzmax;
    return 1;
}

long cs_entry(cs *T, long i, long j, double x)
{
    if (T == NULL || T->nz < 0 || i < 0 || j < 0) {
        return 0;
    }
    if (T->nz >= T->nzmax && !grow(T, 2 * T->nzmax)) {
        return 0;
    }
    if (T->x != NULL) {
        T->x[T->nz] = x;
    }
    T->i[T->nz] = i;
    T->p[T->nz] = j;
    T->nz++;
    if (i + 1 > T->m) {
        T->m = i + 1;
    }
    if (j + 1 > T->n) {
        T->n = j + 1;
    }
    return 1;
}

cs *cs_compress(const cs *T)
{
    if (T == NULL || T->nz < 0) {
        return NULL;
    }
    long n = T->n, nz = T->nz;
    cs *C = cs_spalloc(T->m, n, nz, T->x != NULL, 0);
    long *count = (long *)calloc((size_t)n + 1, sizeof(long));
    if (C == NULL || count == NULL) {
        free(count);
        return cs_spfree(C);
    }
    for (long k = 0; k < nz; k++) {
        count[T->p[k]]++;
    }
    long s = 0;
    for (long j = 0; j < n; j++) {
        C->p[j] = s;
        long c = count[j];
        count[j] = s;
        s += c;
    }
    C->p[n] = s;
    for (long k = 0; k < nz; k++) {
        long dst = count[T->p[k]]++;
        C->i[dst] = T->i[k];
        if (C->x != NULL) {
            C->x[dst] = T->x[k];
        }
    }
    free(count);
    return C;
}

long cs_dupl(cs *A)
{
    if (A == NULL || A->nz != -1) {
        return 0;
    }
    long m = A->m, n = A->n;
    long *where = (long *)malloc(sizeof(long) * (size_t)(m > 0 ? m : 1));
    if (where == NULL) {
        return 0;
    }
    for (long r = 0; r < m; r++) {
        where[r] = -1;
    }
    long nz = 0;
    for (long j = 0; j < n; j++) {
        long q = nz;
        for (long k = A->p[j]; k < A->p[j + 1]; k++) {
            long r = A->i[k];
            if (where[r] >= q) {
                if (A->x != NULL) {
                    A->x[where[r]] += A->x[k];
                }
            } else {
                where[r] = nz;
                A->i[nz] = r;
                if (A->x != NULL) {
                    A->x[nz] = A->x[k];
                }
                nz++;
            }
        }
        A->p[j] = q;
    }
    A->p[n] = nz;
    free(where);
    return 1;
}

long cs_lusol(long order, const cs *A, double *b, double tol)
{
    (void)order;
    (void)tol;
    if (A == NULL || A->nz != -1 || b == NULL || A->m != A->n || A->x == NULL) {
        return 0;
    }
    return oracle_band_ldlt_solve_csc(A->n, A->p, A->i, A->x, b);
}

long cs_qrsol(long order, const cs *A, double *b)
{
    return cs_lusol(order, A, b, 0.0);
}

long cs_gaxpy(const cs *A, const double *x, double *y)
{
    if (A == NULL || A->nz != -1 || x == NULL || y == NULL) {
        return 0;
    }
    for (long j = 0; j < A->n; j++) {
        for (long k = A->p[j]; k < A->p[j + 1]; k++) {
            y[A->i[k]] += A->x[k] * x[j];
        }
    }
    return 1;
}

cs *cs_spfree(cs *A)
{
    if (A != NULL) {
        free(A->p);
        free(A->i);
        free(A->x);
        free(A);
    }
    return NULL;
}
