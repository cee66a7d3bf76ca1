/*
 * Test infrastructure (oracle only): a minimal stand-in for the CXSparse
 * header.  CXSparse is not installed here, so the reference's libmpm and its
 * nonlocal material plugins are compiled against this header and linked with
 * oracle/ref/cs_shim.c.
 *
 * Only the calls the reference makes are declared:
 *   libmpm/process.h:16 and libmpm/process_usl.c:22 include this header but
 *   call nothing from it; materialsrc/g_nonlocal_mu2.c:413,497,506,510-519,
 *   566-567 and materialsrc/g_nonlocal.c:436,515,524-533,580-581,596-610 call
 *   cs_spalloc, cs_entry, cs_compress, cs_dupl, cs_lusol, cs_qrsol,
 *   cs_spfree and cs_gaxpy.
 *
 * The matrix record follows CXSparse's published convention: a triplet
 * matrix when nz >= 0 (p holds column indices), compressed-column when
 * nz == -1 (p holds n+1 column pointers).
 */
#ifndef ORACLE_CS_SHIM_H
#define ORACLE_CS_SHIM_H

#include <stddef.h>

typedef struct cs_sparse {
    long nzmax;
    long m;
    long n;
    long *p;
    long *i;
    double *x;
    long nz;
} cs;

cs *cs_spalloc(long m, long n, long nzmax, long values, long triplet);
long cs_entry(cs *T, long i, long j, double x);
cs *cs_compress(const cs *T);
long cs_dupl(cs *A);
long cs_lusol(long order, const cs *A, double *b, double tol);
long cs_qrsol(long order, const cs *A, double *b);
long cs_gaxpy(const cs *A, const double *x, double *y);
cs *cs_spfree(cs *A);

#endif
