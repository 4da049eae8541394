/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's CP-ALS calls four LAPACK/BLAS routines (ssyrk_, spotrf_,
 * spotrs_, sgesv_; src/sptensor/cpd.c:68, src/matrix/matrix_solver.c:51-72).
 * No system LAPACK is installed here, so oracle/_ref/libparti_ref.so resolves
 * those names to this shim, which forwards to function pointers the loader
 * (oracle/__init__.py) takes from scipy's bundled LAPACK.  Integer arguments
 * are 32-bit (f2c `integer` on x86-64 / LP64 LAPACK).
 */
#include <stdio.h>
#include <stdlib.h>

typedef void (*ssyrk_t)(char *, char *, int *, int *, float *, float *, int *, float *, float *, int *);
typedef void (*spotrf_t)(char *, int *, float *, int *, int *);
typedef void (*spotrs_t)(char *, int *, int *, float *, int *, float *, int *, int *);
typedef void (*sgesv_t)(int *, int *, float *, int *, int *, float *, int *, int *);

static ssyrk_t p_ssyrk;
static spotrf_t p_spotrf;
static spotrs_t p_spotrs;
static sgesv_t p_sgesv;

void ref_set_lapack(void *ssyrk, void *spotrf, void *spotrs, void *sgesv) {
    p_ssyrk = (ssyrk_t)ssyrk;
    p_spotrf = (spotrf_t)spotrf;
    p_spotrs = (spotrs_t)spotrs;
    p_sgesv = (sgesv_t)sgesv;
}

static void need(void *p, const char *name) {
    if (!p) {
        fprintf(stderr, "lapack shim: %s called before ref_set_lapack\n", name);
        abort();
    }
}

int ssyrk_(char *uplo, char *trans, int *n, int *k, float *alpha, float *a, int *lda, float *beta, float *c,
           int *ldc) {
    need((void *)p_ssyrk, "ssyrk_");
    p_ssyrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
    return 0;
}

int spotrf_(char *uplo, int *n, float *a, int *lda, int *info) {
    need((void *)p_spotrf, "spotrf_");
    p_spotrf(uplo, n, a, lda, info);
    return 0;
}

int spotrs_(char *uplo, int *n, int *nrhs, float *a, int *lda, float *b, int *ldb, int *info) {
    need((void *)p_spotrs, "spotrs_");
    p_spotrs(uplo, n, nrhs, a, lda, b, ldb, info);
    return 0;
}

int sgesv_(int *n, int *nrhs, float *a, int *lda, int *ipiv, float *b, int *ldb, int *info) {
    need((void *)p_sgesv, "sgesv_");
    p_sgesv(n, nrhs, a, lda, ipiv, b, ldb, info);
    return 0;
}
