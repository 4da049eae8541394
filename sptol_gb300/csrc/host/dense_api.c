/*
 * The reference's dense CP-ALS helpers on caller (host, FP32) matrices, for
 * callers that build their own ALS loop from them:
 *   sptMatrixDotMulSeqTriangle   matrix.c:341-386
 *   sptMatrixSolveNormals        matrix_solver.c:32-83
 *   sptMatrix2Norm, sptMatrixMaxNorm, GetFinalLambda   matrix.c:390-573
 *   sptKruskalTensorFit, sptKruskalTensorFrobeniusNormSquared,
 *   sptSparseKruskalTensorInnerProduct                 ktensor.c:102-257
 * Each call copies its matrices to the device, runs the kernels there and
 * copies the results back.  The normal-equation solve factorises in FP64
 * (Cholesky, LU with partial pivoting when the Hadamard is not positive
 * definite) and applies the inverse in double-float; the norms sum in FP64.
 * Ranks up to 64.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

cudaError_t sptgb_hadamard_upper(const float *const *mats, int nmodes, int mode, int rank, int stride, float *out,
                                 cudaStream_t s);
cudaError_t sptgb_grams_upper_f64(const float *const *mats, int nmodes, int rank, int stride, double *out,
                                  cudaStream_t s);
cudaError_t sptgb_kruskal_normsq(const float *const *ata, int nmodes, int rank, int stride, const float *lambda,
                                 float *tmp, double *out, cudaStream_t s);
cudaError_t sptgb_colmax_scale(float *A, uint32_t nrows, int rank, int stride, float *lambda, float *ws,
                               cudaStream_t s);
cudaError_t sptgb_rowdot(const float *A, const float *B, uint32_t nrows, int rank, int stride, const float *lambda,
                         double *out, double *ws, cudaStream_t s);

#define DMAX 64

/* Device scratch of one call, freed by dfree (the helpers are not on a hot
 * loop of the library; plain allocations keep them independent of the
 * workspace used by the other entry points). */
typedef struct { void *p[12]; int n; } dlist;
static void *dalloc(dlist *l, size_t bytes) {
    void *p = NULL;
    if (l->n >= 12 || cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return NULL;
    l->p[l->n++] = p;
    return p;
}
static void dfree(dlist *l) {
    for (int i = 0; i < l->n; ++i) cudaFree(l->p[i]);
    l->n = 0;
}

#define CK(expr)                                                                 \
    do {                                                                         \
        cudaError_t _e = (expr);                                                 \
        if (_e != cudaSuccess) {                                                 \
            r = sptgb_cuda_fail(_e, module, __FILE__, __LINE__);                 \
            goto out;                                                            \
        }                                                                        \
    } while (0)
#define NEED(ptr)                                                                \
    do {                                                                         \
        if (!(ptr)) {                                                            \
            r = sptgb_cuda_fail(cudaErrorMemoryAllocation, module, __FILE__, __LINE__); \
            goto out;                                                            \
        }                                                                        \
    } while (0)

static int bad_rank(const char *module, sptIndex rank) {
    if (rank >= 1 && rank <= DMAX) return 0;
    spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "rank must be between 1 and 64");
    return 1;
}

/* Uploads the R x stride Grams mats[0..n) into one device block. */
static int upload_grams(dlist *l, sptMatrix **mats, int n, sptIndex rank, sptIndex stride, const float **dptr,
                        cudaStream_t s, const char *module) {
    int r = 0;
    const size_t one = (size_t)rank * stride;
    float *d = (float *)dalloc(l, (size_t)n * one * sizeof(float));
    NEED(d);
    for (int m = 0; m < n; ++m) {
        CK(cudaMemcpyAsync(d + m * one, mats[m]->values, one * sizeof(float), cudaMemcpyHostToDevice, s));
        dptr[m] = d + m * one;
    }
out:
    return r;
}

int sptMatrixDotMulSeqTriangle(sptIndex const mode, sptIndex const nmodes, sptMatrix **mats) {
    const char *module = "Mtx DotMulSeqTriangle";
    const sptIndex rank = mats[0]->ncols, stride = mats[0]->stride;
    if (bad_rank(module, rank) || nmodes < 1 || nmodes > SPTGB_MAX_MODES || mode >= nmodes) return SPTERR_VALUE_ERROR;
    for (sptIndex m = 1; m <= nmodes; ++m)
        if (mats[m]->ncols != rank || mats[m]->nrows != mats[0]->nrows || mats[m]->stride != stride) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "matrices of different shapes");
            return SPTERR_SHAPE_MISMATCH;
        }
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();
    int r = 0;
    dlist l = {{0}, 0};
    const float *dm[SPTGB_MAX_MODES];
    sptgb_lock();
    float *dout = (float *)dalloc(&l, (size_t)rank * stride * sizeof(float));
    NEED(dout);
    if ((r = upload_grams(&l, mats, (int)nmodes, rank, stride, dm, s, module))) goto out;
    /* the output's other entries (padding) are the caller's */
    CK(cudaMemcpyAsync(dout, mats[nmodes]->values, (size_t)rank * stride * sizeof(float), cudaMemcpyHostToDevice, s));
    CK(sptgb_hadamard_upper(dm, (int)nmodes, (int)mode, (int)rank, (int)stride, dout, s));
    CK(cudaMemcpyAsync(mats[nmodes]->values, dout, (size_t)rank * stride * sizeof(float), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
out:
    dfree(&l);
    sptgb_unlock();
    return r;
}

/* X G = rhs for the rows of rhs (matrix_solver.c:32-83 solves the same
 * system through the column-major view); aTa[nmodes] receives the Hadamard
 * of the other Grams as sptMatrixDotMulSeqTriangle leaves it. */
int sptMatrixSolveNormals(sptIndex const mode, sptIndex const nmodes, sptMatrix **aTa, sptMatrix *rhs) {
    const char *module = "Mtx SolveNormals";
    const sptIndex rank = aTa[0]->ncols, stride = aTa[0]->stride;
    if (bad_rank(module, rank)) return SPTERR_VALUE_ERROR;
    if (rhs->ncols != rank || rhs->stride != stride) {
        spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "rhs and Gram shapes differ");
        return SPTERR_SHAPE_MISMATCH;
    }
    int r = sptMatrixDotMulSeqTriangle(mode, nmodes, aTa);
    if (r) return r;
    const cudaStream_t s = sptgb_stream();
    const uint32_t nrows = rhs->nrows;
    dlist l = {{0}, 0};
    const float *dm[SPTGB_MAX_MODES];
    const double *g64[SPTGB_MAX_MODES];
    sptgb_lock();
    {
        if ((r = upload_grams(&l, aTa, (int)nmodes, rank, stride, dm, s, module))) goto out;
        double *d64 = (double *)dalloc(&l, (size_t)nmodes * rank * rank * sizeof(double));
        double *Hinv = (double *)dalloc(&l, (size_t)2 * rank * rank * sizeof(double));
        int *status = (int *)dalloc(&l, 16);
        double *ws = (double *)dalloc(&l, sptgb_dense_ws_bytes((int)rank, SPTGB_NPART));
        float *dM = (float *)dalloc(&l, (size_t)nrows * stride * sizeof(float));
        float *dX = (float *)dalloc(&l, (size_t)nrows * stride * sizeof(float));
        NEED(d64);
        NEED(Hinv);
        NEED(status);
        NEED(ws);
        NEED(dM);
        NEED(dX);
        CK(sptgb_grams_upper_f64(dm, (int)nmodes, (int)rank, (int)stride, d64, s));
        for (sptIndex m = 0; m < nmodes; ++m) g64[m] = d64 + (size_t)m * rank * rank;
        CK(sptgb_solve_prepare(g64, (int)nmodes, (int)mode, (int)rank, Hinv, status, s));
        if (nrows) {
            CK(cudaMemcpyAsync(dM, rhs->values, (size_t)nrows * stride * sizeof(float), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dX, dM, (size_t)nrows * stride * sizeof(float), cudaMemcpyDeviceToDevice, s));
            CK(sptgb_solve_rows(dM, dX, nrows, (int)rank, (int)stride, Hinv, status, ws, s));
            CK(cudaMemcpyAsync(rhs->values, dX, (size_t)nrows * stride * sizeof(float), cudaMemcpyDeviceToHost, s));
        }
        CK(cudaStreamSynchronize(s));
    }
out:
    dfree(&l);
    sptgb_unlock();
    return r;
}

/* use_max: sptMatrixMaxNorm, else sptMatrix2Norm.  lambda_io: multiply the
 * column norms into lambda (GetFinalLambda) instead of storing them. */
static int col_norm(sptMatrix *A, sptValue *lambda, int use_max, int lambda_io, const char *module) {
    const sptIndex rank = A->ncols, stride = A->stride;
    if (bad_rank(module, rank)) return SPTERR_VALUE_ERROR;
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();
    const uint32_t nrows = A->nrows;
    int r = 0;
    dlist l = {{0}, 0};
    sptgb_lock();
    {
        float *dA = (float *)dalloc(&l, (size_t)nrows * stride * sizeof(float));
        float *dl = (float *)dalloc(&l, DMAX * sizeof(float));
        double *ws = (double *)dalloc(&l, sptgb_dense_ws_bytes((int)rank, SPTGB_NPART) + SPTGB_NPART * DMAX * 4);
        NEED(dA);
        NEED(dl);
        NEED(ws);
        if (nrows)
            CK(cudaMemcpyAsync(dA, A->values, (size_t)nrows * stride * sizeof(float), cudaMemcpyHostToDevice, s));
        if (use_max) {
            CK(sptgb_colmax_scale(dA, nrows, (int)rank, (int)stride, dl, (float *)ws, s));
        } else {
            float ones[DMAX];
            for (int j = 0; j < DMAX; ++j) ones[j] = 1.f;
            if (lambda_io) memcpy(ones, lambda, rank * sizeof(float));
            CK(cudaMemcpyAsync(dl, ones, rank * sizeof(float), cudaMemcpyHostToDevice, s));
            CK(sptgb_colnorm_scale(dA, nrows, (int)rank, (int)stride, dl, ws, s));
        }
        if (nrows)
            CK(cudaMemcpyAsync(A->values, dA, (size_t)nrows * stride * sizeof(float), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(lambda, dl, rank * sizeof(float), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
out:
    dfree(&l);
    sptgb_unlock();
    return r;
}

int sptMatrix2Norm(sptMatrix *const A, sptValue *const lambda) { return col_norm(A, lambda, 0, 0, "Mtx 2Norm"); }

int sptMatrixMaxNorm(sptMatrix *const A, sptValue *const lambda) { return col_norm(A, lambda, 1, 0, "Mtx MaxNorm"); }

/* matrix.c:557-573: lambda *= the column 2-norms of every factor, which are
 * normalised by them. */
void GetFinalLambda(sptIndex const rank, sptIndex const nmodes, sptMatrix **mats, sptValue *const lambda) {
    for (sptIndex m = 0; m < nmodes; ++m) {
        if (mats[m]->ncols != rank) {
            spt_ComplainError("GetFinalLambda", SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "rank differs");
            return;
        }
        if (col_norm(mats[m], lambda, 0, 1, "GetFinalLambda")) return;
    }
}

double sptKruskalTensorFrobeniusNormSquared(sptIndex const nmodes, sptValue const *const lambda, sptMatrix **ata) {
    const char *module = "Kruskal NormSquared";
    const sptIndex rank = ata[0]->ncols, stride = ata[0]->stride;
    if (bad_rank(module, rank) || nmodes < 1 || nmodes > SPTGB_MAX_MODES) return NAN;
    if (sptgb_ctx()) return NAN;
    const cudaStream_t s = sptgb_stream();
    int r = 0;
    double result = NAN;
    dlist l = {{0}, 0};
    const float *dm[SPTGB_MAX_MODES];
    sptgb_lock();
    {
        float *tmp = (float *)dalloc(&l, (size_t)rank * stride * sizeof(float));
        float *dl = (float *)dalloc(&l, DMAX * sizeof(float));
        double *dout = (double *)dalloc(&l, sizeof(double));
        NEED(tmp);
        NEED(dl);
        NEED(dout);
        if ((r = upload_grams(&l, ata, (int)nmodes, rank, stride, dm, s, module))) goto out;
        CK(cudaMemcpyAsync(dl, lambda, rank * sizeof(float), cudaMemcpyHostToDevice, s));
        CK(sptgb_kruskal_normsq(dm, (int)nmodes, (int)rank, (int)stride, dl, tmp, dout, s));
        CK(cudaMemcpyAsync(ata[nmodes]->values, tmp, (size_t)rank * stride * sizeof(float), cudaMemcpyDeviceToHost,
                           s));
        CK(cudaMemcpyAsync(&result, dout, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
out:
    dfree(&l);
    sptgb_unlock();
    return r ? NAN : result;
}

/* <X, K> from the last mode's MTTKRP output mats[nmodes] and the last factor
 * mats[nmodes-1]. */
double sptSparseKruskalTensorInnerProduct(sptIndex const nmodes, sptValue const *const lambda, sptMatrix **mats) {
    const char *module = "Kruskal InnerProduct";
    const sptIndex rank = mats[0]->ncols, stride = mats[0]->stride;
    if (bad_rank(module, rank) || nmodes < 1) return NAN;
    if (sptgb_ctx()) return NAN;
    const cudaStream_t s = sptgb_stream();
    const uint32_t I = mats[nmodes - 1]->nrows;
    int r = 0;
    double result = NAN;
    dlist l = {{0}, 0};
    sptgb_lock();
    {
        float *dA = (float *)dalloc(&l, (size_t)I * stride * sizeof(float));
        float *dB = (float *)dalloc(&l, (size_t)I * stride * sizeof(float));
        float *dl = (float *)dalloc(&l, DMAX * sizeof(float));
        double *ws = (double *)dalloc(&l, (size_t)SPTGB_NPART * DMAX * sizeof(double) + 64);
        NEED(dA);
        NEED(dB);
        NEED(dl);
        NEED(ws);
        if (I) {
            CK(cudaMemcpyAsync(dA, mats[nmodes - 1]->values, (size_t)I * stride * sizeof(float),
                               cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dB, mats[nmodes]->values, (size_t)I * stride * sizeof(float), cudaMemcpyHostToDevice,
                               s));
        }
        CK(cudaMemcpyAsync(dl, lambda, rank * sizeof(float), cudaMemcpyHostToDevice, s));
        double *dout = ws + SPTGB_NPART * DMAX;
        CK(sptgb_rowdot(dA, dB, I, (int)rank, (int)stride, dl, dout, ws, s));
        CK(cudaMemcpyAsync(&result, dout, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
out:
    dfree(&l);
    sptgb_unlock();
    return r ? NAN : result;
}

/* ktensor.c:102-120: fit = 1 - r / ||X||, r = sqrt(res) when res > 0. */
double sptKruskalTensorFit(sptSparseTensor const *const spten, sptValue const *const lambda, sptMatrix **mats,
                           sptMatrix **ata) {
    const sptIndex nmodes = spten->nmodes;
    const double normsq = SparseTensorFrobeniusNormSquared(spten);
    const double norm_mats = sptKruskalTensorFrobeniusNormSquared(nmodes, lambda, ata);
    const double inner = sptSparseKruskalTensorInnerProduct(nmodes, lambda, mats);
    double residual = normsq + norm_mats - 2 * inner;
    if (residual > 0.0) residual = sqrt(residual);
    return 1 - residual / sqrt(normsq);
}

/* ---------------------------------------------------- rank-matrix forms -- */
/* The sptRankMatrix forms of the helpers above (rankmatrix.c:137-378,
 * rankmatrix_solver.c:32-84, rankktensor.c:101-257) compute the same thing
 * on matrices whose column count and stride are 8-bit; each runs the
 * sptMatrix form on views of the caller's matrices. */
static void rank_views(sptRankMatrix **in, sptIndex n, sptMatrix *view, sptMatrix **pv) {
    for (sptIndex i = 0; i < n; ++i) {
        view[i].nrows = in[i]->nrows;
        view[i].ncols = in[i]->ncols;
        view[i].cap = in[i]->cap;
        view[i].stride = in[i]->stride;
        view[i].values = in[i]->values;
        pv[i] = &view[i];
    }
}

static int bad_order(const char *module, sptIndex nmodes) {
    if (nmodes >= 1 && nmodes <= SPTGB_MAX_MODES) return 0;
    spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order");
    return 1;
}

int sptRankMatrixDotMulSeqTriangle(sptIndex const mode, sptIndex const nmodes, sptRankMatrix **mats) {
    if (bad_order("RankMtx DotMulSeqTriangle", nmodes)) return SPTERR_VALUE_ERROR;
    sptMatrix v[SPTGB_MAX_MODES + 1], *pv[SPTGB_MAX_MODES + 1];
    rank_views(mats, nmodes + 1, v, pv);
    return sptMatrixDotMulSeqTriangle(mode, nmodes, pv);
}

int sptRankMatrixSolveNormals(sptIndex const mode, sptIndex const nmodes, sptRankMatrix **aTa, sptRankMatrix *rhs) {
    if (bad_order("RankMtx SolveNormals", nmodes)) return SPTERR_VALUE_ERROR;
    sptMatrix v[SPTGB_MAX_MODES + 2], *pv[SPTGB_MAX_MODES + 2];
    rank_views(aTa, nmodes + 1, v, pv);
    rank_views(&rhs, 1, v + nmodes + 1, pv + nmodes + 1);
    return sptMatrixSolveNormals(mode, nmodes, pv, pv[nmodes + 1]);
}

int sptRankMatrix2Norm(sptRankMatrix *const A, sptValue *const lambda) {
    sptMatrix v, *pv;
    sptRankMatrix *a = A;
    rank_views(&a, 1, &v, &pv);
    return col_norm(pv, lambda, 0, 0, "RankMtx 2Norm");
}

int sptRankMatrixMaxNorm(sptRankMatrix *const A, sptValue *const lambda) {
    sptMatrix v, *pv;
    sptRankMatrix *a = A;
    rank_views(&a, 1, &v, &pv);
    return col_norm(pv, lambda, 1, 0, "RankMtx MaxNorm");
}

void GetRankFinalLambda(sptElementIndex const rank, sptIndex const nmodes, sptRankMatrix **mats,
                        sptValue *const lambda) {
    if (bad_order("GetRankFinalLambda", nmodes)) return;
    sptMatrix v[SPTGB_MAX_MODES + 1], *pv[SPTGB_MAX_MODES + 1];
    rank_views(mats, nmodes, v, pv);
    GetFinalLambda(rank, nmodes, pv, lambda);
}

double sptKruskalTensorFrobeniusNormSquaredRank(sptIndex const nmodes, sptValue const *const lambda,
                                                sptRankMatrix **ata) {
    if (bad_order("Kruskal NormSquared", nmodes)) return NAN;
    sptMatrix v[SPTGB_MAX_MODES + 1], *pv[SPTGB_MAX_MODES + 1];
    rank_views(ata, nmodes + 1, v, pv);
    return sptKruskalTensorFrobeniusNormSquared(nmodes, lambda, pv);
}

double sptSparseKruskalTensorInnerProductRank(sptIndex const nmodes, sptValue const *const lambda,
                                              sptRankMatrix **mats) {
    if (bad_order("Kruskal InnerProduct", nmodes)) return NAN;
    sptMatrix v[SPTGB_MAX_MODES + 1], *pv[SPTGB_MAX_MODES + 1];
    rank_views(mats, nmodes + 1, v, pv);
    return sptSparseKruskalTensorInnerProduct(nmodes, lambda, pv);
}

/* rankktensor.c:101-119, the fit of sptKruskalTensorFit over a HiCOO tensor. */
double sptKruskalTensorFitHiCOO(sptSparseTensorHiCOO const *const hitsr, sptValue const *const lambda,
                                sptRankMatrix **mats, sptRankMatrix **ata) {
    const sptIndex nmodes = hitsr->nmodes;
    const double normsq = sptSparseTensorFrobeniusNormSquaredHiCOO(hitsr);
    const double norm_mats = sptKruskalTensorFrobeniusNormSquaredRank(nmodes, lambda, ata);
    const double inner = sptSparseKruskalTensorInnerProductRank(nmodes, lambda, mats);
    double residual = normsq + norm_mats - 2 * inner;
    if (residual > 0.0) residual = sqrt(residual);
    return 1 - residual / sqrt(normsq);
}
