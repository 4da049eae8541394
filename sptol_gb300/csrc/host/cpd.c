/*
 * CP-ALS on the GPU behind the reference's entry points
 * (src/sptensor/cpd.c:32-195; include/includes/cpds.h:26-45).
 *
 * One call uploads the tensor once, builds its per-mode segmented copies (COO)
 * or output-window schedules (HiCOO, sptCpdAlsHiCOO, hicoo/cpd.c:34-195) and
 * keeps factors, Gram matrices and the MTTKRP output in HBM for the whole
 * run.  Per iteration and mode, in the reference's order (cpd.c:76-125):
 *   MTTKRP (FP32) -> H = Hadamard of the other Grams and its inverse (FP64,
 *   Cholesky or LU fallback) -> rows solved in double-float -> 2-norm (first
 *   iteration) or max-norm column normalisation -> new Gram (double-float,
 *   fused with the solve, stored FP64).
 * After the modes the fit is computed on the device with full symmetric
 * Grams; only that scalar returns to the host each iteration (the tolerance
 * test and the progress line need it).  GetFinalLambda (matrix.c:557-573)
 * runs at the end, then factors and lambda are copied back.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

cudaError_t sptgb_normalize(float *X, uint32_t nrows, int rank, int stride, double *gram, int use_2norm,
                            float *lambda_f32, const double *ws, cudaStream_t s);

typedef struct {
    float *fac[SPTGB_MAX_MODES];
    float *M;
    float *lambda;
    double *gram[SPTGB_MAX_MODES];
    double *S;
    double *ws;
    double *normX2;
    double *fits;
    int *status;
} cpd_buffers;

static void free_buffers(cpd_buffers *b) {
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) {
        if (b->fac[m]) cudaFree(b->fac[m]);
        if (b->gram[m]) cudaFree(b->gram[m]);
    }
    if (b->M) cudaFree(b->M);
    if (b->lambda) cudaFree(b->lambda);
    if (b->S) cudaFree(b->S);
    if (b->ws) cudaFree(b->ws);
    if (b->normX2) cudaFree(b->normX2);
    if (b->fits) cudaFree(b->fits);
    if (b->status) cudaFree(b->status);
    memset(b, 0, sizeof *b);
}

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + t.tv_nsec * 1e-9;
}

#define CUDA_OR_FAIL(expr)                                                  \
    do {                                                                    \
        cudaError_t _c = (expr);                                            \
        if (_c != cudaSuccess) {                                            \
            r = sptgb_cuda_fail(_c, "GPU CPD-ALS", __FILE__, __LINE__);     \
            goto done;                                                      \
        }                                                                   \
    } while (0)

/* The MTTKRP of one mode into M (device), factors by mode. */
typedef int (*cpd_mttkrp_fn)(void *ctx, sptIndex mode, const sptIndex *order, const float *const *fac, sptIndex rank,
                             sptIndex stride, float *M, cudaStream_t s);

/* The CP-ALS loop for any MTTKRP source: hfac[m] = host factor values
 * (ndims[m] x stride, updated in place), vals / nnz = the tensor's values on
 * the device (for ||X||^2). */
static int cpd_run(int N, const sptIndex *ndims, const float *vals, uint64_t nnz, cpd_mttkrp_fn mttkrp, void *ctx,
                   sptIndex rank, int stride, float *const *hfac, sptIndex niters, double tol, sptValue *lambda,
                   double *fits, sptIndex *iters_done, cudaStream_t s) {
    int r = 0;
    cpd_buffers b;
    memset(&b, 0, sizeof b);
    sptIndex done_iters = 0;
    double *hfits = (double *)calloc(niters ? niters : 1, sizeof(double));
    int *hstatus = (int *)calloc((size_t)N, sizeof(int));

    sptIndex max_dim = 0;
    for (int m = 0; m < N; ++m) {
        const size_t bytes = (size_t)ndims[m] * stride * sizeof(float);
        CUDA_OR_FAIL(cudaMalloc((void **)&b.fac[m], bytes ? bytes : 16));
        if (bytes) CUDA_OR_FAIL(cudaMemcpyAsync(b.fac[m], hfac[m], bytes, cudaMemcpyHostToDevice, s));
        CUDA_OR_FAIL(cudaMalloc((void **)&b.gram[m], (size_t)rank * rank * sizeof(double)));
        if (ndims[m] > max_dim) max_dim = ndims[m];
    }
    CUDA_OR_FAIL(cudaMalloc((void **)&b.M, (size_t)(max_dim ? max_dim : 1) * stride * sizeof(float)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.lambda, (size_t)rank * sizeof(float)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.S, (size_t)rank * rank * sizeof(double)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.ws, sptgb_dense_ws_bytes((int)rank, 0)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.normX2, sizeof(double)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.fits, (size_t)(niters ? niters : 1) * sizeof(double)));
    CUDA_OR_FAIL(cudaMalloc((void **)&b.status, (size_t)N * sizeof(int)));
    CUDA_OR_FAIL(cudaMemsetAsync(b.status, 0, (size_t)N * sizeof(int), s));

    CUDA_OR_FAIL(sptgb_sumsq(vals, nnz, b.normX2, b.ws, s));
    for (int m = 0; m < N; ++m)
        CUDA_OR_FAIL(sptgb_gram(b.fac[m], ndims[m], (int)rank, stride, b.gram[m], b.ws, s));

    double t_prev = sptgb_wall();
    SPTGB_TRACE_POINT("cpd setup", s, t_prev);
    double oldfit = 0.0;
    const double *gptr[SPTGB_MAX_MODES];
    for (int m = 0; m < N; ++m) gptr[m] = b.gram[m];
    for (sptIndex it = 0; it < niters; ++it) {
        const double t0 = now_s();
        for (int m = 0; m < N; ++m) {
            sptIndex order[SPTGB_MAX_MODES];
            order[0] = (sptIndex)m;
            for (int i = 1; i < N; ++i) order[i] = (sptIndex)((m + i) % N);
            r = mttkrp(ctx, (sptIndex)m, order, (const float *const *)b.fac, rank, (sptIndex)stride, b.M, s);
            if (r) goto done;
            CUDA_OR_FAIL(sptgb_solve_prepare(gptr, N, m, (int)rank, b.S, b.status + m, s));
            CUDA_OR_FAIL(sptgb_solve_rows(b.M, b.fac[m], ndims[m], (int)rank, stride, b.S, b.status + m, b.ws, s));
            CUDA_OR_FAIL(sptgb_normalize(b.fac[m], ndims[m], (int)rank, stride, b.gram[m], it == 0 ? 1 : 0,
                                         b.lambda, b.ws, s));
        }
        CUDA_OR_FAIL(sptgb_fit(b.fac[N - 1], b.M, ndims[N - 1], (int)rank, stride, b.lambda, gptr, N, b.normX2,
                               b.fits + it, b.ws, s));
        double fit = 0.0;
        CUDA_OR_FAIL(cudaMemcpyAsync(&fit, b.fits + it, sizeof(double), cudaMemcpyDeviceToHost, s));
        CUDA_OR_FAIL(cudaMemcpyAsync(hstatus, b.status, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, s));
        CUDA_OR_FAIL(cudaStreamSynchronize(s));
        hfits[it] = fit;
        done_iters = it + 1;
        if (!sptgb_quiet()) {
            for (int m = 0; m < N; ++m)
                if (hstatus[m] & 0xff) printf("Gram matrix is not SPD. Trying `gesv`.\n");
            printf("  its = %u ( %.3lf s ) fit = %0.5f  delta = %+0.4e\n", it + 1, now_s() - t0, fit, fit - oldfit);
        }
        if (it > 0 && fabs(fit - oldfit) < tol) break;
        oldfit = fit;
    }

    SPTGB_TRACE_POINT("cpd iters", s, t_prev);
    /* GetFinalLambda: lambda *= column 2-norms of every factor, factors
     * normalised by them (matrix.c:557-573). */
    for (int m = 0; m < N; ++m)
        CUDA_OR_FAIL(sptgb_colnorm_scale(b.fac[m], ndims[m], (int)rank, stride, b.lambda, b.ws, s));
    for (int m = 0; m < N; ++m) {
        const size_t bytes = (size_t)ndims[m] * stride * sizeof(float);
        if (bytes) CUDA_OR_FAIL(cudaMemcpyAsync(hfac[m], b.fac[m], bytes, cudaMemcpyDeviceToHost, s));
    }
    CUDA_OR_FAIL(cudaMemcpyAsync(lambda, b.lambda, (size_t)rank * sizeof(float), cudaMemcpyDeviceToHost, s));
    CUDA_OR_FAIL(cudaStreamSynchronize(s));
    if (fits)
        for (sptIndex it = 0; it < niters; ++it) fits[it] = it < done_iters ? hfits[it] : NAN;
    if (iters_done) *iters_done = done_iters;
    SPTGB_TRACE_POINT("cpd d2h", s, t_prev);

done:
    free_buffers(&b);
    free(hfits);
    free(hstatus);
    return r;
}

static int coo_mttkrp(void *ctx, sptIndex mode, const sptIndex *order, const float *const *fac, sptIndex rank,
                      sptIndex stride, float *M, cudaStream_t s) {
    return sptgbCooMTTKRP((sptgbCoo *)ctx, mode, order, fac, rank, stride, M, (void *)s);
}

static int hicoo_mttkrp_dev(void *ctx, sptIndex mode, const sptIndex *order, const float *const *fac, sptIndex rank,
                            sptIndex stride, float *M, cudaStream_t s) {
    return sptgbHicooMTTKRP((sptgbHicoo *)ctx, mode, order, fac, rank, stride, M, (void *)s);
}

int sptgbCpdAls(sptSparseTensor const *X, sptIndex rank, sptIndex niters, double tol, sptMatrix **mats,
                sptValue *lambda, double *fits, sptIndex *iters_done) {
    const char *module = "GPU CPD-ALS";
    const int N = (int)X->nmodes;
    if (N < 2 || N > SPTGB_MAX_MODES || rank < 1 || rank > 64) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "order in [2,8] and rank in [1,64] required");
        return SPTERR_VALUE_ERROR;
    }
    const int stride = (int)mats[0]->stride;
    float *hfac[SPTGB_MAX_MODES];
    for (int m = 0; m < N; ++m) {
        if (mats[m]->nrows != X->ndims[m] || mats[m]->ncols != rank || (int)mats[m]->stride != stride) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "factor matrix shape");
            return SPTERR_SHAPE_MISMATCH;
        }
        hfac[m] = mats[m]->values;
    }
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();
    double t_prev = sptgb_wall();
    sptgbCoo *t = NULL;
    int r = sptgbCooCreate(&t, X, (void *)s);
    SPTGB_TRACE_POINT("cpd upload", s, t_prev);
    for (int m = 0; m < N && !r; ++m) r = sptgbCooPrepareMode(t, (sptIndex)m, (void *)s);
    SPTGB_TRACE_POINT("cpd sorts", s, t_prev);
    if (!r) r = cpd_run(N, X->ndims, t->vals, t->nnz, coo_mttkrp, t, rank, stride, hfac, niters, tol, lambda, fits,
                        iters_done, s);
    SPTGB_TRACE_POINT("cpd loop", s, t_prev);
    if (t) sptgbCooFree(t);
    SPTGB_TRACE_POINT("cpd free", s, t_prev);
    return r;
}

int sptgbCpdAlsHiCOO(sptSparseTensorHiCOO const *h, sptIndex rank, sptIndex niters, double tol, sptRankMatrix **mats,
                     sptValue *lambda, double *fits, sptIndex *iters_done) {
    const char *module = "GPU HiCOO CPD-ALS";
    const int N = (int)h->nmodes;
    if (N < 2 || N > SPTGB_MAX_MODES || rank < 1 || rank > 64) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "order in [2,8] and rank in [1,64] required");
        return SPTERR_VALUE_ERROR;
    }
    const int stride = (int)mats[0]->stride;
    float *hfac[SPTGB_MAX_MODES];
    for (int m = 0; m < N; ++m) {
        if (mats[m]->nrows != h->ndims[m] || mats[m]->ncols != rank || (int)mats[m]->stride != stride) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "factor matrix shape");
            return SPTERR_SHAPE_MISMATCH;
        }
        hfac[m] = mats[m]->values;
    }
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();
    sptgbHicoo *t = NULL;
    int r = sptgbHicooCreate(&t, h, (void *)s);
    for (int m = 0; m < N && !r; ++m) r = sptgbHicooPrepareMode(t, (sptIndex)m, (void *)s);
    if (!r) r = cpd_run(N, h->ndims, t->vals, t->nnz, hicoo_mttkrp_dev, t, rank, stride, hfac, niters, tol, lambda,
                        fits, iters_done, s);
    if (t) sptgbHicooFree(t);
    return r;
}

double CpdAlsStep(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters, double const tol,
                  sptMatrix **mats, sptValue *const lambda) {
    double *fits = (double *)calloc(niters ? niters : 1, sizeof(double));
    sptIndex done = 0;
    double fit = 0.0;
    if (sptgbCpdAls(spten, rank, niters, tol, mats, lambda, fits, &done) == 0 && done > 0) fit = fits[done - 1];
    free(fits);
    return fit;
}

/* cpd.c:148-195: random factors (seeded here, see sptgbSetSeed), a scratch
 * mats[nmodes] of max_dim rows, CpdAlsStep, factors handed to the Kruskal
 * tensor.  The factor structs stay allocated (the reference frees them while
 * ktensor->factors still points at them); factors[nmodes] is NULL. */
int sptCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters, double const tol,
              sptKruskalTensor *ktensor) {
    const sptIndex N = spten->nmodes;
    sptIndex max_dim = 0;
    for (sptIndex m = 0; m < N; ++m)
        if (spten->ndims[m] > max_dim) max_dim = spten->ndims[m];
    sptMatrix **mats = (sptMatrix **)calloc(N + 1, sizeof(*mats));
    if (!mats) return SPTERR_OS_ERROR;
    for (sptIndex m = 0; m < N; ++m) {
        mats[m] = (sptMatrix *)malloc(sizeof(sptMatrix));
        int e = sptNewMatrix(mats[m], spten->ndims[m], rank);
        if (e) return e;
        sptRandomizeMatrix(mats[m], spten->ndims[m], rank);
    }
    double *fits = (double *)calloc(niters ? niters : 1, sizeof(double));
    sptIndex done = 0;
    const int r = sptgbCpdAls(spten, rank, niters, tol, mats, ktensor->lambda, fits, &done);
    ktensor->fit = done > 0 ? fits[done - 1] : 0.0;
    free(fits);
    ktensor->factors = mats;
    return r;
}

/* hicoo/cpd.c:149-195: random rank-matrix factors (seeded, see sptgbSetSeed),
 * the HiCOO CP-ALS loop, factors handed to the rank Kruskal tensor (the
 * structs stay allocated; factors[nmodes] is NULL). */
int sptCpdAlsHiCOO(sptSparseTensorHiCOO const *const hitsr, sptIndex const rank, sptIndex const niters,
                   double const tol, sptRankKruskalTensor *ktensor) {
    const sptIndex N = hitsr->nmodes;
    if (rank < 1 || rank > 64) return SPTERR_VALUE_ERROR;
    sptRankMatrix **mats = (sptRankMatrix **)calloc(N + 1, sizeof(*mats));
    if (!mats) return SPTERR_OS_ERROR;
    for (sptIndex m = 0; m < N; ++m) {
        mats[m] = (sptRankMatrix *)malloc(sizeof(sptRankMatrix));
        int e = sptNewRankMatrix(mats[m], hitsr->ndims[m], (sptElementIndex)rank);
        if (e) return e;
        sptRandomizeRankMatrix(mats[m], hitsr->ndims[m], (sptElementIndex)rank);
    }
    double *fits = (double *)calloc(niters ? niters : 1, sizeof(double));
    sptIndex done = 0;
    const int r = sptgbCpdAlsHiCOO(hitsr, rank, niters, tol, mats, ktensor->lambda, fits, &done);
    ktensor->fit = done > 0 ? fits[done - 1] : 0.0;
    free(fits);
    ktensor->factors = mats;
    return r;
}

int sptOmpCpdAlsHiCOO(sptSparseTensorHiCOO const *const hitsr, sptIndex const rank, sptIndex const niters,
                      double const tol, const int tk, int balanced, sptRankKruskalTensor *ktensor) {
    (void)tk;
    (void)balanced;
    return sptCpdAlsHiCOO(hitsr, rank, niters, tol, ktensor);
}

int sptOmpCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters, double const tol,
                 const int tk, const int use_reduce, sptKruskalTensor *ktensor) {
    (void)tk;
    (void)use_reduce;
    return sptCpdAls(spten, rank, niters, tol, ktensor);
}

/* Declared but never defined by the reference (cpds.h:40-45). */
int sptCudaCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters, double const tol,
                  sptKruskalTensor *ktensor) {
    return sptCpdAls(spten, rank, niters, tol, ktensor);
}

/* sptensor.c:96-107, FP64 sum on the GPU. */
static double sumsq_host(const float *v, uint64_t n) {
    if (sptgb_ctx()) return NAN;
    const cudaStream_t s = sptgb_stream();
    double out = NAN;
    float *d = NULL;
    double *ws = NULL;
    if (n == 0) return 0.0;
    if (cudaMalloc((void **)&d, n * sizeof(float)) != cudaSuccess) goto done;
    if (cudaMalloc((void **)&ws, SPTGB_NPART * sizeof(double) + 64) != cudaSuccess) goto done;
    if (cudaMemcpyAsync(d, v, n * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess) goto done;
    if (sptgb_sumsq(d, n, ws + SPTGB_NPART, ws, s) != cudaSuccess) goto done;
    if (cudaMemcpyAsync(&out, ws + SPTGB_NPART, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) goto done;
    cudaStreamSynchronize(s);
done:
    if (d) cudaFree(d);
    if (ws) cudaFree(ws);
    return out;
}

double SparseTensorFrobeniusNormSquared(sptSparseTensor const *const spten) {
    return sumsq_host(spten->values.data, spten->nnz);
}

double sptSparseTensorFrobeniusNormSquaredHiCOO(sptSparseTensorHiCOO const *const hitsr) {
    return sumsq_host(hitsr->values.data, hitsr->nnz);
}
