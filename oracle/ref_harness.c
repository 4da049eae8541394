/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * Flat-array entry points over the reference library itself, compiled by
 * oracle/Makefile (target `ref`) together with ParTI!'s own sources into
 * oracle/_ref/libparti_ref.so.  Used only where the reference sources exist:
 * to generate tests/golden/ and to time the reference's OpenMP MTTKRP beside
 * the oracle port.  Every call goes through the reference's public API.
 */
#define _GNU_SOURCE
#include <ParTI.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "clapack.h"

/* Exported by the reference but declared in none of its headers
 * (cpd.c:30-36, cpd_omp.c:32-41). */
double CpdAlsStep(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters, double const tol,
                  sptMatrix **mats, sptValue *const lambda);
double OmpCpdAlsStep(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters,
                     double const tol, const int tk, const int use_reduce, sptMatrix **mats, sptMatrix **copy_mats,
                     sptValue *const lambda);

static void build_tensor(sptSparseTensor *X, uint32_t nmodes, const uint32_t *ndims, uint64_t nnz,
                         uint32_t *const *inds, const float *vals) {
    sptNewSparseTensor(X, nmodes, ndims);
    for (uint32_t m = 0; m < nmodes; ++m) {
        sptResizeIndexVector(&X->inds[m], nnz);
        memcpy(X->inds[m].data, inds[m], nnz * sizeof(uint32_t));
    }
    sptResizeValueVector(&X->values, nnz);
    memcpy(X->values.data, vals, nnz * sizeof(float));
    X->nnz = nnz;
}

static sptMatrix **build_mats(uint32_t nmodes, const uint32_t *ndims, uint32_t R, float *const *mats, uint32_t stride) {
    sptMatrix **U = (sptMatrix **)malloc((nmodes + 1) * sizeof(*U));
    uint32_t maxd = 0;
    for (uint32_t m = 0; m < nmodes; ++m) {
        U[m] = (sptMatrix *)malloc(sizeof(sptMatrix));
        sptNewMatrix(U[m], ndims[m], R);
        if (U[m]->stride != stride) abort();
        memcpy(U[m]->values, mats[m], (size_t)ndims[m] * stride * sizeof(float));
        if (ndims[m] > maxd) maxd = ndims[m];
    }
    U[nmodes] = (sptMatrix *)malloc(sizeof(sptMatrix));
    sptNewMatrix(U[nmodes], maxd, R);
    sptConstantMatrix(U[nmodes], 0);
    return U;
}

static void free_mats(sptMatrix **U, uint32_t nmodes) {
    for (uint32_t m = 0; m <= nmodes; ++m) {
        sptFreeMatrix(U[m]);
        free(U[m]);
    }
    free(U);
}

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* order == NULL: sptSparseTensorSortIndex; else SortIndexCustomOrder. */
int ref_sort(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, float *vals,
             const uint32_t *order) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    if (order) sptSparseTensorSortIndexCustomOrder(&X, order, 1, 1);
    else sptSparseTensorSortIndex(&X, 1, 1);
    for (uint32_t m = 0; m < nmodes; ++m) memcpy(inds[m], X.inds[m].data, nnz * 4);
    memcpy(vals, X.values.data, nnz * 4);
    sptFreeSparseTensor(&X);
    return 0;
}

/* which: 0 sptMTTKRP, 1 sptOmpMTTKRP_Reduce, 2 sptOmpMTTKRP.  Returns the
 * time of `reps` calls (after one warm-up call) in *seconds. */
int ref_mttkrp(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, const float *vals,
               uint32_t R, float *const *mats, uint32_t stride, const uint32_t *mats_order, uint32_t mode, float *out,
               int which, int tk, int reps, double *seconds) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    sptMatrix **U = build_mats(nmodes, ndims, R, mats, stride);
    U[nmodes]->nrows = ndims[mode];
    sptMatrix **copies = NULL;
    if (which == 1) {
        copies = (sptMatrix **)malloc(tk * sizeof(*copies));
        for (int t = 0; t < tk; ++t) {
            copies[t] = (sptMatrix *)malloc(sizeof(sptMatrix));
            sptNewMatrix(copies[t], ndims[mode], R);
        }
    }
    int r = 0;
    double t0 = 0;
    for (int k = 0; k <= reps; ++k) {
        if (k == 1) t0 = now_s();
        if (which == 0) r = sptMTTKRP(&X, U, (sptIndex *)mats_order, mode);
        else if (which == 1) r = sptOmpMTTKRP_Reduce(&X, U, copies, (sptIndex *)mats_order, mode, tk);
        else r = sptOmpMTTKRP(&X, U, (sptIndex *)mats_order, mode, tk);
    }
    if (seconds) *seconds = reps ? (now_s() - t0) / reps : 0.0;
    memcpy(out, U[nmodes]->values, (size_t)ndims[mode] * stride * 4);
    if (copies) {
        for (int t = 0; t < tk; ++t) {
            sptFreeMatrix(copies[t]);
            free(copies[t]);
        }
        free(copies);
    }
    free_mats(U, nmodes);
    sptFreeSparseTensor(&X);
    return r;
}

typedef struct {
    uint64_t nb, nk, ncptr, max_nnzb;
    uint64_t *bptr, *kptr, *cptr;
    uint32_t *binds;
    uint8_t *einds;
    uint32_t *nkiters;
    uint32_t *kschr_len;
    uint32_t *kschr;
} ref_hicoo_out;

/* sptSparseTensorToHiCOO with tk = 1; inds/vals receive the sorted COO. */
int ref_hicoo(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, float *vals, int sb_bits,
              int sk_bits, ref_hicoo_out *o) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    sptSparseTensorHiCOO H;
    sptNnzIndex mx = 0;
    int r = sptSparseTensorToHiCOO(&H, &mx, &X, (sptElementIndex)sb_bits, (sptElementIndex)sk_bits, 1);
    for (uint32_t m = 0; m < nmodes; ++m) memcpy(inds[m], X.inds[m].data, nnz * 4);
    memcpy(vals, X.values.data, nnz * 4);
    o->nb = H.bptr.len - 1;
    o->nk = H.kptr.len - 1;
    o->ncptr = H.cptr.len;
    o->max_nnzb = mx;
    memcpy(o->bptr, H.bptr.data, H.bptr.len * 8);
    memcpy(o->kptr, H.kptr.data, H.kptr.len * 8);
    memcpy(o->cptr, H.cptr.data, H.cptr.len * 8);
    for (uint32_t m = 0; m < nmodes; ++m) {
        memcpy(o->binds + (size_t)m * o->nb, H.binds[m].data, o->nb * 4);
        memcpy(o->einds + (size_t)m * nnz, H.einds[m].data, nnz);
        o->nkiters[m] = H.nkiters[m];
    }
    uint64_t row = 0, ent = 0;
    const uint64_t sk = 1ull << sk_bits;
    for (uint32_t m = 0; m < nmodes; ++m) {
        const uint64_t kn = (ndims[m] + sk - 1) / sk;
        for (uint64_t i = 0; i < kn; ++i) {
            o->kschr_len[row++] = (uint32_t)H.kschr[m][i].len;
            for (uint64_t e = 0; e < H.kschr[m][i].len; ++e) o->kschr[ent++] = H.kschr[m][i].data[e];
        }
    }
    sptFreeSparseTensorHiCOO(&H);
    sptFreeSparseTensor(&X);
    return r;
}

int ref_mttkrp_hicoo(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, const float *vals,
                     int sb_bits, int sk_bits, uint32_t R, float *const *mats, uint32_t stride,
                     const uint32_t *mats_order, uint32_t mode, float *out) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    sptSparseTensorHiCOO H;
    sptNnzIndex mx = 0;
    sptSparseTensorToHiCOO(&H, &mx, &X, (sptElementIndex)sb_bits, (sptElementIndex)sk_bits, 1);
    sptMatrix **U = build_mats(nmodes, ndims, R, mats, stride);
    U[nmodes]->nrows = ndims[mode];
    int r = sptMTTKRPHiCOO(&H, U, (sptIndex *)mats_order, mode);
    memcpy(out, U[nmodes]->values, (size_t)ndims[mode] * stride * 4);
    free_mats(U, nmodes);
    sptFreeSparseTensorHiCOO(&H);
    sptFreeSparseTensor(&X);
    return r;
}

/* Fit of the model against the tensor in FP64 from the full symmetric Gram
 * matrices and <X,K> summed over the nonzeros; the reference's own fit reads
 * a Gram triangle its ssyrk_ call never writes. */
static double corrected_fit(const sptSparseTensor *X, sptMatrix **U, const sptValue *lambda, uint32_t R) {
    const uint32_t N = X->nmodes;
    double nx = 0, inner = 0, nk = 0;
#pragma omp parallel for reduction(+ : nx, inner) schedule(static)
    for (uint64_t x = 0; x < X->nnz; ++x) {
        const double v = X->values.data[x];
        nx += v * v;
        double s = 0;
        for (uint32_t r = 0; r < R; ++r) {
            double p = lambda[r];
            for (uint32_t m = 0; m < N; ++m) p *= U[m]->values[(size_t)X->inds[m].data[x] * U[m]->stride + r];
            s += p;
        }
        inner += v * s;
    }
#pragma omp parallel for reduction(+ : nk) schedule(dynamic)
    for (uint32_t p = 0; p < R; ++p)
        for (uint32_t q = 0; q < R; ++q) {
            double h = 1;
            for (uint32_t m = 0; m < N; ++m) {
                double g = 0;
                for (uint32_t i = 0; i < U[m]->nrows; ++i)
                    g += (double)U[m]->values[(size_t)i * U[m]->stride + p] * U[m]->values[(size_t)i * U[m]->stride + q];
                h *= g;
            }
            nk += h * lambda[p] * lambda[q];
        }
    nk = fabs(nk);
    double res = nx + nk - 2 * inner;
    if (res > 0) res = sqrt(res);
    return 1 - res / sqrt(nx);
}

/* The CP-ALS loop of cpd.c:76-127 driven through the reference's exported
 * pieces (sptMTTKRP, sptMatrixSolveNormals, sptMatrix2Norm/MaxNorm, ssyrk_,
 * GetFinalLambda) from caller factors, recording the corrected fit after
 * every iteration; then CpdAlsStep itself from the same factors, so that the
 * caller can check both end in the same factors bit for bit. */
int ref_cpd_trace(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, const float *vals,
                  uint32_t R, uint32_t niters, float *const *init, uint32_t stride, float *const *final_loop,
                  float *lambda_loop, double *fits, float *const *final_step, float *lambda_step, double *step_fit) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    sptMatrix **U = build_mats(nmodes, ndims, R, init, stride);
    sptMatrix **ata = (sptMatrix **)malloc((nmodes + 1) * sizeof(*ata));
    for (uint32_t m = 0; m <= nmodes; ++m) {
        ata[m] = (sptMatrix *)malloc(sizeof(sptMatrix));
        sptNewMatrix(ata[m], R, R);
    }
    char uplo = 'L', notrans = 'N';
    float alpha = 1, beta = 0;
    int br = (int)R, bs = (int)stride;
    for (uint32_t m = 0; m < nmodes; ++m) {
        int nr = (int)U[m]->nrows;
        ssyrk_(&uplo, &notrans, &br, &nr, &alpha, U[m]->values, &bs, &beta, ata[m]->values, &bs);
    }
    sptIndex *order = (sptIndex *)malloc(nmodes * sizeof(sptIndex));
    for (uint32_t it = 0; it < niters; ++it) {
        for (uint32_t m = 0; m < nmodes; ++m) {
            U[nmodes]->nrows = U[m]->nrows;
            order[0] = m;
            for (uint32_t i = 1; i < nmodes; ++i) order[i] = (m + i) % nmodes;
            sptMTTKRP(&X, U, order, m);
            memcpy(U[m]->values, U[nmodes]->values, (size_t)U[m]->nrows * stride * sizeof(float));
            sptMatrixSolveNormals(m, nmodes, ata, U[m]);
            if (it == 0) sptMatrix2Norm(U[m], lambda_loop);
            else sptMatrixMaxNorm(U[m], lambda_loop);
            int nr = (int)U[m]->nrows;
            ssyrk_(&uplo, &notrans, &br, &nr, &alpha, U[m]->values, &bs, &beta, ata[m]->values, &bs);
        }
        fits[it] = corrected_fit(&X, U, lambda_loop, R);
    }
    GetFinalLambda(R, nmodes, U, lambda_loop);
    for (uint32_t m = 0; m < nmodes; ++m) memcpy(final_loop[m], U[m]->values, (size_t)ndims[m] * stride * 4);
    free_mats(U, nmodes);

    sptMatrix **V = build_mats(nmodes, ndims, R, init, stride);
    *step_fit = CpdAlsStep(&X, R, niters, 0.0, V, lambda_step);
    for (uint32_t m = 0; m < nmodes; ++m) memcpy(final_step[m], V[m]->values, (size_t)ndims[m] * stride * 4);
    free_mats(V, nmodes);
    for (uint32_t m = 0; m <= nmodes; ++m) {
        sptFreeMatrix(ata[m]);
        free(ata[m]);
    }
    free(ata);
    free(order);
    sptFreeSparseTensor(&X);
    return 0;
}

/* The reference's sptSparseTensorMulMatrix (mmul.c:37-97) on a tensor marked
 * unsorted (sortorder all zero, as its text loader leaves it).  Writes the
 * sorted coordinates/values back, the fiber coordinates (fib[m], m != mode)
 * and Y (nfib x ystride); returns the number of fibers. */
uint64_t ref_ttm(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, float *vals,
                 uint32_t mode, const float *U, uint32_t urows, uint32_t ncols, uint32_t *const *fib, float *Y,
                 uint32_t *ystride_out) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    for (uint32_t m = 0; m < nmodes; ++m) X.sortorder[m] = 0;
    sptMatrix Um;
    sptNewMatrix(&Um, urows, ncols);
    for (uint32_t i = 0; i < urows; ++i) memcpy(Um.values + (size_t)i * Um.stride, U + (size_t)i * ncols, ncols * 4);
    sptSemiSparseTensor Yt;
    sptSparseTensorMulMatrix(&Yt, &X, &Um, mode);
    for (uint32_t m = 0; m < nmodes; ++m) memcpy(inds[m], X.inds[m].data, nnz * 4);
    memcpy(vals, X.values.data, nnz * 4);
    for (uint32_t m = 0; m < nmodes; ++m)
        if (m != mode) memcpy(fib[m], Yt.inds[m].data, Yt.nnz * 4);
    memcpy(Y, Yt.values.values, (size_t)Yt.nnz * Yt.stride * 4);
    *ystride_out = Yt.stride;
    const uint64_t nf = Yt.nnz;
    sptFreeSemiSparseTensor(&Yt);
    sptFreeMatrix(&Um);
    sptFreeSparseTensor(&X);
    return nf;
}

/* The reference's text reader, sptLoadSparseTensor (sptensor/load.c with
 * collect.c): the tensor it builds copied out into caller arrays of `cap`
 * entries.  Returns the reader's own code (or -2 when the file does not
 * open, -3 when cap is too small or the order above 8). */
int ref_load_tns(const char *path, uint32_t start_index, uint32_t *nmodes_out, uint32_t *ndims_out, uint64_t cap,
                 uint32_t *const *inds, float *vals, uint64_t *nnz_out) {
    FILE *fp = fopen(path, "r");
    if (!fp) return -2;
    sptSparseTensor X;
    memset(&X, 0, sizeof X);
    const int r = sptLoadSparseTensor(&X, start_index, fp);
    fclose(fp);
    if (r) return r;
    if (X.nmodes > 8 || X.nnz > cap) {
        sptFreeSparseTensor(&X);
        return -3;
    }
    *nmodes_out = X.nmodes;
    for (uint32_t m = 0; m < X.nmodes; ++m) {
        ndims_out[m] = X.ndims[m];
        memcpy(inds[m], X.inds[m].data, X.nnz * sizeof(uint32_t));
    }
    memcpy(vals, X.values.data, X.nnz * sizeof(float));
    *nnz_out = X.nnz;
    sptFreeSparseTensor(&X);
    return 0;
}

/* The reference's dense CP-ALS helpers on flat R x stride (Grams) or
 * nrows x stride (factors) arrays: sptMatrixDotMulSeqTriangle,
 * sptMatrix2Norm / sptMatrixMaxNorm, sptKruskalTensorFrobeniusNormSquared and
 * sptSparseKruskalTensorInnerProduct. */
static sptMatrix *mat_from(uint32_t nrows, uint32_t R, const float *vals, uint32_t stride) {
    sptMatrix *M = (sptMatrix *)malloc(sizeof(sptMatrix));
    sptNewMatrix(M, nrows, R);
    if (M->stride != stride) abort();
    if (vals) memcpy(M->values, vals, (size_t)nrows * stride * sizeof(float));
    else memset(M->values, 0, (size_t)M->cap * stride * sizeof(float));
    return M;
}

static void mats_free(sptMatrix **M, uint32_t n) {
    for (uint32_t m = 0; m < n; ++m) {
        sptFreeMatrix(M[m]);
        free(M[m]);
    }
}

int ref_dotmul_triangle(uint32_t nmodes, uint32_t mode, uint32_t R, float *const *grams, uint32_t stride, float *out) {
    sptMatrix *M[9];
    if (nmodes > 8) return -3;
    for (uint32_t m = 0; m < nmodes; ++m) M[m] = mat_from(R, R, grams[m], stride);
    M[nmodes] = mat_from(R, R, NULL, stride);
    const int r = sptMatrixDotMulSeqTriangle(mode, nmodes, M);
    memcpy(out, M[nmodes]->values, (size_t)R * stride * sizeof(float));
    mats_free(M, nmodes + 1);
    return r;
}

int ref_colnorm(int use_max, uint32_t nrows, uint32_t R, float *A, uint32_t stride, float *lambda) {
    sptMatrix *M = mat_from(nrows, R, A, stride);
    const int r = use_max ? sptMatrixMaxNorm(M, lambda) : sptMatrix2Norm(M, lambda);
    memcpy(A, M->values, (size_t)nrows * stride * sizeof(float));
    mats_free(&M, 1);
    return r;
}

double ref_kruskal_normsq(uint32_t nmodes, uint32_t R, float *const *ata, uint32_t stride, const float *lambda) {
    sptMatrix *M[9];
    if (nmodes > 8) return NAN;
    for (uint32_t m = 0; m < nmodes; ++m) M[m] = mat_from(R, R, ata[m], stride);
    M[nmodes] = mat_from(R, R, NULL, stride);
    const double v = sptKruskalTensorFrobeniusNormSquared(nmodes, (sptValue *)lambda, M);
    mats_free(M, nmodes + 1);
    return v;
}

/* mats[0..nmodes-1]: factors (only the last one is read), mout: the last
 * mode's MTTKRP output, both I x stride with I the last mode's size. */
double ref_kruskal_inner(uint32_t nmodes, uint32_t R, const uint32_t *ndims, float *const *mats, const float *mout,
                         uint32_t stride, const float *lambda) {
    sptMatrix *M[9];
    if (nmodes > 8) return NAN;
    for (uint32_t m = 0; m < nmodes; ++m) M[m] = mat_from(ndims[m], R, mats[m], stride);
    M[nmodes] = mat_from(ndims[nmodes - 1], R, mout, stride);
    const double v = sptSparseKruskalTensorInnerProduct(nmodes, (sptValue *)lambda, M);
    mats_free(M, nmodes + 1);
    return v;
}

/* sptMatrixSolveNormals (matrix_solver.c:32-83): rhs (nrows x stride) is
 * overwritten with X, X G = rhs, G the Hadamard of the other Grams. */
int ref_solve_normals(uint32_t nmodes, uint32_t mode, uint32_t R, float *const *grams, uint32_t stride, uint32_t nrows,
                      float *rhs) {
    sptMatrix *M[9];
    if (nmodes > 8) return -3;
    for (uint32_t m = 0; m < nmodes; ++m) M[m] = mat_from(R, R, grams[m], stride);
    M[nmodes] = mat_from(R, R, NULL, stride);
    sptMatrix *B = mat_from(nrows, R, rhs, stride);
    const int r = sptMatrixSolveNormals(mode, nmodes, M, B);
    memcpy(rhs, B->values, (size_t)nrows * stride * sizeof(float));
    mats_free(M, nmodes + 1);
    mats_free(&B, 1);
    return r;
}

/* The reference's text writers into `path`: sptDumpSparseTensor,
 * sptDumpMatrix, sptDumpIndexArray, sptDumpNnzIndexArray. */
int ref_dump_tensor(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, const float *vals,
                    uint32_t start_index, const char *path) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    FILE *fp = fopen(path, "w");
    if (!fp) return -2;
    const int r = sptDumpSparseTensor(&X, start_index, fp);
    fclose(fp);
    sptFreeSparseTensor(&X);
    return r;
}

int ref_dump_matrix(uint32_t nrows, uint32_t ncols, const float *vals, uint32_t stride, const char *path) {
    sptMatrix *M = mat_from(nrows, ncols, vals, stride);
    FILE *fp = fopen(path, "w");
    if (!fp) return -2;
    const int r = sptDumpMatrix(M, fp);
    fclose(fp);
    mats_free(&M, 1);
    return r;
}

int ref_dump_arrays(const uint32_t *a, uint64_t na, const uint64_t *b, uint64_t nb, const char *path) {
    FILE *fp = fopen(path, "w");
    if (!fp) return -2;
    int r = sptDumpIndexArray((sptIndex *)a, na, fp);
    if (!r) r = sptDumpNnzIndexArray((sptNnzIndex *)b, nb, fp);
    fclose(fp);
    return r;
}

/* ----------------------------------------------------- timing sessions --
 * The reference's own CPU path timed on a tensor it holds in its own
 * containers: the tensor comes from the library's seeded generator
 * (sptgbGenerate, gen.c linked into this library, where it builds the tensor
 * through the reference's sptNewSparseTensor), the factors from the same
 * generator's sptgbFillMatrix, so a process timing the reference loads no
 * part of libParTI.so.  Protocol of examples/mttkrp.c:160-274 (sortcase 0):
 * the tensor is put in lexicographic order with sptSparseTensorSortIndex
 * (force = 0: the generator's output is already in that order and its
 * sortorder is the identity, so the reference skips the sort), mats_order =
 * {mode, mode+1, ...}, and each call is timed alone. */
int sptgbGenerate(sptSparseTensor *X, const void *spec);
int sptgbFillMatrix(sptMatrix *mtx, uint64_t seed, uint64_t stream_id, float lo, float hi);

typedef struct {
    sptSparseTensor X;
    sptMatrix **U;      /* nmodes factors, then the output mats[nmodes] */
    sptMatrix **copies; /* tk thread-private outputs of sptOmpMTTKRP_Reduce */
    uint32_t R;
    int tk;
} ref_session;

void ref_session_close(ref_session *s) {
    if (!s) return;
    if (s->U) free_mats(s->U, s->X.nmodes);
    if (s->copies) {
        for (int t = 0; t < s->tk; ++t) {
            sptFreeMatrix(s->copies[t]);
            free(s->copies[t]);
        }
        free(s->copies);
    }
    sptFreeSparseTensor(&s->X);
    free(s);
}

/* Generates the tensor and factors U[0,1) (seed fac_seed, stream m for mode
 * m, as sptgbFillMatrix fills them for the GPU arm) and the tk copies. */
ref_session *ref_session_open(const void *spec, uint32_t R, uint64_t fac_seed, int tk) {
    ref_session *s = (ref_session *)calloc(1, sizeof *s);
    if (!s) return NULL;
    if (sptgbGenerate(&s->X, spec)) {
        free(s);
        return NULL;
    }
    sptSparseTensorSortIndex(&s->X, 0, tk);
    const uint32_t N = s->X.nmodes;
    uint32_t maxd = 0;
    s->U = (sptMatrix **)malloc((N + 1) * sizeof(*s->U));
    for (uint32_t m = 0; m < N; ++m) {
        s->U[m] = (sptMatrix *)malloc(sizeof(sptMatrix));
        sptNewMatrix(s->U[m], s->X.ndims[m], R);
        sptgbFillMatrix(s->U[m], fac_seed, m, 0.0f, 1.0f);
        if (s->X.ndims[m] > maxd) maxd = s->X.ndims[m];
    }
    s->U[N] = (sptMatrix *)malloc(sizeof(sptMatrix));
    sptNewMatrix(s->U[N], maxd, R);
    sptConstantMatrix(s->U[N], 0);
    s->copies = (sptMatrix **)malloc(tk * sizeof(*s->copies));
    for (int t = 0; t < tk; ++t) {
        s->copies[t] = (sptMatrix *)malloc(sizeof(sptMatrix));
        sptNewMatrix(s->copies[t], maxd, R);
        sptConstantMatrix(s->copies[t], 0);
    }
    s->R = R;
    s->tk = tk;
    return s;
}

uint64_t ref_session_nnz(const ref_session *s) { return s->X.nnz; }

void ref_session_ndims(const ref_session *s, uint32_t *out) {
    for (uint32_t m = 0; m < s->X.nmodes; ++m) out[m] = s->X.ndims[m];
}

/* One MTTKRP of `mode`: which 0 sptMTTKRP, 1 sptOmpMTTKRP_Reduce,
 * 2 sptOmpMTTKRP (atomics).  Returns the seconds of the call (negative when
 * the call fails); out (ndims[mode] x stride, may be NULL) receives M. */
double ref_session_mttkrp(ref_session *s, int which, uint32_t mode, float *out) {
    const uint32_t N = s->X.nmodes;
    sptIndex order[8];
    order[0] = mode;
    for (uint32_t i = 1; i < N; ++i) order[i] = (mode + i) % N;
    s->U[N]->nrows = s->X.ndims[mode];
    const double t0 = now_s();
    int r;
    if (which == 0) r = sptMTTKRP(&s->X, s->U, order, mode);
    else if (which == 1) r = sptOmpMTTKRP_Reduce(&s->X, s->U, s->copies, order, mode, s->tk);
    else r = sptOmpMTTKRP(&s->X, s->U, order, mode, s->tk);
    const double dt = now_s() - t0;
    if (out) memcpy(out, s->U[N]->values, (size_t)s->X.ndims[mode] * s->U[N]->stride * sizeof(float));
    return r ? -1.0 : dt;
}

/* The reference's own CUDA MTTKRP, sptCudaMTTKRPOneKernel with impl_num =
 * impl (mttkrp_cuda_onekernel.cu:41-427; 15 is its rank-split kernel,
 * spt_MTTKRPKernelRankSplitNnz3DOneKernel, mttkrp_cuda_kernels.cu:544-603):
 * every call copies the tensor and factors to the GPU, runs one kernel with
 * one atomicAdd per (nonzero, column) and copies the result back; it prints
 * its own phase times ("[CUDA SpTns MTTKRP]: <s> s" is the kernel).  Returns
 * the seconds of the whole call, negative when it fails or when the library
 * was built without CUDA. */
double ref_session_cuda_mttkrp(ref_session *s, uint32_t mode, uint32_t impl, float *out) {
#ifdef REF_HAVE_CUDA
    const uint32_t N = s->X.nmodes;
    sptIndex order[8];
    order[0] = mode;
    for (uint32_t i = 1; i < N; ++i) order[i] = (mode + i) % N;
    s->U[N]->nrows = s->X.ndims[mode];
    const double t0 = now_s();
    const int r = sptCudaMTTKRPOneKernel(&s->X, s->U, order, mode, impl);
    const double dt = now_s() - t0;
    if (out) memcpy(out, s->U[N]->values, (size_t)s->X.ndims[mode] * s->U[N]->stride * sizeof(float));
    return r ? -1.0 : dt;
#else
    (void)s, (void)mode, (void)impl, (void)out;
    return -2.0;
#endif
}

/* The reference's sptOmpCpdAls loop, OmpCpdAlsStep (cpd_omp.c:32-157), run
 * from the session's factors as the initial guess (cpd_omp.c:166-228 only
 * adds sptRandomizeMatrix initialisation and the allocations); the factors
 * are overwritten with the result.  Returns the seconds of the call;
 * *fit receives the corrected fit of the result (FP64, full symmetric Grams),
 * lambda (R entries) the final lambda. */
double ref_session_cpd(ref_session *s, uint32_t niters, int use_reduce, float *lambda, double *fit) {
    const double t0 = now_s();
    OmpCpdAlsStep(&s->X, s->R, niters, 0.0, s->tk, use_reduce, s->U, s->copies, lambda);
    const double dt = now_s() - t0;
    if (fit) *fit = corrected_fit(&s->X, s->U, lambda, s->R);
    return dt;
}

/* OmpCpdAlsStep on a tensor given as flat arrays from caller factors (one
 * request of a stream).  Returns the seconds of the OmpCpdAlsStep call. */
double ref_omp_cpd(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, uint32_t *const *inds, const float *vals,
                   uint32_t R, uint32_t niters, float *const *init, uint32_t stride, int tk, float *lambda,
                   double *fit) {
    sptSparseTensor X;
    build_tensor(&X, nmodes, ndims, nnz, inds, vals);
    sptMatrix **U = build_mats(nmodes, ndims, R, init, stride);
    uint32_t maxd = 0;
    for (uint32_t m = 0; m < nmodes; ++m)
        if (ndims[m] > maxd) maxd = ndims[m];
    sptMatrix **copies = (sptMatrix **)malloc(tk * sizeof(*copies));
    for (int t = 0; t < tk; ++t) {
        copies[t] = (sptMatrix *)malloc(sizeof(sptMatrix));
        sptNewMatrix(copies[t], maxd, R);
        sptConstantMatrix(copies[t], 0);
    }
    const double t0 = now_s();
    OmpCpdAlsStep(&X, R, niters, 0.0, tk, 1, U, copies, lambda);
    const double dt = now_s() - t0;
    if (fit) *fit = corrected_fit(&X, U, lambda, R);
    for (int t = 0; t < tk; ++t) {
        sptFreeMatrix(copies[t]);
        free(copies[t]);
    }
    free(copies);
    free_mats(U, nmodes);
    sptFreeSparseTensor(&X);
    return dt;
}
