// Dense FP64 pieces of CP-ALS (rank <= 64).
//
// Reference steps restated here (src/sptensor/cpd.c:64-127):
//   ata[m] = A_m^T A_m                       (ssyrk_, cpd.c:65-70, :106-108)
//   H = Hadamard of ata[n], n != m           (sptMatrixDotMulSeqTriangle,
//                                             matrix.c:341-386)
//   A_m = MTTKRP_m * H^{-1}                  (spotrf_/spotrs_, sgesv_ when H
//                                             is not SPD; matrix_solver.c:32-83)
//   normalise columns: 2-norm at it 0, else max-norm clamped to >= 1
//                                            (matrix.c:390-554)
//   fit = 1 - ||X - K|| / ||X||               (ktensor.c:102-257)
// All R x R arithmetic and every reduction over rows runs in FP64; factor
// matrices stay FP32 row-major with `stride` floats per row.  The fit uses
// the full symmetric Gram matrices (the reference reads a triangle that its
// ssyrk_ call never writes, ktensor.c:149-164 vs cpd.c:68).
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "../sptgb_internal.h"

#include "dense_common.cuh"

namespace {
using namespace sptgb_dense;

__global__ void __launch_bounds__(DT) k_gram_partial(const float *__restrict__ A, uint32_t nrows, int rank, int stride, double *__restrict__ part) { gram_partial_body(A, nrows, rank, stride, part, blockIdx.x, gridDim.x); }
__global__ void k_gram_reduce(const double *__restrict__ part, int nblk, int rank, double *__restrict__ G) { gram_reduce_body(part, nblk, rank, G); }
__global__ void __launch_bounds__(DT) k_solve_prepare(GramPtrs grams, int nmodes, int mode, int rank, double *__restrict__ S,
                int *__restrict__ status) { solve_prepare_body(grams, nmodes, mode, rank, S, status); }
__global__ void __launch_bounds__(DT, 2) k_solve_rows(const float *__restrict__ M, float *__restrict__ X, uint32_t nrows, int rank, int stride,
             const double *__restrict__ S, const int *__restrict__ sstatus, double *__restrict__ gpart, double *__restrict__ mpart) { solve_rows_body(M, X, nrows, rank, stride, S, sstatus, gpart, mpart, blockIdx.x, gridDim.x); }
__global__ void k_lambda(const double *__restrict__ gpart, const double *__restrict__ mpart, int nblk, int rank,
                         int use_2norm, double *__restrict__ G, float *__restrict__ lambda_f32,
                         double *__restrict__ colmax_out) { lambda_body(gpart, mpart, nblk, rank, use_2norm, G, lambda_f32, colmax_out); }
__global__ void k_scale_cols(float *__restrict__ X, uint32_t nrows, int rank, int stride,
                             const float *__restrict__ lambda) { scale_cols_body(X, nrows, rank, stride, lambda, blockIdx.x, gridDim.x); }
__global__ void __launch_bounds__(DT) k_inner_partial(const float *__restrict__ A, const float *__restrict__ M, uint32_t nrows, int rank, int stride,
                double *__restrict__ part) { inner_partial_body(A, M, nrows, rank, stride, part, blockIdx.x, gridDim.x); }
__global__ void k_fit_final(const double *__restrict__ part, int nblk, int rank, const float *__restrict__ lambda,
                            GramPtrs gp, int nmodes, const double *__restrict__ normX2, double *__restrict__ fit) { fit_final_body(part, nblk, rank, lambda, gp, nmodes, normX2, fit); }
__global__ void __launch_bounds__(DT) k_sumsq_partial(const float *__restrict__ v, uint64_t n, double *part) { sumsq_partial_body(v, n, part, blockIdx.x, gridDim.x); }
__global__ void k_sum_final(const double *part, int nblk, double *out) { sum_final_body(part, nblk, out); }
__global__ void __launch_bounds__(DT) k_colsq_partial(const float *__restrict__ A, uint32_t nrows, int rank, int stride, double *__restrict__ part) { colsq_partial_body(A, nrows, rank, stride, part, blockIdx.x, gridDim.x); }
__global__ void k_colnorm_final(const double *part, int nblk, int rank, float *lambda_mul, float *norms) { colnorm_final_body(part, nblk, rank, lambda_mul, norms); }
__global__ void k_f32_to_bf16(const float *__restrict__ in, uint16_t *__restrict__ out, uint64_t n) { f32_to_bf16_body(in, out, n, blockIdx.x, gridDim.x); }

}  // namespace

extern "C" size_t sptgb_dense_ws_bytes(int rank, int max_blocks) {
    (void)max_blocks;
    const size_t P = (size_t)rank * (rank + 1) / 2;
    return (NBLK * (P + 2 * (size_t)rank) + 64) * sizeof(double);
}

extern "C" cudaError_t sptgb_gram(const float *A, uint32_t nrows, int rank, int stride, double *G, double *ws,
                                  cudaStream_t s) {
    if (rank < 1 || rank > RMAX) return cudaErrorInvalidValue;
    const int nb = nblocks_for_rows(nrows);
    k_gram_partial<<<nb, DT, 0, s>>>(A, nrows, rank, stride, ws);
    k_gram_reduce<<<1, DT, 0, s>>>(ws, nb, rank, G);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_solve_prepare(const double *const *grams, int nmodes, int mode, int rank,
                                           double *Hinv, int *status, cudaStream_t s) {
    if (rank < 1 || rank > RMAX) return cudaErrorInvalidValue;
    // once per process (a function-local static is initialised by one thread
    // while the others wait; a failure shows up as the launch's error)
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_solve_prepare, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PREP_SMEM);
    (void)attr;
    GramPtrs gp;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < nmodes ? grams[m] : nullptr;
    k_solve_prepare<<<1, DT, PREP_SMEM, s>>>(gp, nmodes, mode, rank, Hinv, status);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_solve_rows(const float *M, float *X, uint32_t nrows, int rank, int stride,
                                        const double *Hinv, const int *status, double *ws, cudaStream_t s) {
    if (rank < 1 || rank > RMAX) return cudaErrorInvalidValue;
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_solve_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOLVE_SMEM);
    (void)attr;   // once per process, as in sptgb_solve_prepare
    const int nb = nblocks_for_solve(nrows, rank);
    const size_t P = (size_t)rank * (rank + 1) / 2;
    k_solve_rows<<<nb, DT, SOLVE_SMEM, s>>>(M, X, nrows, rank, stride, Hinv, status, ws, ws + NBLK * P);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

// Consumes the partials left in ws by sptgb_solve_rows (same nrows).
extern "C" cudaError_t sptgb_normalize(float *X, uint32_t nrows, int rank, int stride, double *gram,
                                          int use_2norm, float *lambda_f32, const double *ws, cudaStream_t s) {
    const int nb = nblocks_for_solve(nrows, rank);
    const size_t P = (size_t)rank * (rank + 1) / 2;
    k_lambda<<<1, DT, 0, s>>>(ws, ws + NBLK * P, nb, rank, use_2norm, gram, lambda_f32, nullptr);
    uint64_t total = (uint64_t)nrows * rank;
    uint64_t g = (total + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    if (g < 1) g = 1;
    k_scale_cols<<<(unsigned)g, 256, 0, s>>>(X, nrows, rank, stride, lambda_f32);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_fit(const float *A, const float *M, uint32_t nrows, int rank, int stride,
                                 const float *lambda, const double *const *grams, int nmodes, const double *normX2,
                                 double *fit_out, double *ws, cudaStream_t s) {
    if (rank < 1 || rank > RMAX) return cudaErrorInvalidValue;
    int nb = (int)((nrows + 7) / 8);
    if (nb > NBLK) nb = NBLK;
    if (nb < 1) nb = 1;
    GramPtrs gp;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < nmodes ? grams[m] : nullptr;
    k_inner_partial<<<nb, DT, 0, s>>>(A, M, nrows, rank, stride, ws);
    k_fit_final<<<1, DT, 0, s>>>(ws, nb, rank, lambda, gp, nmodes, normX2, fit_out);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_sumsq(const float *v, uint64_t n, double *out, double *ws, cudaStream_t s) {
    int nb = (int)((n + DT - 1) / DT);
    if (nb > NBLK) nb = NBLK;
    if (nb < 1) nb = 1;
    k_sumsq_partial<<<nb, DT, 0, s>>>(v, n, ws);
    k_sum_final<<<1, 32, 0, s>>>(ws, nb, out);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_colnorm_scale(float *A, uint32_t nrows, int rank, int stride, float *lambda_mul,
                                           double *ws, cudaStream_t s) {
    if (rank < 1 || rank > RMAX) return cudaErrorInvalidValue;
    int nb = (int)((nrows + 7) / 8);
    if (nb > NBLK) nb = NBLK;
    if (nb < 1) nb = 1;
    float *norms = (float *)(ws + (size_t)NBLK * rank);
    k_colsq_partial<<<nb, DT, 0, s>>>(A, nrows, rank, stride, ws);
    k_colnorm_final<<<1, 64, 0, s>>>(ws, nb, rank, lambda_mul, norms);
    uint64_t total = (uint64_t)nrows * rank;
    uint64_t g = (total + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    if (g < 1) g = 1;
    k_scale_cols<<<(unsigned)g, 256, 0, s>>>(A, nrows, rank, stride, norms);
    sptgb_count_launch(3);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_f32_to_bf16(const float *in, uint16_t *out, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t g = (n + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 32) g = (uint64_t)sptgb_sm_count() * 32;
    k_f32_to_bf16<<<(unsigned)g, 256, 0, s>>>(in, out, n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

// --------------------------------------------------------------------------
// The reference's dense helpers on caller matrices (FP32, `stride` floats per
// row): sptMatrixDotMulSeqTriangle, sptMatrixMaxNorm,
// sptKruskalTensorFrobeniusNormSquared, sptSparseKruskalTensorInnerProduct.
namespace {

struct F32Ptrs { const float *p[SPTGB_MAX_MODES]; };

// matrix.c:341-386: the upper triangle (j >= i) of every mats[(mode+m) % N],
// m = 1..N-1, multiplied in FP32 in that order, then mirrored.
__global__ void k_hadamard_upper(F32Ptrs mats, int nmodes, int mode, int rank, int stride, float *__restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rank * rank; e += gridDim.x * blockDim.x) {
        const int i = e / rank, j = e % rank;
        if (j < i) continue;
        float v = 1.f;
        for (int m = 1; m < nmodes; ++m) v = __fmul_rn(v, mats.p[(mode + m) % nmodes][i * stride + j]);
        out[i * stride + j] = v;
        out[j * stride + i] = v;
    }
}

// FP64 R x R copies of the caller's Grams from their upper triangles (the
// triangle the reference's solve reads), for the FP64 factorisation.
__global__ void k_grams_upper_f64(F32Ptrs mats, int nmodes, int rank, int stride, double *__restrict__ out) {
    const int RR = rank * rank;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nmodes * RR; e += gridDim.x * blockDim.x) {
        const int m = e / RR, i = (e % RR) / rank, j = e % rank;
        const int a = i < j ? i : j, b = i < j ? j : i;
        out[e] = (double)mats.p[m][a * stride + b];
    }
}

// ktensor.c:126-168, one thread: tmp = 1 over rank x stride, entries
// (row j, column i), j >= i, multiplied over every mode in FP32; then the
// lambda-weighted sum over those entries in the reference's order (i outer,
// j inner; FP32 terms added to an FP64 sum), absolute value.
__global__ void k_kruskal_normsq(F32Ptrs ata, int nmodes, int rank, int stride, const float *__restrict__ lambda,
                                 float *__restrict__ tmp, double *__restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int x = 0; x < rank * stride; ++x) tmp[x] = 1.f;
    for (int m = 0; m < nmodes; ++m)
        for (int i = 0; i < rank; ++i)
            for (int j = i; j < rank; ++j) tmp[j * stride + i] = __fmul_rn(tmp[j * stride + i], ata.p[m][j * stride + i]);
    double norm = 0.0;
    for (int i = 0; i < rank; ++i) {
        norm += (double)__fmul_rn(__fmul_rn(tmp[i + i * stride], lambda[i]), lambda[i]);
        for (int j = i + 1; j < rank; ++j)
            norm += (double)__fmul_rn(__fmul_rn(__fmul_rn(tmp[i + j * stride], lambda[i]), lambda[j]), 2.f);
    }
    *out = fabs(norm);
}

// Per-block column maxima (signed, starting at 0 as matrix.c:484-486).
__global__ void k_colmax_partial(const float *__restrict__ A, uint32_t nrows, int rank, int stride,
                                 float *__restrict__ part) {
    for (int j = threadIdx.x; j < rank; j += blockDim.x) {
        float mx = 0.f;
        for (uint64_t i = blockIdx.x; i < nrows; i += gridDim.x) {
            const float v = A[i * stride + j];
            if (v > mx) mx = v;
        }
        part[(uint64_t)blockIdx.x * rank + j] = mx;
    }
}

// lambda[j] = max over blocks, clamped to >= 1 (matrix.c:541-547).
__global__ void k_colmax_final(const float *__restrict__ part, int nb, int rank, float *__restrict__ lambda) {
    for (int j = threadIdx.x; j < rank; j += blockDim.x) {
        float mx = 0.f;
        for (int b = 0; b < nb; ++b)
            if (part[(uint64_t)b * rank + j] > mx) mx = part[(uint64_t)b * rank + j];
        lambda[j] = mx < 1.f ? 1.f : mx;
    }
}

// Per-block sum over rows of the FP32 products A[i][r] * B[i][r] in FP64
// (ktensor.c:203-236).
__global__ void k_rowdot_partial(const float *__restrict__ A, const float *__restrict__ B, uint32_t nrows, int rank,
                                 int stride, double *__restrict__ part) {
    for (int r = threadIdx.x; r < rank; r += blockDim.x) {
        double acc = 0.0;
        for (uint64_t i = blockIdx.x; i < nrows; i += gridDim.x)
            acc += (double)__fmul_rn(A[i * stride + r], B[i * stride + r]);
        part[(uint64_t)blockIdx.x * rank + r] = acc;
    }
}

// inner = sum_r (sum over blocks) * lambda[r] (ktensor.c:238-241).
__global__ void k_rowdot_final(const double *__restrict__ part, int nb, int rank, const float *__restrict__ lambda,
                               double *__restrict__ out) {
    if (threadIdx.x != 0) return;
    double inner = 0.0;
    for (int r = 0; r < rank; ++r) {
        double acc = 0.0;
        for (int b = 0; b < nb; ++b) acc += part[(uint64_t)b * rank + r];
        inner += acc * (double)lambda[r];
    }
    *out = inner;
}

int rows_blocks(uint32_t nrows) {
    uint32_t nb = nrows < (uint32_t)NBLK ? nrows : (uint32_t)NBLK;
    return nb ? (int)nb : 1;
}

}  // namespace

extern "C" cudaError_t sptgb_hadamard_upper(const float *const *mats, int nmodes, int mode, int rank, int stride,
                                            float *out, cudaStream_t s) {
    if (nmodes < 1 || nmodes > SPTGB_MAX_MODES || rank < 1) return cudaErrorInvalidValue;
    F32Ptrs p;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) p.p[m] = m < nmodes ? mats[m] : nullptr;
    k_hadamard_upper<<<(rank * rank + 255) / 256, 256, 0, s>>>(p, nmodes, mode, rank, stride, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_grams_upper_f64(const float *const *mats, int nmodes, int rank, int stride, double *out,
                                             cudaStream_t s) {
    if (nmodes < 1 || nmodes > SPTGB_MAX_MODES || rank < 1) return cudaErrorInvalidValue;
    F32Ptrs p;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) p.p[m] = m < nmodes ? mats[m] : nullptr;
    k_grams_upper_f64<<<(nmodes * rank * rank + 255) / 256, 256, 0, s>>>(p, nmodes, rank, stride, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_kruskal_normsq(const float *const *ata, int nmodes, int rank, int stride,
                                            const float *lambda, float *tmp, double *out, cudaStream_t s) {
    if (nmodes < 1 || nmodes > SPTGB_MAX_MODES || rank < 1) return cudaErrorInvalidValue;
    F32Ptrs p;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) p.p[m] = m < nmodes ? ata[m] : nullptr;
    k_kruskal_normsq<<<1, 32, 0, s>>>(p, nmodes, rank, stride, lambda, tmp, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

// ws: at least rows_blocks(nrows) * rank floats.
extern "C" cudaError_t sptgb_colmax_scale(float *A, uint32_t nrows, int rank, int stride, float *lambda, float *ws,
                                          cudaStream_t s) {
    if (rank < 1) return cudaErrorInvalidValue;
    const int nb = rows_blocks(nrows);
    k_colmax_partial<<<nb, 64, 0, s>>>(A, nrows, rank, stride, ws);
    k_colmax_final<<<1, 64, 0, s>>>(ws, nb, rank, lambda);
    uint64_t total = (uint64_t)nrows * (stride / 4);
    uint64_t g = (total + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    if (g < 1) g = 1;
    k_scale_cols<<<(unsigned)g, 256, 0, s>>>(A, nrows, rank, stride, lambda);
    sptgb_count_launch(3);
    return cudaGetLastError();
}

// ws: at least rows_blocks(nrows) * rank doubles.
extern "C" cudaError_t sptgb_rowdot(const float *A, const float *B, uint32_t nrows, int rank, int stride,
                                    const float *lambda, double *out, double *ws, cudaStream_t s) {
    if (rank < 1) return cudaErrorInvalidValue;
    const int nb = rows_blocks(nrows);
    k_rowdot_partial<<<nb, 64, 0, s>>>(A, B, nrows, rank, stride, ws);
    k_rowdot_final<<<1, 32, 0, s>>>(ws, nb, rank, lambda, out);
    sptgb_count_launch(2);
    return cudaGetLastError();
}
