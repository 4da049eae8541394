// Block-level bodies of the FP64 CP-ALS kernels, shared by the single-tensor
// kernels (dense.cu) and the batched ones (batch.cu) so that both compute the
// same arithmetic.  Functions that walk row tiles take (bid, nbk): this block's
// index and the number of blocks sharing the rows.  See dense.cu for the
// reference steps each piece restates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "../sptgb_internal.h"

namespace sptgb_dense {


constexpr int DT = 256;          // threads per block
constexpr int TR = 32;           // rows per tile
constexpr int RMAX = 64;
constexpr int PMAX = RMAX * (RMAX + 1) / 2;
constexpr int PPT = (PMAX + DT - 1) / DT;   // pairs per thread (9)
constexpr int NBLK = 2 * 152;    // partial-reduction blocks

__device__ __forceinline__ void pair_of(int idx, int rank, int *p, int *q) {
    // idx enumerates (p, q), p <= q, row by row.
    int pp = 0, rem = idx;
    while (rem >= rank - pp) {
        rem -= rank - pp;
        ++pp;
    }
    *p = pp;
    *q = pp + rem;
}

// Per-block partial of A^T A over a grid-stride set of row tiles.
__device__ __forceinline__ void gram_partial_body(const float *__restrict__ A, uint32_t nrows, int rank, int stride, double *__restrict__ part, unsigned bid, unsigned nbk) {
    __shared__ double tile[TR][RMAX + 1];
    __shared__ unsigned char pp_s[PMAX], qq_s[PMAX];
    const int P = rank * (rank + 1) / 2;
    for (int i = threadIdx.x; i < P; i += DT) {
        int p, q;
        pair_of(i, rank, &p, &q);
        pp_s[i] = (unsigned char)p;
        qq_s[i] = (unsigned char)q;
    }
    double acc[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) acc[k] = 0.0;
    for (uint64_t t0 = (uint64_t)bid * TR; t0 < nrows; t0 += (uint64_t)nbk * TR) {
        __syncthreads();
        for (int e = threadIdx.x; e < TR * rank; e += DT) {
            const int r = e / rank, c = e % rank;
            const uint64_t row = t0 + r;
            tile[r][c] = row < nrows ? (double)A[row * stride + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const int i = threadIdx.x + k * DT;
            if (i < P) {
                const int p = pp_s[i], q = qq_s[i];
                double s = 0.0;
#pragma unroll 8
                for (int r = 0; r < TR; ++r) s = fma(tile[r][p], tile[r][q], s);
                acc[k] += s;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int i = threadIdx.x + k * DT;
        if (i < P) part[(uint64_t)bid * P + i] = acc[k];
    }
}

// Sums the per-block pair partials (fixed order) into a full symmetric
// rank x rank matrix G (row-major, leading dimension rank).
__device__ __forceinline__ void gram_reduce_body(const double *__restrict__ part, int nblk, int rank, double *__restrict__ G) {
    const int P = rank * (rank + 1) / 2;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(uint64_t)b * P + i];
        int p, q;
        pair_of(i, rank, &p, &q);
        G[p * rank + q] = s;
        G[q * rank + p] = s;
    }
}

// H = Hadamard of grams[(mode+k) % nmodes], k = 1..nmodes-1, then
// S = (H^{-1})^T via Cholesky (or LU with partial pivoting when H is not
// positive definite, as the reference falls back from spotrf_ to sgesv_).
struct GramPtrs { const double *g[SPTGB_MAX_MODES]; };

__device__ __forceinline__ void solve_prepare_body(GramPtrs grams, int nmodes, int mode, int rank, double *__restrict__ S,
                int *__restrict__ status) {
    extern __shared__ double sm[];
    double *H = sm;                       // [rank][rank+1]
    double *L = sm + RMAX * (RMAX + 1);   // [rank][rank+1]
    __shared__ int fail;
    __shared__ int piv[RMAX];
    const int ld = RMAX + 1;
    const int tid = threadIdx.x;
    const int RR = rank * rank;

    for (int e = tid; e < RR; e += DT) {
        const int p = e / rank, q = e % rank;
        double v = 1.0;
        for (int k = 1; k < nmodes; ++k) v *= grams.g[(mode + k) % nmodes][e];
        H[p * ld + q] = v;
        L[p * ld + q] = v;
    }
    if (tid == 0) fail = 0;
    __syncthreads();

    // Right-looking Cholesky of L (lower triangle).
    for (int k = 0; k < rank; ++k) {
        if (tid == 0) {
            const double d = L[k * ld + k];
            if (!(d > 0.0)) fail = 1;
            else L[k * ld + k] = sqrt(d);
        }
        __syncthreads();
        if (fail) break;
        const double dk = L[k * ld + k];
        for (int i = k + 1 + tid; i < rank; i += DT) L[i * ld + k] /= dk;
        __syncthreads();
        const int m = rank - k - 1;
        for (int e = tid; e < m * m; e += DT) {
            const int i = k + 1 + e / m, j = k + 1 + e % m;
            if (j <= i) L[i * ld + j] -= L[i * ld + k] * L[j * ld + k];
        }
        __syncthreads();
    }

    if (!fail) {
        // Column j of L^{-1} by forward substitution; kept in H's upper part
        // is unsafe, so reuse H entirely (H is no longer needed).
        for (int j = tid; j < rank; j += DT) {
            for (int i = 0; i < rank; ++i) H[i * ld + j] = 0.0;
            H[j * ld + j] = 1.0 / L[j * ld + j];
            for (int i = j + 1; i < rank; ++i) {
                double s = 0.0;
                for (int k = j; k < i; ++k) s += L[i * ld + k] * H[k * ld + j];
                H[i * ld + j] = -s / L[i * ld + i];
            }
        }
        __syncthreads();
        // H^{-1} = L^{-T} L^{-1}; symmetric, so S = H^{-1}.
        for (int e = tid; e < RR; e += DT) {
            const int p = e / rank, q = e % rank;
            const int k0 = p > q ? p : q;
            double s = 0.0;
            for (int k = k0; k < rank; ++k) s += H[k * ld + p] * H[k * ld + q];
            S[e] = s;
        }
        if (tid == 0) *status = 0;
        return;
    }

    // LU with partial pivoting on a fresh copy of H (kept in L).
    __syncthreads();
    for (int e = tid; e < RR; e += DT) {
        const int p = e / rank, q = e % rank;
        L[p * ld + q] = H[p * ld + q];
    }
    __shared__ int singular;
    if (tid == 0) singular = 0;
    __syncthreads();
    for (int k = 0; k < rank; ++k) {
        if (tid == 0) {
            int best = k;
            double bv = fabs(L[k * ld + k]);
            for (int i = k + 1; i < rank; ++i)
                if (fabs(L[i * ld + k]) > bv) { bv = fabs(L[i * ld + k]); best = i; }
            piv[k] = best;
            if (bv == 0.0) singular = 1;
        }
        __syncthreads();
        const int b = piv[k];
        if (b != k)
            for (int j = tid; j < rank; j += DT) {
                const double t = L[k * ld + j];
                L[k * ld + j] = L[b * ld + j];
                L[b * ld + j] = t;
            }
        __syncthreads();
        const double d = L[k * ld + k];
        if (d != 0.0)
            for (int i = k + 1 + tid; i < rank; i += DT) L[i * ld + k] /= d;
        __syncthreads();
        const int m = rank - k - 1;
        for (int e = tid; e < m * m; e += DT) {
            const int i = k + 1 + e / m, j = k + 1 + e % m;
            L[i * ld + j] -= L[i * ld + k] * L[k * ld + j];
        }
        __syncthreads();
    }
    // Inverse column by column: solve L U x = P e_j.  S = (H^{-1})^T, so
    // row j of S is column j of the inverse.
    for (int j = tid; j < rank; j += DT) {
        double x[RMAX];
        for (int i = 0; i < rank; ++i) x[i] = (i == j) ? 1.0 : 0.0;
        for (int k = 0; k < rank; ++k) {
            const int b = piv[k];
            const double t = x[k];
            x[k] = x[b];
            x[b] = t;
        }
        for (int i = 0; i < rank; ++i) {
            double s = x[i];
            for (int k = 0; k < i; ++k) s -= L[i * ld + k] * x[k];
            x[i] = s;
        }
        for (int i = rank - 1; i >= 0; --i) {
            double s = x[i];
            for (int k = i + 1; k < rank; ++k) s -= L[i * ld + k] * x[k];
            x[i] = s / L[i * ld + i];
        }
        for (int i = 0; i < rank; ++i) S[j * rank + i] = x[i];
    }
    if (tid == 0) *status = singular ? 2 : 1;
}

// X[i, :] = M[i, :] * S (S = (H^{-1})^T, so row i of X solves H x = m_i),
// computed in FP64, stored FP32; per-block partials of X^T X and of the
// column maxima of the stored values.
__device__ __forceinline__ void solve_rows_body(const float *__restrict__ M, float *__restrict__ X, uint32_t nrows, int rank, int stride,
             const double *__restrict__ S, double *__restrict__ gpart, double *__restrict__ mpart, unsigned bid, unsigned nbk) {
    extern __shared__ double sm[];
    double *Ss = sm;                        // [rank][rank]
    double *Mt = Ss + RMAX * RMAX;          // [TR][RMAX+1]
    double *Xt = Mt + TR * (RMAX + 1);      // [TR][RMAX+1]
    __shared__ unsigned char pp_s[PMAX], qq_s[PMAX];
    const int ld = RMAX + 1;
    const int P = rank * (rank + 1) / 2;
    for (int e = threadIdx.x; e < rank * rank; e += DT) Ss[e] = S[e];
    for (int i = threadIdx.x; i < P; i += DT) {
        int p, q;
        pair_of(i, rank, &p, &q);
        pp_s[i] = (unsigned char)p;
        qq_s[i] = (unsigned char)q;
    }
    double acc[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) acc[k] = 0.0;
    double cmax = 0.0;   // column maximum, starting at 0 as matrix.c:484-486
    for (uint64_t t0 = (uint64_t)bid * TR; t0 < nrows; t0 += (uint64_t)nbk * TR) {
        __syncthreads();
        for (int e = threadIdx.x; e < TR * rank; e += DT) {
            const int r = e / rank, c = e % rank;
            const uint64_t row = t0 + r;
            Mt[r * ld + c] = row < nrows ? (double)M[row * stride + c] : 0.0;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < TR * rank; e += DT) {
            const int r = e / rank, c = e % rank;
            const uint64_t row = t0 + r;
            double s = 0.0;
            for (int k = 0; k < rank; ++k) s = fma(Mt[r * ld + k], Ss[k * rank + c], s);
            const float xf = (float)s;
            Xt[r * ld + c] = row < nrows ? (double)xf : 0.0;
            if (row < nrows) X[row * stride + c] = xf;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const int i = threadIdx.x + k * DT;
            if (i < P) {
                const int p = pp_s[i], q = qq_s[i];
                double s = 0.0;
#pragma unroll 8
                for (int r = 0; r < TR; ++r) s = fma(Xt[r * ld + p], Xt[r * ld + q], s);
                acc[k] += s;
            }
        }
        if (threadIdx.x < rank) {
            for (int r = 0; r < TR; ++r)
                if (t0 + r < nrows && Xt[r * ld + threadIdx.x] > cmax) cmax = Xt[r * ld + threadIdx.x];
        }
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int i = threadIdx.x + k * DT;
        if (i < P) gpart[(uint64_t)bid * P + i] = acc[k];
    }
    if (threadIdx.x < rank) mpart[(uint64_t)bid * rank + threadIdx.x] = cmax;
}

// Reduces the solve statistics, forms lambda and the normalised Gram.
__device__ __forceinline__ void lambda_body(const double *__restrict__ gpart, const double *__restrict__ mpart, int nblk, int rank,
                         int use_2norm, double *__restrict__ G, float *__restrict__ lambda_f32,
                         double *__restrict__ colmax_out) {
    __shared__ double lam[RMAX];
    const int P = rank * (rank + 1) / 2;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += gpart[(uint64_t)b * P + i];
        int p, q;
        pair_of(i, rank, &p, &q);
        G[p * rank + q] = s;
        G[q * rank + p] = s;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < rank; j += blockDim.x) {
        double mx = 0.0;
        for (int b = 0; b < nblk; ++b) {
            const double v = mpart[(uint64_t)b * rank + j];
            if (v > mx) mx = v;
        }
        if (colmax_out) colmax_out[j] = mx;
        float l;
        if (use_2norm) {
            l = sqrtf((float)G[j * rank + j]);
        } else {
            l = (float)mx;
            if (l < 1.f) l = 1.f;
        }
        lambda_f32[j] = l;
        lam[j] = (double)l;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < rank * rank; e += blockDim.x) {
        const int p = e / rank, q = e % rank;
        G[e] = G[e] / (lam[p] * lam[q]);
    }
}

__device__ __forceinline__ void scale_cols_body(float *__restrict__ X, uint32_t nrows, int rank, int stride,
                             const float *__restrict__ lambda, unsigned bid, unsigned nbk) {
    const uint64_t total = (uint64_t)nrows * rank;
    for (uint64_t e = bid * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)nbk * blockDim.x) {
        const uint64_t i = e / rank;
        const int j = (int)(e % rank);
        X[i * stride + j] = X[i * stride + j] / lambda[j];
    }
}

// Per-block partials of sum_i A[i,r] * M[i,r].
__device__ __forceinline__ void inner_partial_body(const float *__restrict__ A, const float *__restrict__ M, uint32_t nrows, int rank, int stride,
                double *__restrict__ part, unsigned bid, unsigned nbk) {
    __shared__ double red[DT];
    // thread handles column c = tid % rank for rows strided by DT / rank
    const int per = DT / rank;
    const int c = threadIdx.x % rank;
    const int r0 = threadIdx.x / rank;
    double s = 0.0;
    if (r0 < per) {
        for (uint64_t i = (uint64_t)bid * per + r0; i < nrows; i += (uint64_t)nbk * per)
            s += (double)A[i * stride + c] * (double)M[i * stride + c];
    }
    red[threadIdx.x] = (r0 < per) ? s : 0.0;
    __syncthreads();
    if (threadIdx.x < rank) {
        double t = 0.0;
        for (int k = 0; k < per; ++k) t += red[k * rank + threadIdx.x];
        part[(uint64_t)bid * rank + threadIdx.x] = t;
    }
}

__device__ __forceinline__ void fit_final_body(const double *__restrict__ part, int nblk, int rank, const float *__restrict__ lambda,
                            GramPtrs gp, int nmodes, const double *__restrict__ normX2, double *__restrict__ fit) {
    __shared__ double red[DT];
    __shared__ double inner_s;
    double inner = 0.0;
    for (int r = threadIdx.x; r < rank; r += blockDim.x) {
        double t = 0.0;
        for (int b = 0; b < nblk; ++b) t += part[(uint64_t)b * rank + r];
        inner += t * (double)lambda[r];
    }
    red[threadIdx.x] = inner;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < blockDim.x; ++k) s += red[k];
        inner_s = s;
    }
    __syncthreads();
    double nk = 0.0;
    for (int e = threadIdx.x; e < rank * rank; e += blockDim.x) {
        const int p = e / rank, q = e % rank;
        double h = 1.0;
        for (int m = 0; m < nmodes; ++m) h *= gp.g[m][e];
        nk += h * (double)lambda[p] * (double)lambda[q];
    }
    red[threadIdx.x] = nk;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < blockDim.x; ++k) s += red[k];
        const double normK = fabs(s);
        const double nx = *normX2;
        double residual = nx + normK - 2.0 * inner_s;
        if (residual > 0.0) residual = sqrt(residual);
        *fit = 1.0 - residual / sqrt(nx);
    }
}

__device__ __forceinline__ void sumsq_partial_body(const float *__restrict__ v, uint64_t n, double *part, unsigned bid, unsigned nbk) {
    __shared__ double red[DT];
    double s = 0.0;
    for (uint64_t i = bid * (uint64_t)DT + threadIdx.x; i < n; i += (uint64_t)nbk * DT) {
        const double x = v[i];
        s += x * x;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = DT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[bid] = red[0];
}

__device__ __forceinline__ void sum_final_body(const double *part, int nblk, double *out) {
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[b];
        *out = s;
    }
}

// Column sums of squares (FP64) per block.
__device__ __forceinline__ void colsq_partial_body(const float *__restrict__ A, uint32_t nrows, int rank, int stride, double *__restrict__ part, unsigned bid, unsigned nbk) {
    __shared__ double red[DT];
    const int per = DT / rank;
    const int c = threadIdx.x % rank;
    const int r0 = threadIdx.x / rank;
    double s = 0.0;
    if (r0 < per)
        for (uint64_t i = (uint64_t)bid * per + r0; i < nrows; i += (uint64_t)nbk * per) {
            const double x = A[i * stride + c];
            s += x * x;
        }
    red[threadIdx.x] = (r0 < per) ? s : 0.0;
    __syncthreads();
    if (threadIdx.x < rank) {
        double t = 0.0;
        for (int k = 0; k < per; ++k) t += red[k * rank + threadIdx.x];
        part[(uint64_t)bid * rank + threadIdx.x] = t;
    }
}

__device__ __forceinline__ void colnorm_final_body(const double *part, int nblk, int rank, float *lambda_mul, float *norms) {
    for (int r = threadIdx.x; r < rank; r += blockDim.x) {
        double t = 0.0;
        for (int b = 0; b < nblk; ++b) t += part[(uint64_t)b * rank + r];
        const float nrm = sqrtf((float)t);
        norms[r] = nrm;
        lambda_mul[r] = lambda_mul[r] * nrm;
    }
}

__device__ __forceinline__ void f32_to_bf16_body(const float *__restrict__ in, uint16_t *__restrict__ out, uint64_t n, unsigned bid, unsigned nbk) {
    for (uint64_t i = bid * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)nbk * blockDim.x) {
        // round to nearest even
        uint32_t u = __float_as_uint(in[i]);
        if ((u & 0x7f800000u) == 0x7f800000u) {
            out[i] = (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
        } else {
            u += 0x7fffu + ((u >> 16) & 1u);
            out[i] = (uint16_t)(u >> 16);
        }
    }
}

__host__ __device__ inline int nblocks_for_rows(uint64_t nrows) {
    uint64_t b = (nrows + TR - 1) / TR;
    if (b > (uint64_t)NBLK) b = NBLK;
    if (b < 1) b = 1;
    return (int)b;
}

constexpr size_t SOLVE_SMEM = (size_t)(RMAX * RMAX + 2 * TR * (RMAX + 1)) * sizeof(double);
constexpr size_t PREP_SMEM = (size_t)(2 * RMAX * (RMAX + 1)) * sizeof(double);


}  // namespace sptgb_dense
