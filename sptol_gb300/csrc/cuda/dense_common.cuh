// Block-level bodies of the FP64 / double-float CP-ALS kernels, shared by the single-tensor
// kernels (dense.cu) and the batched ones (batch.cu) so that both compute the
// same arithmetic.  Functions that walk row tiles take (bid, nbk): this block's
// index and the number of blocks sharing the rows.  See dense.cu for the
// reference steps each piece restates.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "../sptgb_internal.h"

// Pointer qualifier of the bodies' operands.  A unit whose kernels only read
// data written by earlier launches keeps __restrict__ (const operands may then
// take the read-only load path); the persistent batched step (batch_step.cu),
// whose phases read what earlier phases of the same launch wrote, defines it
// empty before including this file.  Each .cu is its own device module (no
// relocatable device code), so the two forms never meet.
#ifndef SPTGB_RESTRICT
#define SPTGB_RESTRICT __restrict__
#endif

namespace sptgb_dense {


constexpr int DT = 256;          // threads per block
constexpr int TR = 32;           // rows per tile
constexpr int RMAX = 64;
constexpr int PMAX = RMAX * (RMAX + 1) / 2;
constexpr int PPT = (PMAX + DT - 1) / DT;   // pairs per thread (9)
constexpr int NBLK = SPTGB_NPART;   // partial-reduction blocks (fixed, device-independent)

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
__device__ __forceinline__ void gram_partial_body(const float *SPTGB_RESTRICT A, uint32_t nrows, int rank, int stride, double *SPTGB_RESTRICT part, unsigned bid, unsigned nbk) {
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
__device__ __forceinline__ void gram_reduce_body(const double *SPTGB_RESTRICT part, int nblk, int rank, double *SPTGB_RESTRICT G) {
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

// Rewrites the FP64 inverse S[0, RR) in place as two FP32 arrays, hi then
// lo (hi = fl32(S), lo = fl32(S - hi)), the operand form of the double-float
// row solve.  The buffer holds RR doubles = 2 RR floats.
__device__ __forceinline__ void split_inverse(double *S, int RR) {
    constexpr int PER = (RMAX * RMAX + DT - 1) / DT;
    double v[PER];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + i * DT;
        v[i] = e < RR ? S[e] : 0.0;
    }
    __syncthreads();
    float *Sf = reinterpret_cast<float *>(S);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int e = threadIdx.x + i * DT;
        if (e < RR) {
            const float h = (float)v[i];
            Sf[e] = h;
            Sf[RR + e] = (float)(v[i] - (double)h);
        }
    }
}

// Status word of a prepared solve: bits 0-7 the factorisation (0 Cholesky,
// 1 LU, 2 LU with a zero pivot), bits 8 and up the exponent e >= 0 of the
// power of two the inverse was divided by.  An ill-conditioned H has an
// inverse far larger than its rows' solutions; the FP32 words of the
// double-float solve (and the FP32 products of the new Gram) would overflow
// on it, so an inverse whose largest entry exceeds 2^32 is scaled by 2^-e
// (exact) and the solve scales its results back by 2^e in the precision each
// is kept in.
constexpr double INV_SCALE_ABOVE = 4294967296.0;   // 2^32
__device__ __forceinline__ int inverse_exponent(int status) { return status >> 8; }

__device__ __forceinline__ void finish_inverse(double *S, int RR, int *status, int kind) {
    __shared__ double red[DT / 32];
    __shared__ int e_s;
    __syncthreads();
    double m = 0.0;
    for (int i = threadIdx.x; i < RR; i += DT) m = fmax(m, fabs(S[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < DT / 32; ++w) t = fmax(t, red[w]);
        e_s = (t > INV_SCALE_ABOVE && t <= 1.7e308) ? ilogb(t) : 0;
        *status = kind | (e_s << 8);
    }
    __syncthreads();
    const int e = e_s;
    if (e)
        for (int i = threadIdx.x; i < RR; i += DT) S[i] = ldexp(S[i], -e);
    split_inverse(S, RR);
}

__device__ __forceinline__ void solve_prepare_body(GramPtrs grams, int nmodes, int mode, int rank, double *SPTGB_RESTRICT S,
                int *SPTGB_RESTRICT status) {
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
        finish_inverse(S, RR, status, 0);
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
    // An exactly zero pivot: LAPACK's sgesv (the reference's fallback,
    // matrix_solver.c:66-80) stops after the factorisation and leaves the
    // right-hand sides unsolved, so the rows stay the MTTKRP output: S = I.
    if (singular) {
        for (int e = tid; e < RR; e += DT) S[e] = (e / rank == e % rank) ? 1.0 : 0.0;
        finish_inverse(S, RR, status, 2);
        return;
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
    finish_inverse(S, RR, status, 1);
}

// X[i, :] = M[i, :] * S (S = (H^{-1})^T, so row i of X solves H x = m_i).
// Double-float arithmetic (a value is hi + lo, two FP32 numbers, about 48
// significant bits): the row-wise contractions of the solve run on the FP32
// pipes, which on this GPU issue 64 times the FP64 rate.  Products of FP32
// inputs are exact as (p, fma(a, b, -p)); sums use Knuth's TwoSum, so the only
// rounding is in the low word.  Explicit _rn intrinsics keep the compiler from
// contracting or reassociating the error terms.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// (hi, lo) += m * (shi + slo)
__device__ __forceinline__ void df_fma(float &hi, float &lo, float m, float shi, float slo) {
    const float p = __fmul_rn(m, shi);
    const float pe = __fmaf_rn(m, shi, -p);
    float t, e;
    two_sum(hi, p, t, e);
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(e, __fmaf_rn(m, slo, pe)));
}

// (hi, lo) += a * b, exactly up to the low word's rounding
__device__ __forceinline__ void df_prod_acc(float &hi, float &lo, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    float t, e;
    two_sum(hi, p, t, e);
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
}

__device__ __forceinline__ void df_renorm(float &hi, float &lo) {
    const float t = __fadd_rn(hi, lo);
    lo = __fsub_rn(lo, __fsub_rn(t, hi));
    hi = t;
}

// Packed double-float: two independent double-float values in the x and y
// lanes of float2 registers, advanced by the FP32x2 instructions (one
// instruction per pair).  Same operation order as the scalar forms above.
namespace df2 {
__device__ __forceinline__ uint64_t u(float2 a) { return *reinterpret_cast<uint64_t *>(&a); }
__device__ __forceinline__ float2 f(uint64_t a) { return *reinterpret_cast<float2 *>(&a); }
__device__ __forceinline__ float2 add(float2 a, float2 b) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(u(a)), "l"(u(b)));
    return f(r);
}
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(u(a)), "l"(u(b)));
    return f(r);
}
__device__ __forceinline__ float2 mul(float2 a, float2 b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(u(a)), "l"(u(b)));
    return f(r);
}
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(u(a)), "l"(u(b)), "l"(u(c)));
    return f(r);
}
// (hi, lo) += m * (sh + sl); sn = -sh
__device__ __forceinline__ void fma_acc(float2 &hi, float2 &lo, float2 m, float2 sh, float2 sn, float2 sl) {
    const float2 p = mul(m, sh);
    const float2 npe = fma(m, sn, p);   // p - m*sh exactly: minus the product's rounding error
    const float2 t = add(hi, p);
    const float2 bp = sub(t, hi);
    const float2 ap = sub(t, bp);
    const float2 e = add(sub(hi, ap), sub(p, bp));
    lo = add(lo, fma(m, sl, sub(e, npe)));
    hi = t;
}
// (hi, lo) += a * b; nb = -b
__device__ __forceinline__ void prod_acc(float2 &hi, float2 &lo, float2 a, float2 b, float2 nb) {
    const float2 p = mul(a, b);
    const float2 npe = fma(a, nb, p);
    const float2 t = add(hi, p);
    const float2 bp = sub(t, hi);
    const float2 ap = sub(t, bp);
    const float2 e = add(sub(hi, ap), sub(p, bp));
    lo = add(lo, sub(e, npe));
    hi = t;
}
__device__ __forceinline__ void renorm(float2 &hi, float2 &lo) {
    const float2 t = add(hi, lo);
    lo = sub(lo, sub(t, hi));
    hi = t;
}
// the two lanes' double-float values added: (hi, lo) scalar
__device__ __forceinline__ void fold(float2 hi, float2 lo, float &h, float &l) {
    float e;
    two_sum(hi.x, hi.y, h, e);
    l = __fadd_rn(__fadd_rn(lo.x, lo.y), e);
}
}  // namespace df2

constexpr int LDK = RMAX + 2;   // row length of the k-major tiles at rank RMAX (even: 8-byte pairs)
constexpr int LDR = TR + 2;     // row length of the transposed X tile at rank RMAX

// Rows per tile of the row solve: 32 x (64 / the rank's power-of-two class),
// so that a tile holds about 2,048 outputs (8 per thread) at every rank and
// the per-tile barriers and Gram loop are paid per 2,048 outputs, not per 256
// at rank 8.  The shared-memory layout ([rank][rank2 + 2] for S, [2][tiles]
// of M, [rank][rows + 2] for X) stays within the rank-64 layout.
__host__ __device__ inline int solve_tile_rows(int rank) {
    return rank <= 8 ? 256 : rank <= 16 ? 128 : rank <= 32 ? 64 : 32;
}

// One tile of X = M * S for a thread that owns column c0 of rows
// r0 + j * rstep, j < NOUT; the k sum runs over pairs (k, k+1) in the two
// lanes, which are added at the end.
template <int NOUT>
__device__ __forceinline__ void solve_tile_cols(const float *SPTGB_RESTRICT Mt, const float *SPTGB_RESTRICT StH,
                                                const float *SPTGB_RESTRICT StN, const float *SPTGB_RESTRICT StL,
                                                float *SPTGB_RESTRICT XT, float *SPTGB_RESTRICT XN, float *SPTGB_RESTRICT X,
                                                uint64_t t0, uint32_t nrows, int rank2, int stride, int c0, int r0,
                                                int rstep, int sexp, int ldk, int ldr) {
    float2 hi[NOUT], lo[NOUT];
#pragma unroll
    for (int j = 0; j < NOUT; ++j) hi[j] = lo[j] = make_float2(0.f, 0.f);
    const float *sh_p = StH + c0 * ldk, *sn_p = StN + c0 * ldk, *sl_p = StL + c0 * ldk;
#pragma unroll 2
    for (int k = 0; k < rank2; k += 2) {
        const float2 sh = *reinterpret_cast<const float2 *>(sh_p + k);
        const float2 sn = *reinterpret_cast<const float2 *>(sn_p + k);
        const float2 sl = *reinterpret_cast<const float2 *>(sl_p + k);
#pragma unroll
        for (int j = 0; j < NOUT; ++j)
            df2::fma_acc(hi[j], lo[j], *reinterpret_cast<const float2 *>(Mt + (r0 + j * rstep) * ldk + k), sh, sn, sl);
    }
#pragma unroll
    for (int j = 0; j < NOUT; ++j) {
        float h, l;
        df2::fold(hi[j], lo[j], h, l);
        const int r = r0 + j * rstep;
        const uint64_t row = t0 + r;
        const float xf = row < nrows ? __fadd_rn(h, l) : 0.f;
        XT[c0 * ldr + r] = xf;   // the Gram and the column maxima use the scaled values
        XN[c0 * ldr + r] = -xf;
        if (row < nrows) X[row * stride + c0] = sexp ? scalbnf(xf, sexp) : xf;
    }
}

// X = M * S over a grid-stride set of row tiles (S = H^{-1} from
// solve_prepare_body, as hi and lo FP32 arrays), plus this block's partial of
// X^T X (over the FP32 values written) and the column maxima.  Each output
// element and each Gram entry is accumulated in double-float (packed FP32x2)
// and rounded once: outputs to FP32, Gram partials to FP64.  TRC: rows per
// tile (solve_tile_rows of the rank), fixed per instantiation with the
// layout of its rank class RC = 64 * 32 / TRC.
template <int TRC>
__device__ __forceinline__ void solve_rows_tiles(const float *SPTGB_RESTRICT M, float *SPTGB_RESTRICT X, uint32_t nrows, int rank, int stride,
             const double *SPTGB_RESTRICT S, const int *SPTGB_RESTRICT sstatus, double *SPTGB_RESTRICT gpart,
             double *SPTGB_RESTRICT mpart, unsigned bid, unsigned nbk) {
    constexpr int RC = RMAX * TR / TRC;     // largest rank of the class
    constexpr int tr = TRC;                 // rows per tile
    constexpr int ldk = RC + 2;             // row length of the k-major tiles (even: 8-byte pairs)
    constexpr int ldr = TRC + 2;            // row length of the transposed X tile
    const int sexp = inverse_exponent(*sstatus);
    const int P = rank * (rank + 1) / 2;
    const int RR = rank * rank;
    const int rank2 = (rank + 1) & ~1;
    extern __shared__ float smf[];
    float *StH = smf;                       // [RC][ldk]: S^T hi, k-major per column
    float *StN = StH + RC * ldk;            // -hi
    float *StL = StN + RC * ldk;            // lo
    float *Mt2 = StL + RC * ldk;            // [2][tr][ldk]: row tiles of M, double-buffered
    float *XT = Mt2 + 2 * tr * ldk;         // [RC][ldr]: tile of X, transposed
    float *XN = XT + RC * ldr;              // -XT
    __shared__ unsigned char pp_s[PMAX], qq_s[PMAX];
    // TR x rank2 floats of M from row t0 into dst as 8-byte cp.async chunks,
    // one commit group; rows past nrows and columns past rank read as zero
    // (source size 0 or 4 of the 8 bytes)
    auto load_tile = [&](float *dst, uint64_t t0) {
        const int half = rank2 / 2;
        for (int e = threadIdx.x; e < tr * half; e += DT) {
            const int r = e / half, c = 2 * (e % half);
            const uint64_t row = t0 + r;
            const unsigned bytes = row < nrows ? (c + 1 < rank ? 8u : (c < rank ? 4u : 0u)) : 0u;
            const float *src = bytes ? M + row * stride + c : M;
            const unsigned dst_s = (unsigned)__cvta_generic_to_shared(dst + r * ldk + c);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst_s), "l"(src), "r"(bytes) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    int cur = 0;
    if ((uint64_t)bid * tr < nrows) load_tile(Mt2, (uint64_t)bid * tr);
    const float *Sf = reinterpret_cast<const float *>(S);
    for (int e = threadIdx.x; e < rank * rank2; e += DT) {
        const int c = e / rank2, k = e % rank2;   // S[k][c]
        const float h = k < rank ? Sf[k * rank + c] : 0.f;
        StH[c * ldk + k] = h;
        StN[c * ldk + k] = -h;
        StL[c * ldk + k] = k < rank ? Sf[RR + k * rank + c] : 0.f;
    }
    for (int i = threadIdx.x; i < P; i += DT) {
        int p, q;
        pair_of(i, rank, &p, &q);
        pp_s[i] = (unsigned char)p;
        qq_s[i] = (unsigned char)q;
    }
    float2 ghi[PPT], glo[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) ghi[k] = glo[k] = make_float2(0.f, 0.f);
    float cmax = 0.f;   // column maximum, starting at 0 as matrix.c:484-486
    // with rank | DT a thread keeps one column c0 and rows r0 + j * (DT / rank)
    const bool fixed_col = (DT % rank) == 0;
    const int c0 = threadIdx.x % rank, r0 = threadIdx.x / rank, rstep = DT / rank;
    const int nout = (tr * rank + DT - 1) / DT;   // 1, 2, 4 or 8 when fixed_col
    for (uint64_t t0 = (uint64_t)bid * tr; t0 < nrows; t0 += (uint64_t)nbk * tr) {
        // the next tile streams into the other buffer while this one is used;
        // that buffer was last read before the previous iteration's barrier
        const float *Mt = Mt2 + cur * tr * ldk;
        if (t0 + (uint64_t)nbk * tr < nrows) {
            load_tile(Mt2 + (cur ^ 1) * tr * ldk, t0 + (uint64_t)nbk * tr);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        cur ^= 1;
        __syncthreads();
        if (fixed_col) {
            if (r0 < tr) {
                switch (nout) {
                    case 8: solve_tile_cols<8>(Mt, StH, StN, StL, XT, XN, X, t0, nrows, rank2, stride, c0, r0, rstep, sexp, ldk, ldr); break;
                    case 4: solve_tile_cols<4>(Mt, StH, StN, StL, XT, XN, X, t0, nrows, rank2, stride, c0, r0, rstep, sexp, ldk, ldr); break;
                    case 2: solve_tile_cols<2>(Mt, StH, StN, StL, XT, XN, X, t0, nrows, rank2, stride, c0, r0, rstep, sexp, ldk, ldr); break;
                    default: solve_tile_cols<1>(Mt, StH, StN, StL, XT, XN, X, t0, nrows, rank2, stride, c0, r0, rstep, sexp, ldk, ldr); break;
                }
            }
        } else {
            for (int e = threadIdx.x; e < tr * rank; e += DT)
                solve_tile_cols<1>(Mt, StH, StN, StL, XT, XN, X, t0, nrows, rank2, stride, e % rank, e / rank, 0,
                                   sexp, ldk, ldr);
        }
        __syncthreads();
        // Gram partial: this thread's pairs over row pairs (r, r+1)
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const int i = threadIdx.x + k * DT;
            if (i < P) {
                const float *xp = XT + pp_s[i] * ldr, *xq = XT + qq_s[i] * ldr, *nq = XN + qq_s[i] * ldr;
#pragma unroll 4
                for (int r = 0; r < tr; r += 2)
                    df2::prod_acc(ghi[k], glo[k], *reinterpret_cast<const float2 *>(xp + r),
                                  *reinterpret_cast<const float2 *>(xq + r), *reinterpret_cast<const float2 *>(nq + r));
                df2::renorm(ghi[k], glo[k]);
            }
        }
        if (threadIdx.x < rank) {
            for (int r = 0; r < tr; ++r)
                if (t0 + r < nrows && XT[threadIdx.x * ldr + r] > cmax) cmax = XT[threadIdx.x * ldr + r];
        }
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int i = threadIdx.x + k * DT;
        if (i < P) {
            float h, l;
            df2::fold(ghi[k], glo[k], h, l);
            gpart[(uint64_t)bid * P + i] = ldexp((double)h + (double)l, 2 * sexp);
        }
    }
    if (threadIdx.x < rank) mpart[(uint64_t)bid * rank + threadIdx.x] = ldexp((double)cmax, sexp);
}

__device__ __forceinline__ void solve_rows_body(const float *SPTGB_RESTRICT M, float *SPTGB_RESTRICT X, uint32_t nrows, int rank, int stride,
             const double *SPTGB_RESTRICT S, const int *SPTGB_RESTRICT sstatus, double *SPTGB_RESTRICT gpart,
             double *SPTGB_RESTRICT mpart, unsigned bid, unsigned nbk) {
    switch (solve_tile_rows(rank)) {
        case 256: solve_rows_tiles<256>(M, X, nrows, rank, stride, S, sstatus, gpart, mpart, bid, nbk); break;
        case 128: solve_rows_tiles<128>(M, X, nrows, rank, stride, S, sstatus, gpart, mpart, bid, nbk); break;
        case 64: solve_rows_tiles<64>(M, X, nrows, rank, stride, S, sstatus, gpart, mpart, bid, nbk); break;
        default: solve_rows_tiles<32>(M, X, nrows, rank, stride, S, sstatus, gpart, mpart, bid, nbk); break;
    }
}

// Reduces the solve statistics, forms lambda and the normalised Gram.
__device__ __forceinline__ void lambda_body(const double *SPTGB_RESTRICT gpart, const double *SPTGB_RESTRICT mpart, int nblk, int rank,
                         int use_2norm, double *SPTGB_RESTRICT G, float *SPTGB_RESTRICT lambda_f32,
                         double *SPTGB_RESTRICT colmax_out) {
    __shared__ double lam[RMAX];
    const int P = rank * (rank + 1) / 2;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        // four independent running sums (blocks b = 0, 1, 2, 3 mod 4) keep
        // several loads and FP64 adds in flight; combined in a fixed order
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int b = 0;
        for (; b + 4 <= nblk; b += 4) {
            s0 += gpart[(uint64_t)(b + 0) * P + i];
            s1 += gpart[(uint64_t)(b + 1) * P + i];
            s2 += gpart[(uint64_t)(b + 2) * P + i];
            s3 += gpart[(uint64_t)(b + 3) * P + i];
        }
        for (; b < nblk; ++b) s0 += gpart[(uint64_t)b * P + i];
        const double s = (s0 + s1) + (s2 + s3);
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

// X[i, j] /= lambda[j] for j < rank (padding columns untouched), one float4
// of a row per thread: rows are stride floats, so float4 e of the matrix is
// row e / (stride/4), columns 4 * (e % (stride/4)) + 0..3.
__device__ __forceinline__ void scale_cols_body(float *SPTGB_RESTRICT X, uint32_t nrows, int rank, int stride,
                             const float *SPTGB_RESTRICT lambda, unsigned bid, unsigned nbk) {
    const uint32_t c4n = (uint32_t)stride / 4;
    const uint64_t total = (uint64_t)nrows * c4n;
    float4 *X4 = reinterpret_cast<float4 *>(X);
    for (uint64_t e = bid * (uint64_t)blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)nbk * blockDim.x) {
        const int j = (int)((uint32_t)(e % c4n) * 4);
        if (j >= rank) continue;
        float4 v = X4[e];
        v.x = v.x / lambda[j];
        if (j + 1 < rank) v.y = v.y / lambda[j + 1];
        if (j + 2 < rank) v.z = v.z / lambda[j + 2];
        if (j + 3 < rank) v.w = v.w / lambda[j + 3];
        X4[e] = v;
    }
}

// Per-block partials of sum_i A[i,r] * M[i,r].
__device__ __forceinline__ void inner_partial_body(const float *SPTGB_RESTRICT A, const float *SPTGB_RESTRICT M, uint32_t nrows, int rank, int stride,
                double *SPTGB_RESTRICT part, unsigned bid, unsigned nbk) {
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

__device__ __forceinline__ void fit_final_body(const double *SPTGB_RESTRICT part, int nblk, int rank, const float *SPTGB_RESTRICT lambda,
                            GramPtrs gp, int nmodes, const double *SPTGB_RESTRICT normX2, double *SPTGB_RESTRICT fit) {
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

__device__ __forceinline__ void sumsq_partial_body(const float *SPTGB_RESTRICT v, uint64_t n, double *part, unsigned bid, unsigned nbk) {
    __shared__ double red[DT];
    double s = 0.0;
    // vals[n] * vals[n] rounded in FP32 and summed in FP64, as the reference's
    // SparseTensorFrobeniusNormSquared (src/sptensor/sptensor.c:96-107) does
    for (uint64_t i = bid * (uint64_t)DT + threadIdx.x; i < n; i += (uint64_t)nbk * DT) {
        const float x = v[i];
        s += (double)__fmul_rn(x, x);
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
__device__ __forceinline__ void colsq_partial_body(const float *SPTGB_RESTRICT A, uint32_t nrows, int rank, int stride, double *SPTGB_RESTRICT part, unsigned bid, unsigned nbk) {
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

__device__ __forceinline__ void f32_to_bf16_body(const float *SPTGB_RESTRICT in, uint16_t *SPTGB_RESTRICT out, uint64_t n, unsigned bid, unsigned nbk) {
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

// Blocks of the row solve for nrows rows (the partials sptgb_normalize reduces).
__host__ __device__ inline int nblocks_for_solve(uint64_t nrows, int rank) {
    const int tr = solve_tile_rows(rank);
    uint64_t b = (nrows + tr - 1) / tr;
    if (b > (uint64_t)NBLK) b = NBLK;
    if (b < 1) b = 1;
    return (int)b;
}

__host__ __device__ inline int nblocks_for_rows(uint64_t nrows) {
    uint64_t b = (nrows + TR - 1) / TR;
    if (b > (uint64_t)NBLK) b = NBLK;
    if (b < 1) b = 1;
    return (int)b;
}

constexpr size_t SOLVE_SMEM = (size_t)(3 * RMAX * LDK + 2 * TR * LDK + 2 * RMAX * LDR) * sizeof(float);
constexpr size_t PREP_SMEM = (size_t)(2 * RMAX * (RMAX + 1)) * sizeof(double);


}  // namespace sptgb_dense
