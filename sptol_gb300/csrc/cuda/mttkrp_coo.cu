// Segmented COO MTTKRP for sm_103a.
//
// Computes, for a tensor copy sorted by the output mode,
//   out[i, :] = sum over nonzeros x with rows[x] == i of
//               vals[x] * F_1[idx_1[x], :] * ... * F_{N-1}[idx_{N-1}[x], :]
// which is sptMTTKRP (src/sptensor/mttkrp.c:39-115, the 3-D loop at
// :162-171): the product runs over mats_order[1..N-1] in that order and the
// output rows [0, I) are fully written (rows without nonzeros are zero, as the
// reference's memset leaves them).
//
// Order 3 (the hot path) runs k_mttkrp_rec: the mode-sorted copy is stored as
// 16-byte records {row, idx_a, idx_b, value}, so the W lanes of a worker get a
// nonzero with one broadcast 128-bit load; record batches are software-
// pipelined (the next batch is in flight while the current batch's factor rows
// are gathered) and the Hadamard product uses packed FP32x2 arithmetic.  The
// output is zeroed by one memset; rows inside a unit are written with plain
// stores, rows shared by neighbouring units with vector atomics.  Order 4
// runs k_mttkrp_rec4 the same way over records {row, idx_a, idx_b, idx_c}
// with the values in their own array (batches of two records).  Other orders
// run k_mttkrp_seg below.
//
// Work decomposition.  A "worker" is a group of W lanes that owns one nonzero
// at a time; lane l of the group holds columns [4l, 4l+4) of the rank
// (float4, 128-bit gathers of factor rows).  The nonzero stream is cut into
// units of `unit_len` consecutive nonzeros; a worker walks its unit in order,
// keeps the running row sum in registers and writes a row when the output
// coordinate changes.  Rows that lie entirely inside a unit get one plain
// 128-bit store; only the rows a unit shares with its neighbour units (at
// most its first and last row) are accumulated with vector atomics into rows
// that a small pre-pass zeroed.  Rows with no nonzeros are zero-filled by the
// unit whose coordinate range contains them, so every output row is written
// once.  Index and value streams are loaded cooperatively (one element per
// lane, 8 nonzeros per batch) and broadcast with shuffles; the 2*(N-1)
// factor-row gathers of a batch are all issued before the first is used.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "mttkrp_unit.cuh"

namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr int BLOCK = 256;
constexpr int BATCH = 8;

__device__ __forceinline__ float4 f4_zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ float4 load_row4(const void *base, uint32_t row, uint32_t stride, int col4, bool bf16) {
    if (!bf16) {
        const float4 *p = reinterpret_cast<const float4 *>(static_cast<const float *>(base) + (size_t)row * stride);
        return __ldg(p + col4);
    }
    const uint2 *p = reinterpret_cast<const uint2 *>(static_cast<const uint16_t *>(base) + (size_t)row * stride);
    const uint2 u = __ldg(p + col4);
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                       __uint_as_float(u.y & 0xffff0000u));
}

__device__ __forceinline__ void store_row4(float *out, uint32_t row, uint32_t stride, int col4, float4 v,
                                           bool shared) {
    float4 *p = reinterpret_cast<float4 *>(out + (size_t)row * stride) + col4;
    if (shared)
        atomicAdd(p, v);
    else
        *p = v;
}

// NP = number of product modes (N-1); 0 selects the runtime count.
template <int W, int NP, bool BF16>
__global__ void __launch_bounds__(BLOCK)
k_mttkrp_seg(sptgb_mttkrp_args a, uint32_t unit_len, uint64_t nunits) {
    constexpr int SLOTS = (BATCH + W - 1) / W;
    constexpr int MAXP = NP > 0 ? NP : (SPTGB_MAX_MODES - 1);
    const int np = NP > 0 ? NP : (int)a.nprod;
    const int lane = threadIdx.x & 31;
    const int sub = lane / W;
    const int sl = lane % W;
    const unsigned smask = (W == 32) ? 0xffffffffu : (((1u << W) - 1u) << (sub * W));
    const uint64_t worker = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BLOCK) / W;
    const bool col_ok = (uint32_t)(sl * 4) < a.stride;
    const int c0 = sl * 4;
    // Columns at or past the rank are padding: never added (padding of the
    // factors may hold anything, including NaN), so those outputs stay 0.
    const bool m0 = c0 + 0 < (int)a.rank, m1 = c0 + 1 < (int)a.rank;
    const bool m2 = c0 + 2 < (int)a.rank, m3 = c0 + 3 < (int)a.rank;
    const uint32_t *__restrict__ rows = a.rows;
    const float *__restrict__ vals = a.vals;

    for (uint64_t u = worker; u < nunits; u += nworkers) {
        const uint64_t start = u * unit_len;
        const uint64_t end = min(start + unit_len, a.nnz);
        const uint32_t prev = start > 0 ? rows[start - 1] : NONE;
        const uint32_t next = end < a.nnz ? rows[end] : NONE;
        uint32_t cur = rows[start];
        if (col_ok) {
            for (uint32_t r = (start == 0 ? 0u : prev + 1u); r < cur; ++r)
                store_row4(a.out, r, a.stride, sl, f4_zero(), false);
        }
        float4 acc = f4_zero();
        for (uint64_t k0 = start; k0 < end; k0 += BATCH) {
            uint32_t lr[SLOTS];
            float lv[SLOTS];
            uint32_t li[MAXP][SLOTS];
#pragma unroll
            for (int s = 0; s < SLOTS; ++s) {
                const int j = s * W + sl;
                const uint64_t kk = k0 + j;
                const bool ok = j < BATCH && kk < end;
                lr[s] = ok ? rows[kk] : NONE;
                lv[s] = ok ? vals[kk] : 0.f;
#pragma unroll
                for (int p = 0; p < MAXP; ++p)
                    li[p][s] = (ok && p < np) ? a.idx[p][kk] : 0u;
            }
            uint32_t r[BATCH];
            float v[BATCH];
            float4 f[MAXP][BATCH];
#pragma unroll
            for (int j = 0; j < BATCH; ++j) {
                r[j] = __shfl_sync(smask, lr[j / W], j % W, W);
                v[j] = __shfl_sync(smask, lv[j / W], j % W, W);
#pragma unroll
                for (int p = 0; p < MAXP; ++p) {
                    const uint32_t ii = __shfl_sync(smask, li[p][j / W], j % W, W);
                    f[p][j] = (p < np && r[j] != NONE && col_ok) ? load_row4(a.fac[p], ii, a.stride, sl, BF16)
                                                                 : f4_zero();
                }
            }
#pragma unroll
            for (int j = 0; j < BATCH; ++j) {
                if (r[j] == NONE) break;
                float4 pr = make_float4(v[j] * f[0][j].x, v[j] * f[0][j].y, v[j] * f[0][j].z, v[j] * f[0][j].w);
#pragma unroll
                for (int p = 1; p < MAXP; ++p) {
                    if (p < np) {
                        pr.x *= f[p][j].x;
                        pr.y *= f[p][j].y;
                        pr.z *= f[p][j].z;
                        pr.w *= f[p][j].w;
                    }
                }
                if (r[j] != cur) {
                    if (col_ok) {
                        store_row4(a.out, cur, a.stride, sl, acc, cur == prev);
                        for (uint32_t z = cur + 1; z < r[j]; ++z)
                            store_row4(a.out, z, a.stride, sl, f4_zero(), false);
                    }
                    cur = r[j];
                    acc = f4_zero();
                }
                if (m0) acc.x += pr.x;
                if (m1) acc.y += pr.y;
                if (m2) acc.z += pr.z;
                if (m3) acc.w += pr.w;
            }
        }
        if (col_ok) {
            store_row4(a.out, cur, a.stride, sl, acc, cur == prev || cur == next);
            if (end == a.nnz)
                for (uint32_t z = cur + 1; z < a.out_rows; ++z)
                    store_row4(a.out, z, a.stride, sl, f4_zero(), false);
        }
    }
}

// Order-3 record kernel (see the header comment): one work unit per worker,
// the unit body is shared with the batched kernel (mttkrp_unit.cuh).
// FULL: the stride is exactly 4*W floats, so every lane owns real columns.
template <int W, bool BF16, bool FULL>
__global__ void __launch_bounds__(BLOCK, 3)
k_mttkrp_rec(const uint4 *__restrict__ rec, const void *__restrict__ Fa, const void *__restrict__ Fb,
             float *__restrict__ out, uint64_t nnz, uint32_t stride, uint32_t rank, uint32_t ul, uint64_t u0,
             uint64_t nunits) {
    const int sl = (threadIdx.x & 31) % W;
    const uint32_t elem = BF16 ? 2u : 4u;
    const char *F[2] = {static_cast<const char *>(Fa) + (size_t)sl * 4 * elem,
                        static_cast<const char *>(Fb) + (size_t)sl * 4 * elem};
    const uint64_t worker = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BLOCK) / W;
    for (uint64_t u = u0 + worker; u < nunits; u += nworkers) {
        const uint64_t start = u * ul;
        const uint32_t len = (uint32_t)min((uint64_t)ul, nnz - start);
        sptgb_mttkrp::unit<BF16, FULL, 2>(rec, nullptr, F, stride * elem, out, nnz, start, len, stride, rank, sl);
    }
}

// Order-4 record kernel: records {row, a, b, c} with the values in `vals`
// (same order), batches of NB records; otherwise as k_mttkrp_rec.
template <int W, bool BF16, bool FULL, int NB>
__global__ void __launch_bounds__(BLOCK, 3)
k_mttkrp_rec4(const uint4 *__restrict__ rec, const float *__restrict__ vals, const void *__restrict__ Fa,
              const void *__restrict__ Fb, const void *__restrict__ Fc, float *__restrict__ out, uint64_t nnz,
              uint32_t stride, uint32_t rank, uint32_t ul, uint64_t u0, uint64_t nunits) {
    const int sl = (threadIdx.x & 31) % W;
    const uint32_t elem = BF16 ? 2u : 4u;
    const size_t off = (size_t)sl * 4 * elem;
    const char *F[3] = {static_cast<const char *>(Fa) + off, static_cast<const char *>(Fb) + off,
                        static_cast<const char *>(Fc) + off};
    const uint64_t worker = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BLOCK) / W;
    for (uint64_t u = u0 + worker; u < nunits; u += nworkers) {
        const uint64_t start = u * ul;
        const uint32_t len = (uint32_t)min((uint64_t)ul, nnz - start);
        sptgb_mttkrp::unit<BF16, FULL, 3, NB>(rec, vals, F, stride * elem, out, nnz, start, len, stride, rank, sl);
    }
}

__global__ void k_pack_records(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ ia,
                               const uint32_t *__restrict__ ib, const float *__restrict__ vals, uint32_t lim_a,
                               uint32_t lim_b, unsigned int *__restrict__ bad, uint4 *__restrict__ rec, uint64_t n) {
    unsigned int b = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = ia[i], c = ib[i];
        const bool ok = a < lim_a && c < lim_b;
        b |= !ok;
        rec[i] = make_uint4(rows[i], ok ? a : 0u, ok ? c : 0u, __float_as_uint(vals[i]));
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0 && bad) atomicOr(bad, 1u);
}

// Order-4 records {rows, ia, ib, ic}; out-of-range ia / ib / ic as in
// k_pack_records.
__global__ void k_pack_records4(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ ia,
                                const uint32_t *__restrict__ ib, const uint32_t *__restrict__ ic, uint32_t lim_a,
                                uint32_t lim_b, uint32_t lim_c, unsigned int *__restrict__ bad,
                                uint4 *__restrict__ rec, uint64_t n) {
    unsigned int b = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = ia[i], y = ib[i], z = ic[i];
        const bool ok = x < lim_a && y < lim_b && z < lim_c;
        b |= !ok;
        rec[i] = make_uint4(rows[i], ok ? x : 0u, ok ? y : 0u, ok ? z : 0u);
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0 && bad) atomicOr(bad, 1u);
}

// Zero every row that two neighbouring units share, before the main kernel
// accumulates into it with atomics.
__global__ void k_zero_shared(const uint32_t *__restrict__ rows, uint64_t nnz, uint32_t unit_len, uint64_t nunits,
                              float *__restrict__ out, uint32_t stride) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x + 1; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = u * unit_len;
        if (s < nnz && rows[s - 1] == rows[s]) {
            float4 *p = reinterpret_cast<float4 *>(out + (size_t)rows[s] * stride);
            for (uint32_t c = 0; c < stride / 4; ++c) p[c] = f4_zero();
        }
    }
}

template <int W, int NP, bool BF16>
cudaError_t launch(const sptgb_mttkrp_args &a, cudaStream_t s) {
    // once per process (function-local statics are initialised by one thread
    // while the others wait)
    static const int per_sm = [] {
        int p = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_mttkrp_seg<W, NP, BF16>, BLOCK, 0);
        return p < 1 ? 1 : p;
    }();
    const int nsm = sptgb_sm_count();
    const int max_blocks = per_sm * nsm;
    const uint64_t workers_per_block = BLOCK / W;
    const uint64_t concurrent = workers_per_block * (uint64_t)max_blocks;
    // Units: about four per concurrent worker, between 64 and 4096 nonzeros.
    uint64_t ul = a.nnz / (4 * concurrent);
    if (ul < 64) ul = 64;
    if (ul > 4096) ul = 4096;
    ul = (ul + BATCH - 1) / BATCH * BATCH;
    const uint64_t nunits = (a.nnz + ul - 1) / ul;
    uint64_t blocks = (nunits + workers_per_block - 1) / workers_per_block;
    if (blocks > (uint64_t)max_blocks) blocks = max_blocks;
    if (nunits > 1) {
        uint64_t zb = (nunits + 255) / 256;
        if (zb > (uint64_t)nsm * 8) zb = (uint64_t)nsm * 8;
        k_zero_shared<<<(unsigned)zb, 256, 0, s>>>(a.rows, a.nnz, (uint32_t)ul, nunits, a.out, a.stride);
        sptgb_count_launch(1);
    }
    k_mttkrp_seg<W, NP, BF16><<<(unsigned)blocks, BLOCK, 0, s>>>(a, (uint32_t)ul, nunits);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

template <int W, bool BF16, bool FULL, int NF>
cudaError_t launch_rec_k(const sptgb_mttkrp_args &a, cudaStream_t s) {
    constexpr int NB = 2;   // order-4 records per batch (3: register spills at 3 CTAs/SM)
    static const int per_sm = [] {
        int p = 0;
        if (NF == 2)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_mttkrp_rec<W, BF16, FULL>, BLOCK, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_mttkrp_rec4<W, BF16, FULL, NB>, BLOCK, 0);
        return p < 1 ? 1 : p;
    }();
    const int max_blocks = per_sm * sptgb_sm_count();
    // 256-nonzero units: enough of them to balance a power-law row distribution
    const uint32_t ul = SPTGB_REC_UNIT;
    const uint64_t nunits = (a.nnz + ul - 1) / ul;
    const uint64_t u1 = a.unit_end && a.unit_end < nunits ? a.unit_end : nunits;
    if (a.unit_begin >= u1) return cudaSuccess;
    const uint64_t wpb = BLOCK / W;
    uint64_t blocks = (u1 - a.unit_begin + wpb - 1) / wpb;
    if (blocks > (uint64_t)max_blocks) blocks = max_blocks;
    if (!a.out_zeroed) {
        cudaError_t e = cudaMemsetAsync(a.out, 0, (size_t)a.out_rows * a.stride * sizeof(float), s);
        if (e != cudaSuccess) return e;
    }
    if (NF == 2)
        k_mttkrp_rec<W, BF16, FULL><<<(unsigned)blocks, BLOCK, 0, s>>>(static_cast<const uint4 *>(a.rec), a.fac[0],
                                                                      a.fac[1], a.out, a.nnz, a.stride, a.rank, ul,
                                                                      a.unit_begin, u1);
    else
        k_mttkrp_rec4<W, BF16, FULL, NB><<<(unsigned)blocks, BLOCK, 0, s>>>(
            static_cast<const uint4 *>(a.rec), a.vals, a.fac[0], a.fac[1], a.fac[2], a.out, a.nnz, a.stride, a.rank,
            ul, a.unit_begin, u1);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

template <int W, bool BF16, int NF>
cudaError_t launch_rec(const sptgb_mttkrp_args &a, cudaStream_t s) {
    return a.stride == 4u * W ? launch_rec_k<W, BF16, true, NF>(a, s) : launch_rec_k<W, BF16, false, NF>(a, s);
}

template <int W, bool BF16>
cudaError_t dispatch_np(const sptgb_mttkrp_args &a, cudaStream_t s) {
    if (a.rec && a.nprod == 2) return launch_rec<W, BF16, 2>(a, s);
    if (a.rec && a.nprod == 3) return launch_rec<W, BF16, 3>(a, s);
    switch (a.nprod) {
        case 1: return launch<W, 1, BF16>(a, s);
        case 2: return launch<W, 2, BF16>(a, s);
        case 3: return launch<W, 3, BF16>(a, s);
        default: return launch<W, 0, BF16>(a, s);
    }
}

template <bool BF16>
cudaError_t dispatch_w(const sptgb_mttkrp_args &a, cudaStream_t s) {
    const uint32_t c4 = a.stride / 4;
    if (c4 <= 2) return dispatch_np<2, BF16>(a, s);
    if (c4 <= 4) return dispatch_np<4, BF16>(a, s);
    if (c4 <= 8) return dispatch_np<8, BF16>(a, s);
    if (c4 <= 16) return dispatch_np<16, BF16>(a, s);
    return dispatch_np<32, BF16>(a, s);
}

}  // namespace

__global__ void k_rec_chunk_bounds(const uint4 *__restrict__ rec, uint64_t n, uint32_t rows, int k,
                                   uint32_t *__restrict__ out) {
    const int c = threadIdx.x + 1;
    if (c >= k) return;
    const uint32_t r = (uint32_t)((uint64_t)rows * c / k);
    uint64_t lo = 0, hi = n;   // first position with rec.x >= r
    while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if (rec[mid].x < r) lo = mid + 1;
        else hi = mid;
    }
    const uint64_t u = lo / SPTGB_REC_UNIT;
    out[2 * (c - 1)] = (uint32_t)u;
    out[2 * (c - 1) + 1] = u ? rec[u * SPTGB_REC_UNIT - 1].x : 0u;
}

extern "C" cudaError_t sptgb_rec_chunk_bounds(const void *rec, uint64_t n, uint32_t rows, int k, uint32_t *out,
                                              cudaStream_t s) {
    if (k < 2 || k > 8 || n == 0) return cudaErrorInvalidValue;
    k_rec_chunk_bounds<<<1, 32, 0, s>>>(static_cast<const uint4 *>(rec), n, rows, k, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_pack_records(const uint32_t *rows, const uint32_t *ia, const uint32_t *ib,
                                          const float *vals, uint32_t lim_a, uint32_t lim_b, unsigned int *bad,
                                          void *rec, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t g = (n + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    k_pack_records<<<(unsigned)g, 256, 0, s>>>(rows, ia, ib, vals, lim_a, lim_b, bad, static_cast<uint4 *>(rec), n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_mttkrp_coo(const sptgb_mttkrp_args *a, cudaStream_t s) {
    if (a->stride % 8 != 0 || a->stride > 128 || a->nprod < 1 || a->nprod > SPTGB_MAX_MODES - 1)
        return cudaErrorInvalidValue;
    if (a->out_rows == 0) return cudaSuccess;
    if (a->nnz == 0) {
        sptgb_count_launch(0);
        return cudaMemsetAsync(a->out, 0, (size_t)a->out_rows * a->stride * sizeof(float), s);
    }
    return a->bf16 ? dispatch_w<true>(*a, s) : dispatch_w<false>(*a, s);
}

extern "C" cudaError_t sptgb_pack_records4(const uint32_t *rows, const uint32_t *ia, const uint32_t *ib,
                                           const uint32_t *ic, uint32_t lim_a, uint32_t lim_b, uint32_t lim_c,
                                           unsigned int *bad, void *rec, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t g = (n + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    k_pack_records4<<<(unsigned)g, 256, 0, s>>>(rows, ia, ib, ic, lim_a, lim_b, lim_c, bad, static_cast<uint4 *>(rec),
                                                n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}
