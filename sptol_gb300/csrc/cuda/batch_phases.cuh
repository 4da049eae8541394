// The phases of the batched CP-ALS step as block-level device functions,
// shared by the kernel sequence (batch.cu: one launch per phase) and the
// persistent step (batch_step.cu: all phases in one cooperative launch).
//
// Every phase takes a work list in device memory (count of listed slots,
// their ids, the exclusive prefix of work items per slot) and walks the items
// grid-stride; a worker finds its slot by binary search over the prefix.  The
// items a slot is split into do not depend on the grid, so both launch forms
// compute the same arithmetic.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "dense_common.cuh"
#include "mttkrp_unit.cuh"

namespace sptgb_batch {

using namespace sptgb_dense;

constexpr int BT = 256;
constexpr uint32_t ZERO_ROWS = 256;   // rows per zeroing item
constexpr uint32_t FIT_ROWS = 8;      // rows per fit block (as sptgb_fit)

__device__ __forceinline__ uint32_t find_entry(const uint64_t *pre, uint32_t cnt, uint64_t g) {
    uint32_t lo = 0, hi = cnt;   // last e with pre[e] <= g
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pre[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}


__device__ __forceinline__ void ph_zero(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t g = blockIdx.x; g < total; g += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &sl = slots[w.ids[e]];
        const uint64_t r0 = (g - w.pre[e]) * ZERO_ROWS;
        const uint64_t r1 = min(r0 + ZERO_ROWS, (uint64_t)sl.ndims[mode]);
        float4 *p = reinterpret_cast<float4 *>(sl.M + r0 * sl.stride);
        const uint64_t n4 = (r1 - r0) * sl.stride / 4;
        for (uint64_t i = threadIdx.x; i < n4; i += BT) p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// DEEP: records software-pipelined in batches of 4 (order 3) / 2 (order 4),
// else 2 / 1; the batch depth changes the loads in flight, not the arithmetic.
template <int W, bool COH, bool DEEP>
__device__ __forceinline__ void ph_mttkrp(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w, int mode,
                                          uint32_t ul) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    const int sl = (threadIdx.x & 31) % W;
    const uint64_t worker = ((uint64_t)blockIdx.x * BT + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BT) / W;
    for (uint64_t g = worker; g < total; g += nworkers) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &s = slots[w.ids[e]];
        const uint64_t start = (g - w.pre[e]) * ul;
        const uint32_t len = (uint32_t)min((uint64_t)ul, s.nnz - start);
        // the other modes in ascending order: i, skipping 'mode'
        const char *F[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
            F[i] = (i < (int)s.nmodes - 1) ? reinterpret_cast<const char *>(s.fac[i + (i >= mode)] + sl * 4) : nullptr;
        const uint4 *rec = static_cast<const uint4 *>(s.rec[mode]);
        const uint32_t rb = s.stride * 4;
        if (s.nmodes == 3) {
            if (s.stride == 4u * W)
                sptgb_mttkrp::unit<false, true, 2, DEEP ? 4 : 2, COH>(rec, nullptr, F, rb, s.M, s.nnz, start, len, s.stride, s.rank,
                                                          sl);
            else
                sptgb_mttkrp::unit<false, false, 2, DEEP ? 4 : 2, COH>(rec, nullptr, F, rb, s.M, s.nnz, start, len, s.stride, s.rank,
                                                           sl);
        } else {
            if (s.stride == 4u * W)
                sptgb_mttkrp::unit<false, true, 3, DEEP ? 2 : 1, COH>(rec, s.val4[mode], F, rb, s.M, s.nnz, start, len, s.stride,
                                                        s.rank, sl);
            else
                sptgb_mttkrp::unit<false, false, 3, DEEP ? 2 : 1, COH>(rec, s.val4[mode], F, rb, s.M, s.nnz, start, len, s.stride,
                                                         s.rank, sl);
        }
    }
}

__device__ __forceinline__ void ph_prepare(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        GramPtrs gp;
        for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < 4 && m < (int)s.nmodes ? s.gram[m] : nullptr;
        solve_prepare_body(gp, (int)s.nmodes, mode, (int)s.rank, s.S, s.status + mode);
        __syncthreads();
    }
}

__device__ __forceinline__ void ph_solve(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t g = blockIdx.x; g < total; g += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &s = slots[w.ids[e]];
        const uint32_t b = (uint32_t)(g - w.pre[e]);
        const uint32_t nb = (uint32_t)(w.pre[e + 1] - w.pre[e]);
        const size_t P = (size_t)s.rank * (s.rank + 1) / 2;
        solve_rows_body(s.M, s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride, s.S, s.status + mode, s.ws,
                        s.ws + NBLK * P, b, nb);
        __syncthreads();
    }
}

// w: one item per slot; parts: the solve's list (same slots, same order), its
// item count per slot is the number of partials to reduce.
__device__ __forceinline__ void ph_lambda(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w,
                                          const sptgb_wlist &parts, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        const size_t P = (size_t)s.rank * (s.rank + 1) / 2;
        lambda_body(s.ws, s.ws + NBLK * P, (int)(parts.pre[e + 1] - parts.pre[e]), (int)s.rank, s.status[4] == 0 ? 1 : 0,
                    s.gram[mode], s.lambda, nullptr);
        __syncthreads();
    }
}

__device__ __forceinline__ void ph_scale(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t g = blockIdx.x; g < total; g += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &s = slots[w.ids[e]];
        scale_cols_body(s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride, s.lambda,
                        (unsigned)(g - w.pre[e]), (unsigned)(w.pre[e + 1] - w.pre[e]));
    }
}

__device__ __forceinline__ void ph_fit_partial(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t g = blockIdx.x; g < total; g += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &s = slots[w.ids[e]];
        const uint32_t last = s.nmodes - 1;
        inner_partial_body(s.fac[last], s.M, s.ndims[last], (int)s.rank, (int)s.stride, s.ws,
                           (unsigned)(g - w.pre[e]), (unsigned)(w.pre[e + 1] - w.pre[e]));
        __syncthreads();
    }
}

__device__ __forceinline__ void ph_fit_final(const sptgb_slot *__restrict__ slots, const sptgb_wlist &w,
                                             const sptgb_wlist &parts) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        GramPtrs gp;
        for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < 4 && m < (int)s.nmodes ? s.gram[m] : nullptr;
        const int nbf = (int)(parts.pre[e + 1] - parts.pre[e]);
        fit_final_body(s.ws, nbf, (int)s.rank, s.lambda, gp, (int)s.nmodes, s.normX2, s.fits + s.status[4]);
        __syncthreads();
        if (threadIdx.x == 0) s.status[4] += 1;
        __syncthreads();
    }
}

}  // namespace sptgb_batch
