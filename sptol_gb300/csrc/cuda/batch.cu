// Batched CP-ALS: one ALS iteration for every tensor ("slot") of a batch as a
// fixed sequence of kernels.
//
// Every kernel takes a work list in device memory (count of listed slots,
// their ids, the exclusive prefix of work items per slot) and a fixed,
// persistent grid that walks the items; a worker finds its slot by binary
// search over the prefix.  Sizes are read on the device, so the host can
// change which slots are listed between launches without touching the launch
// parameters, and the whole step can be captured once in a CUDA graph and
// replayed.
//
// Per mode m (slots with fewer modes are simply not listed):
//   zero      rows of the slot's MTTKRP output
//   mttkrp    one launch per lane group W in {2,4,8,16} (rank <= 8, 16, 32,
//             64), work items = 'ul'-nonzero units, same unit body as the
//             single-tensor kernel (mttkrp_unit.cuh)
//   prepare   one block per slot: Hadamard of the other Grams, FP64
//             Cholesky / LU, inverse (dense_common.cuh)
//   solve     row blocks: rows solved in FP64, Gram and column-max partials
//   lambda    one block per slot: 2-norm at the slot's first iteration, else
//             max-norm, normalised Gram
//   scale     row blocks: columns divided by lambda
// then the fit (inner-product partials, final) and the slot's iteration
// counter.  The per-slot decomposition into blocks is the single-tensor one,
// so a slot computes the same arithmetic alone, in a batch, or through
// sptgbCpdAls.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "dense_common.cuh"
#include "mttkrp_unit.cuh"

namespace {

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


__global__ void k_b_zero(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
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

template <int W>
__global__ void __launch_bounds__(BT, 2)
k_b_mttkrp(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode, uint32_t ul) {
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
                sptgb_mttkrp::unit<false, true, 2>(rec, nullptr, F, rb, s.M, s.nnz, start, len, s.stride, s.rank, sl);
            else
                sptgb_mttkrp::unit<false, false, 2>(rec, nullptr, F, rb, s.M, s.nnz, start, len, s.stride, s.rank, sl);
        } else {
            if (s.stride == 4u * W)
                sptgb_mttkrp::unit<false, true, 3, 2>(rec, s.val4[mode], F, rb, s.M, s.nnz, start, len, s.stride, s.rank,
                                                   sl);
            else
                sptgb_mttkrp::unit<false, false, 3, 2>(rec, s.val4[mode], F, rb, s.M, s.nnz, start, len, s.stride, s.rank,
                                                    sl);
        }
    }
}

__global__ void __launch_bounds__(DT) k_b_prepare(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        GramPtrs gp;
        for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < 4 && m < (int)s.nmodes ? s.gram[m] : nullptr;
        solve_prepare_body(gp, (int)s.nmodes, mode, (int)s.rank, s.S, s.status + mode);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(DT) k_b_solve(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t g = blockIdx.x; g < total; g += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, g);
        const sptgb_slot &s = slots[w.ids[e]];
        const uint32_t b = (uint32_t)(g - w.pre[e]);
        const uint32_t nb = (uint32_t)(w.pre[e + 1] - w.pre[e]);
        const size_t P = (size_t)s.rank * (s.rank + 1) / 2;
        solve_rows_body(s.M, s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride, s.S, s.ws, s.ws + NBLK * P, b,
                        nb);
        __syncthreads();
    }
}

__global__ void k_b_lambda(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        const size_t P = (size_t)s.rank * (s.rank + 1) / 2;
        lambda_body(s.ws, s.ws + NBLK * P, nblocks_for_rows(s.ndims[mode]), (int)s.rank, s.iter == 0 ? 1 : 0,
                    s.gram[mode], s.lambda, nullptr);
        __syncthreads();
    }
}

__global__ void k_b_scale(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
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

__global__ void __launch_bounds__(DT) k_b_fit_partial(const sptgb_slot *__restrict__ slots, sptgb_wlist w) {
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

__global__ void k_b_fit_final(sptgb_slot *__restrict__ slots, sptgb_wlist w, sptgb_wlist parts) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        sptgb_slot &s = slots[w.ids[e]];
        GramPtrs gp;
        for (int m = 0; m < SPTGB_MAX_MODES; ++m) gp.g[m] = m < 4 && m < (int)s.nmodes ? s.gram[m] : nullptr;
        const int nbf = (int)(parts.pre[e + 1] - parts.pre[e]);
        fit_final_body(s.ws, nbf, (int)s.rank, s.lambda, gp, (int)s.nmodes, s.normX2, s.fits + s.iter);
        __syncthreads();
        if (threadIdx.x == 0) s.iter += 1;
        __syncthreads();
    }
}

__global__ void k_pack_records4(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ ia,
                                const uint32_t *__restrict__ ib, const uint32_t *__restrict__ ic,
                                uint4 *__restrict__ rec, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        rec[i] = make_uint4(rows[i], ia[i], ib[i], ic[i]);
}

int g_nsm = 0;
int g_mt_blocks[4];

int nsm() {
    if (!g_nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_b_prepare, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PREP_SMEM);
        cudaFuncSetAttribute(k_b_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOLVE_SMEM);
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_mttkrp<2>, BT, 0);
        g_mt_blocks[0] = (per < 1 ? 1 : per) * g_nsm;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_mttkrp<4>, BT, 0);
        g_mt_blocks[1] = (per < 1 ? 1 : per) * g_nsm;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_mttkrp<8>, BT, 0);
        g_mt_blocks[2] = (per < 1 ? 1 : per) * g_nsm;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_mttkrp<16>, BT, 0);
        g_mt_blocks[3] = (per < 1 ? 1 : per) * g_nsm;
    }
    return g_nsm;
}

cudaError_t mttkrp_group(const sptgb_slot *slots, const sptgb_wlist &w, int mode, int group, uint32_t ul,
                         cudaStream_t s) {
    switch (group) {
        case 0: k_b_mttkrp<2><<<g_mt_blocks[0], BT, 0, s>>>(slots, w, mode, ul); break;
        case 1: k_b_mttkrp<4><<<g_mt_blocks[1], BT, 0, s>>>(slots, w, mode, ul); break;
        case 2: k_b_mttkrp<8><<<g_mt_blocks[2], BT, 0, s>>>(slots, w, mode, ul); break;
        default: k_b_mttkrp<16><<<g_mt_blocks[3], BT, 0, s>>>(slots, w, mode, ul); break;
    }
    sptgb_count_launch(1);
    return cudaGetLastError();
}

}  // namespace

extern "C" uint32_t sptgb_batch_rows_per_block(void) { return TR; }
extern "C" uint32_t sptgb_batch_fit_rows_per_block(void) { return FIT_ROWS; }
extern "C" uint32_t sptgb_batch_zero_rows(void) { return ZERO_ROWS; }
extern "C" uint32_t sptgb_batch_max_blocks(void) { return NBLK; }

extern "C" cudaError_t sptgb_batch_mttkrp(const sptgb_slot *slots, const sptgb_wlist *w, int mode, int group,
                                          uint32_t ul, cudaStream_t s) {
    nsm();
    return mttkrp_group(slots, *w, mode, group, ul, s);
}

extern "C" cudaError_t sptgb_batch_step(const sptgb_slot *slots, const sptgb_step_lists *L, cudaStream_t s) {
    const int n = nsm();
    sptgb_slot *mslots = const_cast<sptgb_slot *>(slots);
    for (int m = 0; m < 4; ++m) {
        k_b_zero<<<n * 8, BT, 0, s>>>(slots, L->zr[m], m);
        sptgb_count_launch(1);
        for (int g = 0; g < 4; ++g) {
            cudaError_t e = mttkrp_group(slots, L->mt[m][g], m, g, L->ul[g], s);
            if (e != cudaSuccess) return e;
        }
        k_b_prepare<<<n * 2, DT, PREP_SMEM, s>>>(slots, L->one[m], m);
        k_b_solve<<<n * 3, DT, SOLVE_SMEM, s>>>(slots, L->dn[m], m);
        k_b_lambda<<<n * 2, DT, 0, s>>>(slots, L->one[m], m);
        k_b_scale<<<n * 8, 256, 0, s>>>(slots, L->dn[m], m);
        sptgb_count_launch(4);
    }
    k_b_fit_partial<<<n * 4, DT, 0, s>>>(slots, L->fit);
    k_b_fit_final<<<n * 2, DT, 0, s>>>(mslots, L->fit_one, L->fit);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_pack_records4(const uint32_t *rows, const uint32_t *ia, const uint32_t *ib,
                                           const uint32_t *ic, void *rec, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint64_t g = (n + 255) / 256;
    if (g > 152ull * 16) g = 152ull * 16;
    k_pack_records4<<<(unsigned)g, 256, 0, s>>>(rows, ia, ib, ic, static_cast<uint4 *>(rec), n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}
