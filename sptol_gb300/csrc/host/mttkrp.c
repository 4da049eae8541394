/*
 * Drop-in COO MTTKRP entry points.
 *
 * sptMTTKRP / sptCudaMTTKRP keep the reference's calling convention
 * (src/sptensor/mttkrp.c:39-115, src/sptensor/mttkrp_cuda_onekernel.cu:41-427):
 * host tensor and host factor matrices in, mats[nmodes] rows [0, ndims[mode])
 * out, nothing retained between calls.  On the GPU each call
 *   1. copies the coordinates the product needs, the values and the N-1
 *      multiplied factor matrices to the device,
 *   2. checks every coordinate against its mode size (kernels never see an
 *      out-of-range row) and whether the output-mode coordinates are already
 *      non-decreasing,
 *   3. if not, sorts the nonzeros stably by the output-mode coordinate,
 *   4. runs the segmented MTTKRP kernel and copies the result back.
 * Shape errors return SPTERR_SHAPE_MISMATCH like mttkrp.c:58-65 (the
 * reference aborts through sptAssert in its 3-D path; this library returns).
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include <time.h>
#include "devtensor.h"

/* SPTGB_TRACE=1 prints the wall time of each phase of a host-buffer call to
 * stderr (the reference prints its H2D / kernel / D2H times the same way,
 * src/sptensor/mttkrp_cuda_onekernel.cu:151-155, :381-404). */
static int trace_on(void) {
    static int on = -1;
    if (on < 0) {
        const char *e = getenv("SPTGB_TRACE");
        on = (e && e[0] && e[0] != '0') ? 1 : 0;
    }
    return on;
}
static double wall(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}
#define TRACE(name)                                                              \
    do {                                                                         \
        if (trace_on()) {                                                        \
            cudaStreamSynchronize(s);                                            \
            const double _t = wall();                                            \
            fprintf(stderr, "[sptgb trace] %-10s %8.3f ms\n", name, (_t - t_prev) * 1e3); \
            t_prev = _t;                                                         \
        }                                                                        \
    } while (0)

static int check_mats(sptIndex nmodes, const sptIndex *ndims, sptMatrix *mats[], sptIndex mode, const char *module) {
    if (nmodes < 2 || nmodes > SPTGB_MAX_MODES || mode >= nmodes) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order or mode");
        return SPTERR_VALUE_ERROR;
    }
    for (sptIndex i = 0; i < nmodes; ++i) {
        if (mats[i]->ncols != mats[nmodes]->ncols) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__,
                              "mats[i]->cols != mats[nmodes]->ncols");
            return SPTERR_SHAPE_MISMATCH;
        }
        if (mats[i]->nrows != ndims[i]) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "mats[i]->nrows != ndims[i]");
            return SPTERR_SHAPE_MISMATCH;
        }
        if (mats[i]->stride != mats[nmodes]->stride) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "factor strides differ");
            return SPTERR_SHAPE_MISMATCH;
        }
    }
    if (mats[nmodes]->cap < mats[mode]->nrows) {
        spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "mats[nmodes] has too few rows");
        return SPTERR_SHAPE_MISMATCH;
    }
    if (mats[mode]->stride > 128) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "rank above 128 is not supported");
        return SPTERR_VALUE_ERROR;
    }
    return 0;
}

static int mttkrp_host_locked(sptSparseTensor const *X, sptMatrix *mats[], sptIndex const *mats_order,
                              sptIndex mode, const char *module) {
    const cudaStream_t s = sptgb_stream();
    const sptIndex N = X->nmodes;
    const uint64_t n = X->nnz;
    const sptIndex stride = mats[mode]->stride;
    const sptIndex R = mats[mode]->ncols;
    const sptIndex tmpI = mats[mode]->nrows;
    sptMatrix *M = mats[N];
    double t_prev = wall();

    int need[SPTGB_MAX_MODES] = {0};
    need[mode] = 1;
    for (sptIndex i = 1; i < N; ++i) {
        if (mats_order[i] >= N) {
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "mats_order entry out of range");
            return SPTERR_VALUE_ERROR;
        }
        need[mats_order[i]] = 1;
    }
    SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.out, (size_t)(tmpI ? tmpI : 1) * stride * sizeof(float)), module);
    if (n == 0) {
        SPTGB_CUDA(cudaMemsetAsync(g_ws.out.ptr, 0, (size_t)tmpI * stride * sizeof(float), s), module);
    } else {
        SPTGB_CHECK(sptgb_upload_tensor(X, g_ws.inds, &g_ws.vals, need, s), module);
        TRACE("h2d tensor");
        uint32_t *din[SPTGB_MAX_MODES] = {0};
        for (sptIndex m = 0; m < N; ++m)
            if (need[m]) din[m] = (uint32_t *)g_ws.inds[m].ptr;
        for (sptIndex i = 1; i < N; ++i) {
            const sptIndex pm = mats_order[i];
            const size_t bytes = (size_t)mats[pm]->nrows * stride * sizeof(float);
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.fac[pm], bytes ? bytes : 16), module);
            if (bytes)
                SPTGB_CUDA(cudaMemcpyAsync(g_ws.fac[pm].ptr, mats[pm]->values, bytes, cudaMemcpyHostToDevice, s),
                           module);
        }
        TRACE("h2d mats");
        int unsorted = 1;
        SPTGB_CHECK(sptgb_validate(din, X->ndims, (int)N, n, din[mode], &unsorted, s), module);
        TRACE("validate");
        uint32_t *rows = din[mode];
        uint32_t *cols[SPTGB_MAX_MODES] = {0};
        float *vals = (float *)g_ws.vals.ptr;
        for (sptIndex m = 0; m < N; ++m) cols[m] = din[m];
        if (unsorted) {
            /* Stable sort by the output coordinate: within a row the nonzeros
             * keep the caller's order, as the reference accumulates them. */
            sptgb_sortpass pass = {0, (int)mode, 0, 0, sptgb_bitwidth(X->ndims[mode] ? X->ndims[mode] - 1 : 0)};
            uint32_t *perm = NULL;
            SPTGB_CHECK(sptgb_sort_perm(din, (int)N, n, &pass, 1, &perm, s), module);
            uint32_t *dout[SPTGB_MAX_MODES] = {0};
            for (sptIndex m = 0; m < N; ++m)
                if (need[m]) {
                    SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.sinds[m], n * sizeof(uint32_t)), module);
                    dout[m] = (uint32_t *)g_ws.sinds[m].ptr;
                }
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.svals, n * sizeof(float)), module);
            SPTGB_CHECK(sptgb_gather_tensor(din, vals, dout, (float *)g_ws.svals.ptr, (int)N, perm, n, s), module);
            for (sptIndex m = 0; m < N; ++m) cols[m] = dout[m];
            rows = dout[mode];
            vals = (float *)g_ws.svals.ptr;
            TRACE("sort");
        }
        sptgb_mttkrp_args a;
        memset(&a, 0, sizeof a);
        a.rows = rows;
        for (sptIndex i = 1; i < N; ++i) {
            a.idx[i - 1] = cols[mats_order[i]];
            a.fac[i - 1] = g_ws.fac[mats_order[i]].ptr;
        }
        a.vals = vals;
        if (N == 3) {
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.misc[0], n * 16), module);
            SPTGB_CUDA(sptgb_pack_records(rows, cols[mats_order[1]], cols[mats_order[2]], vals, g_ws.misc[0].ptr, n, s),
                       module);
            a.rec = g_ws.misc[0].ptr;
        }
        a.out = (float *)g_ws.out.ptr;
        a.nnz = n;
        a.out_rows = tmpI;
        a.nprod = N - 1;
        a.rank = R;
        a.stride = stride;
        SPTGB_CUDA(sptgb_mttkrp_coo(&a, s), module);
        TRACE("kernel");
    }
    if (tmpI)
        SPTGB_CUDA(cudaMemcpyAsync(M->values, g_ws.out.ptr, (size_t)tmpI * stride * sizeof(float),
                                   cudaMemcpyDeviceToHost, s),
                   module);
    SPTGB_CUDA(cudaStreamSynchronize(s), module);
    TRACE("d2h out");
    return 0;
}

static int mttkrp_host(sptSparseTensor const *X, sptMatrix *mats[], sptIndex const *mats_order, sptIndex mode,
                       const char *module) {
    SPTGB_CHECK(check_mats(X->nmodes, X->ndims, mats, mode, module), module);
    if (X->nnz >= 0xffffffffull) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "more than 2^32-2 nonzeros");
        return SPTERR_VALUE_ERROR;
    }
    SPTGB_CHECK(sptgb_ctx(), module);
    sptgb_lock();
    const int r = mttkrp_host_locked(X, mats, mats_order, mode, module);
    sptgb_unlock();
    return r;
}

int sptMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[], sptIndex const mode) {
    return mttkrp_host(X, mats, mats_order, mode, "GPU SpTns MTTKRP");
}

int sptOmpMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[], sptIndex const mode,
                 const int tk) {
    (void)tk;
    return mttkrp_host(X, mats, mats_order, mode, "GPU SpTns MTTKRP");
}

int sptOmpMTTKRP_Reduce(sptSparseTensor const *const X, sptMatrix *mats[], sptMatrix *copy_mats[],
                        sptIndex const mats_order[], sptIndex const mode, const int tk) {
    (void)tk;
    (void)copy_mats;
    return mttkrp_host(X, mats, mats_order, mode, "GPU SpTns MTTKRP");
}

int sptCudaMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex *const mats_order, sptIndex const mode,
                  sptIndex const impl_num) {
    (void)impl_num;
    return mttkrp_host(X, mats, mats_order, mode, "CUDA SpTns MTTKRP");
}

int sptCudaMTTKRPOneKernel(sptSparseTensor const *const X, sptMatrix **const mats, sptIndex *const mats_order,
                           sptIndex const mode, sptIndex const impl_num) {
    (void)impl_num;
    return mttkrp_host(X, mats, mats_order, mode, "CUDA SpTns MTTKRP");
}
