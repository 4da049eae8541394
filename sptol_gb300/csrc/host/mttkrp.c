/*
 * Drop-in COO MTTKRP entry points.
 *
 * sptMTTKRP / sptCudaMTTKRP keep the reference's calling convention
 * (src/sptensor/mttkrp.c:39-115, src/sptensor/mttkrp_cuda_onekernel.cu:41-427):
 * host tensor and host factor matrices in, mats[nmodes] rows [0, ndims[mode])
 * out, nothing retained between calls.  On the GPU each call
 *   1. copies the output-mode coordinates first and checks them against the
 *      mode size and for being non-decreasing (one small read-back),
 *   2. uploads the other coordinates, the values and the N-1 multiplied
 *      factor matrices on a second stream while, when the coordinates were
 *      not sorted, the stable sort by the output coordinate runs,
 *   3. order 3: packs 16-byte records in the caller's order (the other
 *      coordinates range-checked on the way; an out-of-range one becomes row 0
 *      and fails the call after the kernel) and gathers whole records through
 *      the sort permutation; other orders check all coordinates, then gather
 *      the arrays,
 *   4. runs the MTTKRP kernel and copies the result back.
 * No kernel reads a factor row outside its matrix.
 * Shape errors return SPTERR_SHAPE_MISMATCH like mttkrp.c:58-65 (the
 * reference aborts through sptAssert in its 3-D path; this library returns).
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

#define TRACE(name) SPTGB_TRACE_POINT(name, s, t_prev)

/* SPTGB_TRACE=2: one line per host-buffer call with the host times at which
 * its synchronising points returned and the device times of its copy and
 * compute milestones, from timing events; unlike SPTGB_TRACE=1 it adds no
 * synchronisation, so the call overlaps its work as it does untraced. */
enum { T2_START, T2_KEY, T2_FIRST_H2D, T2_ARRAYS, T2_FACTORS, T2_KERNELS, T2_D2H, T2_NEV };
enum { T2H_START, T2H_KEY, T2H_CHUNKS, T2H_END, T2_NHOST };
static cudaEvent_t t2_ev[T2_NEV];
static double t2_host[T2_NHOST];
static int t2_on(void) {
    static int on = -1;
    if (on < 0) {
        const char *e = getenv("SPTGB_TRACE");
        on = e && e[0] == '2';
    }
    return on;
}
static void t2_event(int i, cudaStream_t st) {
    if (!t2_on()) return;
    if (!t2_ev[i]) cudaEventCreate(&t2_ev[i]);
    cudaEventRecord(t2_ev[i], st);
}
static void t2_mark(int i) {
    if (t2_on()) t2_host[i] = sptgb_wall();
}
static void t2_print(sptIndex mode) {
    if (!t2_on()) return;
    float d[T2_NEV] = {0};
    for (int i = 1; i < T2_NEV; ++i)
        if (t2_ev[i] && cudaEventElapsedTime(&d[i], t2_ev[T2_START], t2_ev[i]) != cudaSuccess) d[i] = -1.f;
    fprintf(stderr,
            "[sptgb trace2] mode %u host: key %.2f chunks %.2f end %.2f ms | device: key %.2f first h2d %.2f "
            "arrays %.2f factors %.2f kernels %.2f d2h %.2f ms\n",
            (unsigned)mode, (t2_host[T2H_KEY] - t2_host[T2H_START]) * 1e3,
            (t2_host[T2H_CHUNKS] - t2_host[T2H_START]) * 1e3, (t2_host[T2H_END] - t2_host[T2H_START]) * 1e3,
            d[T2_KEY], d[T2_FIRST_H2D], d[T2_ARRAYS], d[T2_FACTORS], d[T2_KERNELS], d[T2_D2H]);
}

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

/* Order-3 host-buffer calls of at least CHUNKED_MIN_NNZ nonzeros run the
 * kernel in OUT_CHUNKS unit ranges so that the result copy overlaps it. */
#define OUT_CHUNKS 4
#define CHUNKED_MIN_NNZ (1u << 22)

/* Waits for the uploads still in flight on the copy stream (their host
 * buffers belong to the caller) and returns r. */
static int drain_copies(int r) {
    cudaStreamSynchronize(sptgb_copy_stream());
    return r;
}

static int mttkrp_host_locked(sptSparseTensor const *X, sptMatrix *mats[], sptIndex const *mats_order,
                              sptIndex mode, const char *module) {
    const cudaStream_t s = sptgb_stream(), cs = sptgb_copy_stream();
    const sptIndex N = X->nmodes;
    const uint64_t n = X->nnz;
    const sptIndex stride = mats[mode]->stride;
    const sptIndex R = mats[mode]->ncols;
    const sptIndex tmpI = mats[mode]->nrows;
    sptMatrix *M = mats[N];
    double t_prev = sptgb_wall();

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
        for (sptIndex m = 0; m < N; ++m)
            if (need[m] && X->ndims[m] == 0) {   /* no coordinate can be in range */
                spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                                  "a coordinate is not smaller than its mode size");
                return SPTERR_VALUE_ERROR;
            }
        const int recs = N == 3 || N == 4;   /* 16-byte records (order 4: the values in their own array) */
        /* Every buffer is reserved before the first copy: growing one frees
         * and reallocates, which would serialise the two streams. */
        SPTGB_CHECK(sptgb_ws_sync_objects(), module);
        for (sptIndex m = 0; m < N; ++m)
            if (need[m]) SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.inds[m], n * sizeof(uint32_t)), module);
        SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.vals, n * sizeof(float)), module);
        for (sptIndex i = 1; i < N; ++i) {
            const sptIndex pm = mats_order[i];
            const size_t bytes = (size_t)mats[pm]->nrows * stride * sizeof(float);
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.fac[pm], bytes ? bytes : 16), module);
        }
        SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.flag, 32 * sizeof(unsigned int)), module);
        if (recs) {
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.misc[0], n * 16), module);
            SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.misc[1], n * 16), module);
        }
        if (N == 4) SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.svals, n * sizeof(float)), module);
        uint32_t *din[SPTGB_MAX_MODES] = {0};
        for (sptIndex m = 0; m < N; ++m)
            if (need[m]) din[m] = (uint32_t *)g_ws.inds[m].ptr;
        unsigned int *dflag = (unsigned int *)g_ws.flag.ptr, *hflag = g_ws.hflag;

        /* 1. the output coordinates first: the range check, the sortedness
         *    check and the sort need only them. */
        t2_mark(T2H_START);
        t2_event(T2_START, s);
        SPTGB_CUDA(cudaMemcpyAsync(din[mode], X->inds[mode].data, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s),
                   module);
        {
            const uint32_t lim = X->ndims[mode];
            const uint32_t *one[1] = {din[mode]};
            SPTGB_CUDA(sptgb_check_bounds(one, &lim, 1, n, dflag, s), module);
            SPTGB_CUDA(sptgb_check_sorted(din[mode], n, dflag + 1, s), module);
            SPTGB_CUDA(cudaMemsetAsync(dflag + 2, 0, sizeof(unsigned int), s), module);
            SPTGB_CUDA(cudaMemcpyAsync(hflag, dflag, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s), module);
            SPTGB_CUDA(cudaEventRecord(g_ws.ev[0], s), module);
            t2_event(T2_KEY, s);
        }
        /* 2. the other arrays and the factor matrices on the copy stream;
         *    the first one goes while the checks above run. */
        const void *src[2 * SPTGB_MAX_MODES + 1];
        void *dst[2 * SPTGB_MAX_MODES + 1];
        size_t len[2 * SPTGB_MAX_MODES + 1];
        int nup = 0;
        for (sptIndex m = 0; m < N; ++m)
            if (need[m] && m != mode) {
                src[nup] = X->inds[m].data, dst[nup] = din[m], len[nup++] = n * sizeof(uint32_t);
            }
        src[nup] = X->values.data, dst[nup] = g_ws.vals.ptr, len[nup++] = n * sizeof(float);
        const int narr = nup;   /* coordinate and value arrays (at least one); the factor matrices follow */
        for (sptIndex i = 1; i < N; ++i) {
            const sptIndex pm = mats_order[i];
            const size_t bytes = (size_t)mats[pm]->nrows * stride * sizeof(float);
            if (bytes) src[nup] = mats[pm]->values, dst[nup] = g_ws.fac[pm].ptr, len[nup++] = bytes;
        }
        SPTGB_CUDA(cudaMemcpyAsync(dst[0], src[0], len[0], cudaMemcpyHostToDevice, cs), module);
        t2_event(T2_FIRST_H2D, cs);
        cudaError_t e = cudaEventSynchronize(g_ws.ev[0]);
        if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));
        t2_mark(T2H_KEY);
        TRACE("h2d key");
        if (hflag[0]) {
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                              "a coordinate is not smaller than its mode size");
            return drain_copies(SPTERR_VALUE_ERROR);
        }
        const int unsorted = (int)hflag[1];
        /* 3. the stable sort by the output coordinate (within a row the
         *    nonzeros keep the caller's order, as the reference accumulates
         *    them) overlaps the remaining uploads. */
        uint32_t *perm = NULL;
        if (unsorted) {
            sptgb_sortpass pass = {0, (int)mode, 0, 0, sptgb_bitwidth(X->ndims[mode] ? X->ndims[mode] - 1 : 0)};
            const int r = sptgb_sort_perm(din, (int)N, n, &pass, 1, &perm, s);
            if (r) return drain_copies(r);
        }
        /* ev[2]: the coordinate and value arrays are on the device; ev[1]:
         * the factor matrices too.  A pageable upload returns to the host only
         * when its bytes are staged, so the device work that can overlap the
         * factor uploads (order 3: packing and permuting the records) is
         * enqueued before they are issued. */
        for (int k = 1; k < narr; ++k) {
            e = cudaMemcpyAsync(dst[k], src[k], len[k], cudaMemcpyHostToDevice, cs);
            if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));
        }
        e = cudaEventRecord(g_ws.ev[2], cs);
        t2_event(T2_ARRAYS, cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g_ws.ev[2], 0);
        if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));

        sptgb_mttkrp_args a;
        memset(&a, 0, sizeof a);
        if (recs) {
            /* 4. records in the caller's order with the other coordinates
             *    range-checked (an out-of-range one becomes row 0 and flags
             *    the call), then whole records through the permutation. */
            const sptIndex pa = mats_order[1], pb = mats_order[2];
            void *rec = g_ws.misc[0].ptr, *tmp = g_ws.misc[1].ptr;
            if (N == 3) {
                e = sptgb_pack_records(din[mode], din[pa], din[pb], (const float *)g_ws.vals.ptr, X->ndims[pa],
                                       X->ndims[pb], dflag + 2, unsorted ? tmp : rec, n, s);
                a.vals = NULL;
            } else {
                /* order 4: {row, a, b, c} in the caller's product order, the
                 * values permuted alongside */
                const sptIndex pc = mats_order[3];
                e = sptgb_pack_records4(din[mode], din[pa], din[pb], din[pc], X->ndims[pa], X->ndims[pb],
                                        X->ndims[pc], dflag + 2, unsorted ? tmp : rec, n, s);
                a.vals = (const float *)g_ws.vals.ptr;
                if (e == cudaSuccess && unsorted) {
                    e = sptgb_gather_u32((const uint32_t *)g_ws.vals.ptr, perm, (uint32_t *)g_ws.svals.ptr, n, s);
                    a.vals = (const float *)g_ws.svals.ptr;
                }
            }
            if (e == cudaSuccess && unsorted) e = sptgb_gather_records(tmp, perm, rec, n, s);
            if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));
            a.rec = rec;
        }
        for (int k = narr; k < nup; ++k) {
            e = cudaMemcpyAsync(dst[k], src[k], len[k], cudaMemcpyHostToDevice, cs);
            if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));
        }
        e = cudaEventRecord(g_ws.ev[1], cs);
        t2_event(T2_FACTORS, cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g_ws.ev[1], 0);
        if (e != cudaSuccess) return drain_copies(sptgb_cuda_fail(e, module, __FILE__, __LINE__));
        TRACE("h2d rest");
        if (!recs) {
            /* other orders read the coordinate arrays directly: check them
             * all before the kernel runs */
            SPTGB_CHECK(sptgb_validate(din, X->ndims, (int)N, n, NULL, NULL, s), module);
            uint32_t *cols[SPTGB_MAX_MODES] = {0};
            float *vals = (float *)g_ws.vals.ptr;
            for (sptIndex m = 0; m < N; ++m) cols[m] = din[m];
            if (unsorted) {
                uint32_t *dout[SPTGB_MAX_MODES] = {0};
                for (sptIndex m = 0; m < N; ++m)
                    if (need[m]) {
                        SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.sinds[m], n * sizeof(uint32_t)), module);
                        dout[m] = (uint32_t *)g_ws.sinds[m].ptr;
                    }
                SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.svals, n * sizeof(float)), module);
                SPTGB_CHECK(sptgb_gather_tensor(din, vals, dout, (float *)g_ws.svals.ptr, (int)N, perm, n, s), module);
                for (sptIndex m = 0; m < N; ++m) cols[m] = dout[m];
                vals = (float *)g_ws.svals.ptr;
            }
            TRACE("sort");
            a.rows = cols[mode];
            for (sptIndex i = 1; i < N; ++i) a.idx[i - 1] = cols[mats_order[i]];
            a.vals = vals;
        }
        for (sptIndex i = 1; i < N; ++i) a.fac[i - 1] = g_ws.fac[mats_order[i]].ptr;
        a.out = (float *)g_ws.out.ptr;
        a.nnz = n;
        a.out_rows = tmpI;
        a.nprod = N - 1;
        a.rank = R;
        a.stride = stride;
        const uint64_t nunits = (n + SPTGB_REC_UNIT - 1) / SPTGB_REC_UNIT;
        const int nchunk = recs && tmpI && n >= CHUNKED_MIN_NNZ ? OUT_CHUNKS : 1;
        if (nchunk == 1) {
            SPTGB_CUDA(sptgb_mttkrp_coo(&a, s), module);
            t2_event(T2_KERNELS, s);
            TRACE("kernel");
            if (recs)
                SPTGB_CUDA(cudaMemcpyAsync(hflag + 2, dflag + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, s),
                           module);
            if (tmpI)
                SPTGB_CUDA(cudaMemcpyAsync(M->values, g_ws.out.ptr, (size_t)tmpI * stride * sizeof(float),
                                           cudaMemcpyDeviceToHost, s),
                           module);
        } else {
            /* 5. the kernel in unit ranges cut at row quantiles, launched
             *    last rows first; after the launches of ranges c..K-1 every
             *    row above the last row before range c is final and goes back
             *    on the copy stream while the earlier ranges run (power-law
             *    tensors put most rows in the light tail and most nonzeros in
             *    the first rows, so the copy overlaps the heavy range). */
            uint32_t *dcb = (uint32_t *)g_ws.flag.ptr + 4;
            SPTGB_CUDA(sptgb_rec_chunk_bounds(a.rec, n, tmpI, nchunk, dcb, s), module);
            SPTGB_CUDA(cudaMemcpyAsync(hflag + 8, dcb, 2 * (nchunk - 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                       module);
            SPTGB_CUDA(cudaMemsetAsync(g_ws.out.ptr, 0, (size_t)tmpI * stride * sizeof(float), s), module);
            SPTGB_CUDA(cudaStreamSynchronize(s), module);
            t2_mark(T2H_CHUNKS);
            uint64_t ub[OUT_CHUNKS + 1];
            uint32_t last[OUT_CHUNKS];
            ub[0] = 0, last[0] = 0, ub[nchunk] = nunits;
            for (int c = 1; c < nchunk; ++c) {
                ub[c] = hflag[8 + 2 * (c - 1)];
                last[c] = hflag[8 + 2 * (c - 1) + 1];
                if (ub[c] < ub[c - 1]) ub[c] = ub[c - 1];   /* monotone for sorted rows; kept so regardless */
                if (ub[c] > nunits) ub[c] = nunits;
            }
            a.out_zeroed = 1;
            for (int c = nchunk - 1; c >= 0; --c) {
                a.unit_begin = ub[c];
                a.unit_end = ub[c + 1];
                if (ub[c] < ub[c + 1]) SPTGB_CUDA(sptgb_mttkrp_coo(&a, s), module);
                SPTGB_CUDA(cudaEventRecord(g_ws.cev[c], s), module);
            }
            t2_event(T2_KERNELS, s);
            SPTGB_CUDA(cudaMemcpyAsync(hflag + 2, dflag + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, s),
                       module);
            uint32_t hi = tmpI;
            for (int c = nchunk - 1; c >= 0; --c) {
                uint32_t lo = c > 0 && ub[c] > 0 ? last[c] + 1 : 0;
                if (lo > hi) lo = hi;
                if (hi > lo) {
                    SPTGB_CUDA(cudaStreamWaitEvent(cs, g_ws.cev[c], 0), module);
                    SPTGB_CUDA(cudaMemcpyAsync(M->values + (size_t)lo * stride, (const float *)g_ws.out.ptr +
                                                   (size_t)lo * stride,
                                               (size_t)(hi - lo) * stride * sizeof(float), cudaMemcpyDeviceToHost, cs),
                               module);
                }
                hi = lo;
            }
            t2_event(T2_D2H, cs);
            SPTGB_CUDA(cudaStreamSynchronize(cs), module);
        }
    }
    if (n == 0 && tmpI)
        SPTGB_CUDA(cudaMemcpyAsync(M->values, g_ws.out.ptr, (size_t)tmpI * stride * sizeof(float),
                                   cudaMemcpyDeviceToHost, s),
                   module);
    SPTGB_CUDA(cudaStreamSynchronize(s), module);
    if (n) {
        t2_mark(T2H_END);
        t2_print(mode);
    }
    TRACE("d2h out");
    if (n && (N == 3 || N == 4) && g_ws.hflag[2]) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                          "a coordinate is not smaller than its mode size");
        return SPTERR_VALUE_ERROR;
    }
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
    if (r) drain_copies(r);   /* no upload from the caller's buffers outlives the call */
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

int sptOmpMTTKRP_Lock(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[],
                      sptIndex const mode, const int tk, sptMutexPool *lock_pool) {
    (void)tk;
    (void)lock_pool;
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
