/*
 * COO -> HiCOO conversion and HiCOO MTTKRP behind the reference's entry
 * points (src/sptensor/hicoo/convert.c:237-497, hicoo/mttkrp.c:53-144).
 *
 * Conversion on the GPU:
 *   1. stable device sort in the HiCOO order: kernels (idx >> sk_bits) in
 *      row-major order, Morton order of the full coordinates inside a kernel
 *      (convert.c:160-226); the sorted COO is written back into the caller's
 *      tensor, as the reference sorts it in place;
 *   2. block / kernel heads are flagged where (idx >> sb_bits) /
 *      (idx >> sk_bits) change, scanned into block and kernel numbers, and
 *      compacted into bptr, the first block of every kernel and binds;
 *      einds = idx & (2^sb - 1) (convert.c:397-456).
 * The kernel scheduler kschr (one entry per kernel, convert.c:103-146) and
 * the chunk pointers cptr, whose rule carries a running count across blocks
 * and kernels (convert.c:386-452), are filled on the host from those
 * device-built boundaries.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

#define SC_BITS 14

static int fail_cuda(cudaError_t e, const char *module, unsigned line) {
    return sptgb_cuda_fail(e, module, __FILE__, line);
}

#define C(expr)                                                   \
    do {                                                          \
        cudaError_t _c = (expr);                                  \
        if (_c != cudaSuccess) {                                  \
            r = fail_cuda(_c, module, __LINE__);                  \
            goto out;                                             \
        }                                                         \
    } while (0)
#define H(expr)                                                   \
    do {                                                          \
        r = (expr);                                               \
        if (r) goto out;                                          \
    } while (0)

/* The reference's output for an empty tensor (it reads the zero-filled
 * first slot of the coordinate vectors): one kernel, one empty block. */
static int empty_hicoo(sptSparseTensorHiCOO *h, sptNnzIndex *max_nnzb) {
    int r;
    if ((r = sptAppendNnzIndexVector(&h->kptr, 0)) || (r = sptAppendNnzIndexVector(&h->kptr, 1))) return r;
    if ((r = sptAppendNnzIndexVector(&h->cptr, 0)) || (r = sptAppendNnzIndexVector(&h->cptr, 1))) return r;
    if ((r = sptAppendNnzIndexVector(&h->bptr, 0)) || (r = sptAppendNnzIndexVector(&h->bptr, 0))) return r;
    for (sptIndex m = 0; m < h->nmodes; ++m) {
        if ((r = sptAppendBlockIndexVector(&h->binds[m], 0))) return r;
        if ((r = sptAppendIndexVector(&h->kschr[m][0], 0))) return r;
        h->nkiters[m] = 1;
    }
    *max_nnzb = 0;
    return 0;
}

int sptSparseTensorToHiCOO(sptSparseTensorHiCOO *hitsr, sptNnzIndex *max_nnzb, sptSparseTensor *tsr,
                           const sptElementIndex sb_bits, const sptElementIndex sk_bits, int const tk) {
    (void)tk;
    const char *module = "HiSpTns Convert";
    int r = 0;
    const sptElementIndex sc_bits = SC_BITS;
    if (!(sk_bits >= sb_bits) || !(sc_bits >= sb_bits) || sb_bits > 8 || sk_bits > 31) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "need sb_bits <= min(sk_bits, 14, 8)");
        return SPTERR_VALUE_ERROR;
    }
    const int N = (int)tsr->nmodes;
    const uint64_t n = tsr->nnz;
    if (N < 1 || N > SPTGB_MAX_MODES || n >= 0xffffffffull) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported tensor shape");
        return SPTERR_VALUE_ERROR;
    }
    SPTGB_CHECK(sptNewSparseTensorHiCOO(hitsr, (sptIndex)N, tsr->ndims, n, sb_bits, sk_bits, sc_bits), module);
    for (int m = 0; m < N; ++m) tsr->sortorder[m] = (sptIndex)m;
    if (n == 0) return empty_hicoo(hitsr, max_nnzb);
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();

    uint64_t *h_bstart = NULL, *h_kstart = NULL;
    uint32_t *h_kblk = NULL;
    sptgb_lock();
    uint32_t *din[SPTGB_MAX_MODES] = {0}, *dsrt[SPTGB_MAX_MODES] = {0};
    for (int m = 0; m < N; ++m) {
        H(sptgb_dbuf_reserve(&g_ws.inds[m], n * 4));
        H(sptgb_dbuf_reserve(&g_ws.sinds[m], n * 4));
        din[m] = (uint32_t *)g_ws.inds[m].ptr;
        dsrt[m] = (uint32_t *)g_ws.sinds[m].ptr;
        C(cudaMemcpyAsync(din[m], tsr->inds[m].data, n * 4, cudaMemcpyHostToDevice, s));
    }
    H(sptgb_dbuf_reserve(&g_ws.vals, n * 4));
    H(sptgb_dbuf_reserve(&g_ws.svals, n * 4));
    C(cudaMemcpyAsync(g_ws.vals.ptr, tsr->values.data, n * 4, cudaMemcpyHostToDevice, s));
    H(sptgb_validate(din, tsr->ndims, N, n, NULL, NULL, s));

    sptgb_sortpass passes[24];
    const int np = sptgb_hicoo_passes(tsr->ndims, N, sk_bits, 1, passes);
    uint32_t *perm = NULL;
    H(sptgb_sort_perm(din, N, n, passes, np, &perm, s));
    H(sptgb_gather_tensor(din, (float *)g_ws.vals.ptr, dsrt, (float *)g_ws.svals.ptr, N, perm, n, s));

    /* Scratch: kflags, bflags, kpos, bpos (u32 x n each), scan tmp, totals. */
    H(sptgb_dbuf_reserve(&g_ws.misc[0], n * 4));
    H(sptgb_dbuf_reserve(&g_ws.misc[1], n * 4));
    H(sptgb_dbuf_reserve(&g_ws.misc[2], n * 4));
    H(sptgb_dbuf_reserve(&g_ws.misc[3], n * 4));
    H(sptgb_dbuf_reserve(&g_ws.misc[4], sptgb_scan_tmp_bytes(n)));
    H(sptgb_dbuf_reserve(&g_ws.misc[5], 64));
    uint32_t *kflags = (uint32_t *)g_ws.misc[0].ptr, *bflags = (uint32_t *)g_ws.misc[1].ptr;
    uint32_t *kpos = (uint32_t *)g_ws.misc[2].ptr, *bpos = (uint32_t *)g_ws.misc[3].ptr;
    uint32_t *totals = (uint32_t *)g_ws.misc[5].ptr;
    C(sptgb_mark_groups((const uint32_t *const *)dsrt, N, sk_bits, n, kflags, s));
    C(sptgb_mark_groups((const uint32_t *const *)dsrt, N, sb_bits, n, bflags, s));
    C(sptgb_exclusive_scan_u32(kflags, kpos, n, totals, g_ws.misc[4].ptr, s));
    C(sptgb_exclusive_scan_u32(bflags, bpos, n, totals + 1, g_ws.misc[4].ptr, s));
    uint32_t htot[2] = {0, 0};
    C(cudaMemcpyAsync(htot, totals, sizeof htot, cudaMemcpyDeviceToHost, s));
    /* Sorted COO back into the caller's tensor. */
    for (int m = 0; m < N; ++m)
        C(cudaMemcpyAsync(tsr->inds[m].data, dsrt[m], n * 4, cudaMemcpyDeviceToHost, s));
    C(cudaMemcpyAsync(tsr->values.data, g_ws.svals.ptr, n * 4, cudaMemcpyDeviceToHost, s));
    C(cudaStreamSynchronize(s));
    const uint64_t nk = htot[0], nb = htot[1];

    /* bstart (u64 x nb), kstart (u64 x nk), kblk (u32 x nk), binds (u32 x nb
     * per mode), einds (u8 x n per mode). */
    H(sptgb_dbuf_reserve(&g_ws.misc[6], nb * 8 + nk * 8 + nk * 4 + 64));
    H(sptgb_dbuf_reserve(&g_ws.misc[7], (size_t)N * (nb * 4 + n) + 64));
    uint64_t *bstart = (uint64_t *)g_ws.misc[6].ptr;
    uint64_t *kstart = bstart + nb;
    uint32_t *kblk = (uint32_t *)(kstart + nk);
    uint32_t *dbinds[SPTGB_MAX_MODES];
    uint8_t *deinds[SPTGB_MAX_MODES];
    for (int m = 0; m < N; ++m) {
        dbinds[m] = (uint32_t *)g_ws.misc[7].ptr + (size_t)m * nb;
        deinds[m] = (uint8_t *)((uint32_t *)g_ws.misc[7].ptr + (size_t)N * nb) + (size_t)m * n;
    }
    C(sptgb_compact_starts(bflags, bpos, n, bstart, s));
    C(sptgb_compact_starts(kflags, kpos, n, kstart, s));
    C(sptgb_compact_u32(kflags, kpos, bpos, n, kblk, s));
    C(sptgb_hicoo_split((const uint32_t *const *)dsrt, N, sb_bits, n, bflags, bpos, deinds, dbinds, s));

    h_bstart = (uint64_t *)malloc(nb * 8);
    h_kstart = (uint64_t *)malloc(nk * 8);
    h_kblk = (uint32_t *)malloc(nk * 4);
    if (!h_bstart || !h_kstart || !h_kblk) {
        r = SPTERR_OS_ERROR;
        goto out;
    }
    for (int m = 0; m < N; ++m) {
        H(sptResizeBlockIndexVector(&hitsr->binds[m], nb));
        H(sptResizeElementIndexVector(&hitsr->einds[m], n));
        C(cudaMemcpyAsync(hitsr->binds[m].data, dbinds[m], nb * 4, cudaMemcpyDeviceToHost, s));
        C(cudaMemcpyAsync(hitsr->einds[m].data, deinds[m], n, cudaMemcpyDeviceToHost, s));
    }
    C(cudaMemcpyAsync(h_bstart, bstart, nb * 8, cudaMemcpyDeviceToHost, s));
    C(cudaMemcpyAsync(h_kstart, kstart, nk * 8, cudaMemcpyDeviceToHost, s));
    C(cudaMemcpyAsync(h_kblk, kblk, nk * 4, cudaMemcpyDeviceToHost, s));
    H(sptResizeValueVector(&hitsr->values, n));
    memcpy(hitsr->values.data, tsr->values.data, n * 4);
    C(cudaStreamSynchronize(s));

    /* bptr: block starts then nnz (convert.c:379, :438, :472). */
    H(sptResizeNnzIndexVector(&hitsr->bptr, nb + 1));
    for (uint64_t b = 0; b < nb; ++b) hitsr->bptr.data[b] = (sptNnzIndex)(sptBlockIndex)h_bstart[b];
    hitsr->bptr.data[nb] = n;
    /* kptr: first block of every kernel, then #blocks (convert.c:386-388, :470). */
    H(sptResizeNnzIndexVector(&hitsr->kptr, nk + 1));
    for (uint64_t k = 0; k < nk; ++k) hitsr->kptr.data[k] = h_kblk[k];
    hitsr->kptr.data[nk] = nb;
    /* kschr / nkiters (convert.c:117-143). */
    for (uint64_t k = 0; k < nk; ++k)
        for (int m = 0; m < N; ++m) {
            const sptIndex kc = tsr->inds[m].data[h_kstart[k]] >> sk_bits;
            H(sptAppendIndexVector(&hitsr->kschr[m][kc], (sptIndex)k));
        }
    for (int m = 0; m < N; ++m) {
        const uint64_t sk = 1ull << sk_bits;
        const sptIndex kn = (sptIndex)(((uint64_t)tsr->ndims[m] + sk - 1) / sk);
        sptIndex mx = 0;
        for (sptIndex i = 0; i < kn; ++i)
            if (hitsr->kschr[m][i].len > mx) mx = (sptIndex)hitsr->kschr[m][i].len;
        hitsr->nkiters[m] = mx;
    }
    /* cptr (convert.c:386-452): a chunk starts at every kernel, and at a new
     * block once the running count plus the previous block's size reaches
     * 2^sc_bits; the running count resets at each kernel start but the first
     * block of a kernel still tests the previous kernel's last block. */
    {
        const uint64_t sc = 1ull << sc_bits;
        uint64_t chunk = 0;
        for (uint64_t k = 0; k < nk; ++k) {
            H(sptAppendNnzIndexVector(&hitsr->cptr, h_kblk[k]));
            chunk = 0;
            const uint64_t bend = (k + 1 < nk) ? h_kblk[k + 1] : nb;
            for (uint64_t b = h_kblk[k]; b < bend; ++b) {
                if (b == 0) continue;
                const uint64_t ne = h_bstart[b] - h_bstart[b - 1];
                if (chunk + ne >= sc) {
                    H(sptAppendNnzIndexVector(&hitsr->cptr, b));
                    chunk = 0;
                } else {
                    chunk += ne;
                }
            }
        }
        H(sptAppendNnzIndexVector(&hitsr->cptr, nb));
    }
    {
        sptNnzIndex mx = hitsr->bptr.data[1] - hitsr->bptr.data[0];
        for (uint64_t b = 0; b < nb; ++b) {
            const sptNnzIndex c = hitsr->bptr.data[b + 1] - hitsr->bptr.data[b];
            if (c > mx) mx = c;
        }
        *max_nnzb = mx;
    }
out:
    sptgb_unlock();
    free(h_bstart);
    free(h_kstart);
    free(h_kblk);
    return r;
}

/* convert.c:237-288 on a tensor already in row-block order: kernel start
 * positions, then nnz. */
int sptSetKernelPointers(sptNnzIndexVector *kptr, sptSparseTensor *tsr, const sptElementIndex sk_bits) {
    const sptIndex N = tsr->nmodes;
    const uint64_t n = tsr->nnz;
    int r = sptAppendNnzIndexVector(kptr, 0);
    if (r) return r;
    for (uint64_t z = 1; z < n; ++z) {
        int diff = 0;
        for (sptIndex m = 0; m < N; ++m)
            diff |= (tsr->inds[m].data[z] >> sk_bits) != (tsr->inds[m].data[z - 1] >> sk_bits);
        if (diff && (r = sptAppendNnzIndexVector(kptr, z))) return r;
    }
    return sptAppendNnzIndexVector(kptr, n);
}

/* ------------------------------------------------------- HiCOO MTTKRP -- */
/* Kernel timing of the HiCOO MTTKRP (sptgbHiCOOSetTiming); guarded by the
 * workspace lock like every use of the library stream. */
static int g_hicoo_timing = 0;
static cudaEvent_t g_hicoo_ev[2];
static float g_hicoo_ms = 0.f;

void sptgbHiCOOSetTiming(int enable) {
    sptgb_lock();
    if (enable && !g_hicoo_timing && sptgb_ctx() == 0) {
        if (cudaEventCreate(&g_hicoo_ev[0]) == cudaSuccess && cudaEventCreate(&g_hicoo_ev[1]) == cudaSuccess)
            g_hicoo_timing = 1;
    } else if (!enable && g_hicoo_timing) {
        cudaEventDestroy(g_hicoo_ev[0]);
        cudaEventDestroy(g_hicoo_ev[1]);
        g_hicoo_timing = 0;
    }
    sptgb_unlock();
}

float sptgbHiCOOLastKernelMs(void) { return g_hicoo_ms; }

static int hicoo_mttkrp(sptSparseTensorHiCOO const *h, sptMatrix *mats[], sptIndex const *mats_order, sptIndex mode,
                        const char *module) {
    const sptIndex N = h->nmodes;
    int r = 0;
    if (N < 2 || N > SPTGB_MAX_MODES || mode >= N) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order or mode");
        return SPTERR_VALUE_ERROR;
    }
    for (sptIndex i = 0; i < N; ++i) {
        if (mats[i]->ncols != mats[N]->ncols) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__,
                              "mats[i]->cols != mats[nmodes]->ncols");
            return SPTERR_SHAPE_MISMATCH;
        }
        if (mats[i]->nrows != h->ndims[i]) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "mats[i]->nrows != ndims[i]");
            return SPTERR_SHAPE_MISMATCH;
        }
    }
    for (sptIndex i = 1; i < N; ++i)
        if (mats_order[i] >= N) {
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "mats_order entry out of range");
            return SPTERR_VALUE_ERROR;
        }
    const sptIndex stride = mats[0]->stride;
    if (stride > 128 || mats[N]->cap < mats[mode]->nrows) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "rank above 128 or output too small");
        return SPTERR_VALUE_ERROR;
    }
    const uint64_t nb = h->bptr.len ? h->bptr.len - 1 : 0;
    const uint64_t n = h->nnz;
    const sptIndex tmpI = mats[mode]->nrows;
    /* Structural checks of the caller's HiCOO arrays, so that no kernel reads
     * past them: vectors long enough here; bptr non-decreasing from 0 to nnz
     * on the device, before any kernel uses it. */
    int bad = h->values.len < n || h->sb_bits > 8;
    for (sptIndex m = 0; m < N && !bad; ++m) bad = h->binds[m].len < nb || h->einds[m].len < n;
    if (bad) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "inconsistent HiCOO arrays");
        return SPTERR_VALUE_ERROR;
    }
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = sptgb_stream();
    sptgb_lock();
    sptgb_hicoo_args a;
    memset(&a, 0, sizeof a);
    /* bptr, binds, einds, values */
    double t_prev = sptgb_wall();
    H(sptgb_dbuf_reserve(&g_ws.misc[0], (nb + 1) * 8));
    C(cudaMemcpyAsync(g_ws.misc[0].ptr, h->bptr.data, (nb + 1) * 8, cudaMemcpyHostToDevice, s));
    H(sptgb_dbuf_reserve(&g_ws.misc[1], (size_t)N * (nb * 4 + n) + 64));
    for (sptIndex m = 0; m < N; ++m) {
        uint32_t *db = (uint32_t *)g_ws.misc[1].ptr + (size_t)m * nb;
        uint8_t *de = (uint8_t *)((uint32_t *)g_ws.misc[1].ptr + (size_t)N * nb) + (size_t)m * n;
        if (nb) C(cudaMemcpyAsync(db, h->binds[m].data, nb * 4, cudaMemcpyHostToDevice, s));
        if (n) C(cudaMemcpyAsync(de, h->einds[m].data, n, cudaMemcpyHostToDevice, s));
        a.binds[m] = db;
        a.einds[m] = de;
    }
    H(sptgb_dbuf_reserve(&g_ws.vals, (n ? n : 1) * 4));
    if (n) C(cudaMemcpyAsync(g_ws.vals.ptr, h->values.data, n * 4, cudaMemcpyHostToDevice, s));
    for (sptIndex i = 1; i < N; ++i) {
        const sptIndex pm = mats_order[i];
        const size_t bytes = (size_t)mats[pm]->nrows * stride * 4;
        H(sptgb_dbuf_reserve(&g_ws.fac[pm], bytes ? bytes : 16));
        if (bytes) C(cudaMemcpyAsync(g_ws.fac[pm].ptr, mats[pm]->values, bytes, cudaMemcpyHostToDevice, s));
        a.fac[pm] = (const float *)g_ws.fac[pm].ptr;
    }
    H(sptgb_dbuf_reserve(&g_ws.out, (size_t)(tmpI ? tmpI : 1) * stride * 4));
    SPTGB_TRACE_POINT("h2d", s, t_prev);
    a.bptr = (const uint64_t *)g_ws.misc[0].ptr;
    a.vals = (const float *)g_ws.vals.ptr;
    a.out = (float *)g_ws.out.ptr;
    a.nb = nb;
    a.out_rows = tmpI;
    a.nmodes = N;
    a.mode = mode;
    for (sptIndex i = 0; i < N; ++i) a.order[i] = mats_order[i];
    a.rank = mats[mode]->ncols;
    a.stride = stride;
    a.sb_bits = h->sb_bits;
    for (sptIndex m = 0; m < N; ++m) a.ndims[m] = h->ndims[m];
    H(sptgb_dbuf_reserve(&g_ws.flag, 2 * sizeof(unsigned int)));
    a.err = (unsigned int *)g_ws.flag.ptr;
    a.nnz = n;
    {   /* bptr non-decreasing from 0 to nnz, before the schedule or a kernel indexes with it */
        unsigned int hbad = 0;
        C(sptgb_hicoo_check_bptr(a.bptr, nb, n, a.err + 1, s));
        C(cudaMemcpyAsync(&hbad, a.err + 1, sizeof hbad, cudaMemcpyDeviceToHost, s));
        C(cudaStreamSynchronize(s));
        if (hbad) {
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "inconsistent HiCOO arrays");
            r = SPTERR_VALUE_ERROR;
            goto out;
        }
    }
    SPTGB_TRACE_POINT("bptr check", s, t_prev);
    /* orders 3 and 4: output-window schedule of this mode, then the window kernel */
    if ((N == 3 || N == 4) && nb && n < 0xffffffffull && ((size_t)1 << h->sb_bits) * stride * 4 <= 200 * 1024) {
        sptgb_hicoo_sched_scratch w;
        for (int i = 0; i < 2; ++i) {
            H(sptgb_dbuf_reserve(&g_ws.keys[i], nb * 4));
            H(sptgb_dbuf_reserve(&g_ws.perm[i], nb * 4));
            w.keys[i] = (uint32_t *)g_ws.keys[i].ptr;
            w.vals[i] = (uint32_t *)g_ws.perm[i].ptr;
        }
        H(sptgb_dbuf_reserve(&g_ws.rtmp, sptgb_radix_tmp_bytes(nb)));
        H(sptgb_dbuf_reserve(&g_ws.misc[2], (2 * nb + 1) * 4));
        H(sptgb_dbuf_reserve(&g_ws.misc[3], (2 * nb + 1) * 4));
        H(sptgb_dbuf_reserve(&g_ws.misc[4], (2 * nb + 1) * 8));
        H(sptgb_dbuf_reserve(&g_ws.misc[5], sptgb_scan_tmp_bytes(nb)));
        w.rtmp = g_ws.rtmp.ptr;
        w.stmp = g_ws.misc[5].ptr;
        w.flags = (uint32_t *)g_ws.misc[2].ptr;
        w.pos = w.flags + nb;
        uint32_t *perm = (uint32_t *)g_ws.misc[3].ptr, *pnnz = perm + nb;
        const uint32_t maxb = h->ndims[mode] ? (h->ndims[mode] - 1) >> h->sb_bits : 0;
        uint32_t nwin = 0, nheavy = 0;
        uint64_t *wst = (uint64_t *)g_ws.misc[4].ptr;
        a.heavy_nnz = sptgb_hicoo_heavy_nnz(a.nnz);
        C(sptgb_hicoo_schedule(a.binds[mode], a.bptr, nb, sptgb_bitwidth(maxb), a.heavy_nnz, &w, perm, pnnz, wst,
                               &nwin, wst + nb + 1, &nheavy, s));
        a.perm = perm;
        a.pnnz = pnnz;
        a.wst = wst;
        a.nwin = nwin;
        a.heavy = wst + nb + 1;
        a.nheavy = nheavy;
    }
    SPTGB_TRACE_POINT("schedule", s, t_prev);
    C(cudaMemsetAsync(a.err, 0, sizeof(unsigned int), s));
    if (g_hicoo_timing) C(cudaEventRecord(g_hicoo_ev[0], s));
    C(sptgb_mttkrp_hicoo(&a, s));
    if (g_hicoo_timing) C(cudaEventRecord(g_hicoo_ev[1], s));
    SPTGB_TRACE_POINT("kernel", s, t_prev);
    unsigned int herr = 0;
    C(cudaMemcpyAsync(&herr, a.err, sizeof herr, cudaMemcpyDeviceToHost, s));
    if (tmpI) C(cudaMemcpyAsync(mats[N]->values, g_ws.out.ptr, (size_t)tmpI * stride * 4, cudaMemcpyDeviceToHost, s));
    C(cudaStreamSynchronize(s));
    if (g_hicoo_timing) C(cudaEventElapsedTime(&g_hicoo_ms, g_hicoo_ev[0], g_hicoo_ev[1]));
    SPTGB_TRACE_POINT("d2h out", s, t_prev);
    if (herr) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                          "a coordinate is not smaller than its mode size");
        r = SPTERR_VALUE_ERROR;
    }
out:
    sptgb_unlock();
    return r;
}

int sptMTTKRPHiCOO(sptSparseTensorHiCOO const *const hitsr, sptMatrix *mats[], sptIndex const mats_order[],
                   sptIndex const mode) {
    return hicoo_mttkrp(hitsr, mats, mats_order, mode, "GPU HiCOO SpTns MTTKRP");
}

int sptOmpMTTKRPHiCOO(sptSparseTensorHiCOO const *const hitsr, sptMatrix *mats[], sptIndex const mats_order[],
                      sptIndex const mode, const int nt) {
    (void)nt;
    return hicoo_mttkrp(hitsr, mats, mats_order, mode, "GPU HiCOO SpTns MTTKRP");
}

/* Rank-matrix factors and output, viewed as sptMatrix over the same rows. */
static int hicoo_mttkrp_rank(sptSparseTensorHiCOO const *h, sptRankMatrix *mats[], sptIndex const *mats_order,
                             sptIndex mode) {
    const char *module = "GPU HiCOO SpTns MTTKRP";
    const sptIndex N = h->nmodes;
    if (N < 2 || N > SPTGB_MAX_MODES) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order");
        return SPTERR_VALUE_ERROR;
    }
    sptMatrix view[SPTGB_MAX_MODES + 1];
    sptMatrix *pv[SPTGB_MAX_MODES + 1];
    for (sptIndex i = 0; i <= N; ++i) {
        view[i].nrows = mats[i]->nrows;
        view[i].ncols = mats[i]->ncols;
        view[i].cap = mats[i]->cap;
        view[i].stride = mats[i]->stride;
        view[i].values = mats[i]->values;
        pv[i] = &view[i];
    }
    return hicoo_mttkrp(h, pv, mats_order, mode, module);
}

int sptMTTKRPHiCOO_MatrixTiling(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                sptIndex const mats_order[], sptIndex const mode) {
    return hicoo_mttkrp_rank(hitsr, mats, mats_order, mode);
}

int sptOmpMTTKRPHiCOO_MatrixTiling(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                   sptIndex const mats_order[], sptIndex const mode, const int nt) {
    (void)nt;
    return hicoo_mttkrp_rank(hitsr, mats, mats_order, mode);
}

int sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                             sptIndex const mats_order[], sptIndex const mode, const int tk,
                                             int balanced) {
    (void)tk;
    (void)balanced;
    return hicoo_mttkrp_rank(hitsr, mats, mats_order, mode);
}

int sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                                    sptRankMatrix *copy_mats[], sptIndex const mats_order[],
                                                    sptIndex const mode, const int tk, int balanced) {
    (void)copy_mats;
    (void)tk;
    (void)balanced;
    return hicoo_mttkrp_rank(hitsr, mats, mats_order, mode);
}

/* ------------------------------------------------ resident HiCOO tensor -- */
static int hicoo_window_ok(const sptgbHicoo *t, sptIndex stride) {
    return (t->nmodes == 3 || t->nmodes == 4) && t->nb && t->nnz < 0xffffffffull &&
           ((size_t)1 << t->sb_bits) * stride * 4 <= 200 * 1024;
}

void sptgbHicooFree(sptgbHicoo *t) {
    if (!t) return;
    if (t->bptr) cudaFree(t->bptr);
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) {
        if (t->binds[m]) cudaFree(t->binds[m]);
        if (t->einds[m]) cudaFree(t->einds[m]);
        if (t->perm[m]) cudaFree(t->perm[m]);
        if (t->wst[m]) cudaFree(t->wst[m]);
    }
    if (t->vals) cudaFree(t->vals);
    if (t->err) cudaFree(t->err);
    free(t);
}

size_t sptgbHicooDeviceBytes(const sptgbHicoo *t) { return t ? t->bytes : 0; }

int sptgbHicooCreate(sptgbHicoo **out, const sptSparseTensorHiCOO *h, void *stream) {
    const char *module = "GPU HiCOO create";
    *out = NULL;
    const sptIndex N = h->nmodes;
    if (N < 2 || N > SPTGB_MAX_MODES || h->sb_bits > 8) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order or block size");
        return SPTERR_VALUE_ERROR;
    }
    const uint64_t nb = h->bptr.len ? h->bptr.len - 1 : 0, n = h->nnz;
    int bad = h->values.len < n || (nb && (h->bptr.data[0] != 0 || h->bptr.data[nb] != n));
    for (uint64_t b = 0; b < nb && !bad; ++b) bad = h->bptr.data[b + 1] < h->bptr.data[b];
    for (sptIndex m = 0; m < N && !bad; ++m) bad = h->binds[m].len < nb || h->einds[m].len < n;
    if (bad) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "inconsistent HiCOO arrays");
        return SPTERR_VALUE_ERROR;
    }
    SPTGB_CHECK(sptgb_ctx(), module);
    const cudaStream_t s = stream ? (cudaStream_t)stream : 0;
    sptgbHicoo *t = (sptgbHicoo *)calloc(1, sizeof *t);
    if (!t) return SPTERR_OS_ERROR;
    t->nmodes = N;
    for (sptIndex m = 0; m < N; ++m) t->ndims[m] = h->ndims[m];
    t->nnz = n;
    t->nb = nb;
    t->sb_bits = h->sb_bits;
    int r = 0;
    cudaError_t e = cudaMalloc((void **)&t->bptr, (nb + 1) * 8);
    if (e == cudaSuccess) e = cudaMalloc((void **)&t->vals, (n ? n : 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&t->err, 16);
    for (sptIndex m = 0; m < N && e == cudaSuccess; ++m) {
        e = cudaMalloc((void **)&t->binds[m], (nb ? nb : 1) * 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&t->einds[m], n ? n : 1);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(t->bptr, h->bptr.data, (nb + 1) * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(t->vals, h->values.data, n * 4, cudaMemcpyHostToDevice, s);
    for (sptIndex m = 0; m < N && e == cudaSuccess; ++m) {
        if (nb) e = cudaMemcpyAsync(t->binds[m], h->binds[m].data, nb * 4, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && n) e = cudaMemcpyAsync(t->einds[m], h->einds[m].data, n, cudaMemcpyHostToDevice, s);
    }
    t->bytes = (nb + 1) * 8 + n * 4 + (size_t)N * (nb * 4 + n);
    /* every element inside its mode, element offsets below 2^sb */
    if (e == cudaSuccess) e = cudaMemsetAsync(t->err, 0, 16, s);
    if (e == cudaSuccess && nb) {
        sptgb_hicoo_args a;
        memset(&a, 0, sizeof a);
        a.bptr = t->bptr;
        for (sptIndex m = 0; m < N; ++m) {
            a.binds[m] = t->binds[m];
            a.einds[m] = t->einds[m];
            a.ndims[m] = t->ndims[m];
        }
        a.nmodes = N;
        a.nb = nb;
        a.sb_bits = (uint32_t)t->sb_bits;
        a.err = t->err;
        e = sptgb_hicoo_check(&a, s);
    }
    unsigned int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, t->err, sizeof herr, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
    else if (herr) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "a coordinate is not smaller than its mode size");
        r = SPTERR_VALUE_ERROR;
    }
    if (r) {
        sptgbHicooFree(t);
        return r;
    }
    *out = t;
    return 0;
}

int sptgbHicooPrepareMode(sptgbHicoo *t, sptIndex mode, void *stream) {
    const char *module = "GPU HiCOO prepare";
    if (mode >= t->nmodes) return SPTERR_VALUE_ERROR;
    if (t->ready[mode] || !hicoo_window_ok(t, 8)) return 0;
    const cudaStream_t s = stream ? (cudaStream_t)stream : 0;
    const uint64_t nb = t->nb;
    cudaError_t e = cudaMalloc((void **)&t->perm[mode], (2 * nb + 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&t->wst[mode], (2 * nb + 1) * 8);
    if (e != cudaSuccess) return sptgb_cuda_fail(e, module, __FILE__, __LINE__);
    t->pnnz[mode] = t->perm[mode] + nb;
    t->bytes += (2 * nb + 1) * 4 + (2 * nb + 1) * 8;
    int r = 0;
    sptgb_lock();
    sptgb_hicoo_sched_scratch w;
    for (int i = 0; i < 2 && !r; ++i) {
        r = sptgb_dbuf_reserve(&g_ws.keys[i], nb * 4);
        if (!r) r = sptgb_dbuf_reserve(&g_ws.perm[i], nb * 4);
        w.keys[i] = (uint32_t *)g_ws.keys[i].ptr;
        w.vals[i] = (uint32_t *)g_ws.perm[i].ptr;
    }
    if (!r) r = sptgb_dbuf_reserve(&g_ws.rtmp, sptgb_radix_tmp_bytes(nb));
    if (!r) r = sptgb_dbuf_reserve(&g_ws.misc[2], (2 * nb + 1) * 4);
    if (!r) r = sptgb_dbuf_reserve(&g_ws.misc[5], sptgb_scan_tmp_bytes(nb));
    if (!r) {
        w.rtmp = g_ws.rtmp.ptr;
        w.stmp = g_ws.misc[5].ptr;
        w.flags = (uint32_t *)g_ws.misc[2].ptr;
        w.pos = w.flags + nb;
        const uint32_t maxb = t->ndims[mode] ? (t->ndims[mode] - 1) >> t->sb_bits : 0;
        e = sptgb_hicoo_schedule(t->binds[mode], t->bptr, nb, sptgb_bitwidth(maxb), sptgb_hicoo_heavy_nnz(t->nnz), &w,
                                 t->perm[mode], t->pnnz[mode], t->wst[mode], &t->nwin[mode], t->wst[mode] + nb + 1,
                                 &t->nheavy[mode], s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
    }
    sptgb_unlock();
    if (!r) t->ready[mode] = 1;
    return r;
}

int sptgbHicooMTTKRP(sptgbHicoo *t, sptIndex mode, const sptIndex *mats_order, const float *const *d_mats,
                     sptIndex rank, sptIndex stride, float *d_out, void *stream) {
    const char *module = "GPU HiCOO MTTKRP";
    const sptIndex N = t->nmodes;
    if (mode >= N || rank < 1 || stride % 8 || stride > 128 || rank > stride) return SPTERR_VALUE_ERROR;
    for (sptIndex i = 1; i < N; ++i)
        if (mats_order[i] >= N) return SPTERR_VALUE_ERROR;
    const cudaStream_t s = stream ? (cudaStream_t)stream : 0;
    if (hicoo_window_ok(t, stride) && !t->ready[mode]) SPTGB_CHECK(sptgbHicooPrepareMode(t, mode, stream), module);
    sptgb_hicoo_args a;
    memset(&a, 0, sizeof a);
    a.bptr = t->bptr;
    for (sptIndex m = 0; m < N; ++m) {
        a.binds[m] = t->binds[m];
        a.einds[m] = t->einds[m];
        a.ndims[m] = t->ndims[m];
        a.fac[m] = d_mats[m];
    }
    a.vals = t->vals;
    a.out = d_out;
    a.nb = t->nb;
    a.out_rows = t->ndims[mode];
    a.nmodes = N;
    a.mode = mode;
    for (sptIndex i = 0; i < N; ++i) a.order[i] = mats_order[i];
    a.rank = rank;
    a.stride = stride;
    a.sb_bits = (uint32_t)t->sb_bits;
    a.err = t->err + 1;   /* checked once at creation; this flag is not read */
    a.nnz = t->nnz;
    if (hicoo_window_ok(t, stride)) {
        a.perm = t->perm[mode];
        a.pnnz = t->pnnz[mode];
        a.wst = t->wst[mode];
        a.nwin = t->nwin[mode];
        a.heavy = t->wst[mode] + t->nb + 1;
        a.nheavy = t->nheavy[mode];
        a.heavy_nnz = sptgb_hicoo_heavy_nnz(t->nnz);
    }
    SPTGB_CUDA(sptgb_mttkrp_hicoo(&a, s), module);
    return 0;
}
