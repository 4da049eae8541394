/*
 * Sparse tensor times matrix (src/sptensor/mmul.c:37-97) and the semi-sparse
 * containers it produces (src/ssptensor/ssptensor.c:32-95, setinds.c:33-71,
 * src/sptensor/fromssp.c:32-78, src/matrix/matrix.c:200-221).
 *
 * X is sorted at `mode` on the GPU (in place, as the reference does); fiber
 * heads (positions where a coordinate other than `mode` changes) are marked,
 * scanned and compacted on the device; the fiber coordinates and the dense
 * fibers (csrc/cuda/ttm.cu) come back into Y.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

cudaError_t sptgb_ttm(const uint64_t *starts, uint64_t nfib, uint64_t nnz, const uint32_t *rows, const float *vals,
                      const float *U, uint32_t ustride, uint32_t ncols, float *Y, uint32_t ystride, cudaStream_t s);

int sptResizeMatrix(sptMatrix *mtx, sptIndex const new_nrows) {
    sptValue *nd = NULL;
    if (posix_memalign((void **)&nd, 8 * sizeof(sptValue),
                       (size_t)(new_nrows ? new_nrows : 1) * mtx->stride * sizeof(sptValue)) != 0 || !nd) {
        spt_ComplainError("Mtx Resize", SPTERR_OS_ERROR, __FILE__, __LINE__, "allocation failed");
        return SPTERR_OS_ERROR;
    }
    const sptIndex keep = mtx->nrows < new_nrows ? mtx->nrows : new_nrows;
    if (mtx->values && keep) memcpy(nd, mtx->values, (size_t)keep * mtx->stride * sizeof(sptValue));
    free(mtx->values);
    mtx->nrows = new_nrows;
    mtx->cap = new_nrows;
    mtx->values = nd;
    return 0;
}

int sptNewSemiSparseTensor(sptSemiSparseTensor *tsr, sptIndex nmodes, sptIndex mode, const sptIndex ndims[]) {
    if (nmodes < 2) {
        spt_ComplainError("SspTns New", SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "nmodes < 2");
        return SPTERR_SHAPE_MISMATCH;
    }
    tsr->nmodes = nmodes;
    tsr->ndims = (sptIndex *)malloc(nmodes * sizeof(sptIndex));
    tsr->inds = (sptIndexVector *)malloc(nmodes * sizeof(sptIndexVector));
    if (!tsr->ndims || !tsr->inds) return SPTERR_OS_ERROR;
    memcpy(tsr->ndims, ndims, nmodes * sizeof(sptIndex));
    tsr->mode = mode;
    tsr->nnz = 0;
    for (sptIndex i = 0; i < nmodes; ++i) {
        const int r = sptNewIndexVector(&tsr->inds[i], 0, 0);
        if (r) return r;
    }
    tsr->stride = ((ndims[mode] - 1) / 8 + 1) * 8;
    return sptNewMatrix(&tsr->values, 0, tsr->stride);
}

void sptFreeSemiSparseTensor(sptSemiSparseTensor *tsr) {
    for (sptIndex i = 0; i < tsr->nmodes; ++i) sptFreeIndexVector(&tsr->inds[i]);
    free(tsr->ndims);
    free(tsr->inds);
    sptFreeMatrix(&tsr->values);
}

/* fromssp.c:32-78: every finite entry with |v| >= epsilon, NaN and +-inf
 * become nonzeros (subnormals and zeros are dropped), then a lexicographic
 * sort. */
int sptSemiSparseTensorToSparseTensor(sptSparseTensor *dest, const sptSemiSparseTensor *src, sptValue epsilon) {
    const sptIndex N = src->nmodes;
    int r = sptNewSparseTensor(dest, N, src->ndims);
    if (r) return r;
    for (sptNnzIndex i = 0; i < src->nnz; ++i)
        for (sptIndex j = 0; j < src->ndims[src->mode]; ++j) {
            const sptValue data = src->values.values[i * src->stride + j];
            const int cls = fpclassify(data);
            if (cls == FP_NAN || cls == FP_INFINITE || (cls == FP_NORMAL && !(data < epsilon && data > -epsilon))) {
                for (sptIndex m = 0; m < N; ++m) {
                    r = sptAppendIndexVector(&dest->inds[m], m != src->mode ? src->inds[m].data[i] : j);
                    if (r) return r;
                }
                r = sptAppendValueVector(&dest->values, data);
                if (r) return r;
                ++dest->nnz;
            }
        }
    sptSparseTensorSortIndex(dest, 1, 1);
    return 0;
}

int sptCudaSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U, sptIndex const mode) {
    const char *module = "GPU  SpTns * Mtx";
    if (mode >= X->nmodes || X->ndims[mode] != U->nrows) {
        spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "shape mismatch");
        return SPTERR_SHAPE_MISMATCH;
    }
    const sptIndex N = X->nmodes;
    if (N > SPTGB_MAX_MODES) return SPTERR_VALUE_ERROR;
    SPTGB_CHECK(sptgb_ctx(), module);
    sptSparseTensorSortIndexAtMode(X, mode, 0, 1);
    sptIndex ind_buf[SPTGB_MAX_MODES];
    for (sptIndex m = 0; m < N; ++m) ind_buf[m] = X->ndims[m];
    ind_buf[mode] = U->ncols;
    SPTGB_CHECK(sptNewSemiSparseTensor(Y, N, mode, ind_buf), module);
    const uint64_t n = X->nnz;
    if (n == 0) return sptResizeMatrix(&Y->values, 0);
    const cudaStream_t s = sptgb_stream();
    int r = 0;
    sptgb_lock();
    uint32_t nfib = 0;
    do {
        if ((r = sptgb_upload_tensor(X, g_ws.inds, &g_ws.vals, NULL, s))) break;
        uint32_t *din[SPTGB_MAX_MODES];
        for (sptIndex m = 0; m < N; ++m) din[m] = (uint32_t *)g_ws.inds[m].ptr;
        if ((r = sptgb_validate(din, X->ndims, (int)N, n, NULL, NULL, s))) break;
        const uint32_t *other[SPTGB_MAX_MODES];
        int no = 0;
        for (sptIndex m = 0; m < N; ++m)
            if (m != mode) other[no++] = din[m];
        if ((r = sptgb_dbuf_reserve(&g_ws.misc[1], (2 * n + 2) * 4))) break;
        if ((r = sptgb_dbuf_reserve(&g_ws.misc[2], (n + 1) * 8))) break;
        if ((r = sptgb_dbuf_reserve(&g_ws.misc[3], sptgb_scan_tmp_bytes(n)))) break;
        uint32_t *flags = (uint32_t *)g_ws.misc[1].ptr, *pos = flags + n, *dn = pos + n;
        uint64_t *starts = (uint64_t *)g_ws.misc[2].ptr;
        cudaError_t e = sptgb_mark_groups(other, no, 0, n, flags, s);
        if (e == cudaSuccess) e = sptgb_exclusive_scan_u32(flags, pos, n, dn, g_ws.misc[3].ptr, s);
        if (e == cudaSuccess) e = sptgb_compact_starts(flags, pos, n, starts, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&nfib, dn, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
            break;
        }
        /* fiber coordinates of the other modes */
        for (sptIndex m = 0; m < N && !r; ++m) {
            if (m == mode) continue;
            if ((r = sptgb_dbuf_reserve(&g_ws.sinds[m], (uint64_t)nfib * 4))) break;
            e = sptgb_compact_u32(flags, pos, din[m], n, (uint32_t *)g_ws.sinds[m].ptr, s);
            if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        }
        if (r) break;
        /* U and the dense fibers */
        const size_t ub = (size_t)U->nrows * U->stride * 4, yb = (size_t)nfib * Y->stride * 4;
        if ((r = sptgb_dbuf_reserve(&g_ws.fac[0], ub ? ub : 16))) break;
        if ((r = sptgb_dbuf_reserve(&g_ws.out, yb ? yb : 16))) break;
        e = ub ? cudaMemcpyAsync(g_ws.fac[0].ptr, U->values, ub, cudaMemcpyHostToDevice, s) : cudaSuccess;
        if (e == cudaSuccess) e = cudaMemsetAsync(g_ws.out.ptr, 0, yb, s);
        if (e == cudaSuccess)
            e = sptgb_ttm(starts, nfib, n, din[mode], (const float *)g_ws.vals.ptr, (const float *)g_ws.fac[0].ptr,
                          U->stride, U->ncols, (float *)g_ws.out.ptr, Y->stride, s);
        if (e != cudaSuccess) {
            r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
            break;
        }
        if ((r = sptResizeMatrix(&Y->values, nfib))) break;
        for (sptIndex m = 0; m < N && !r; ++m) {
            if (m == mode) continue;
            if ((r = sptResizeIndexVector(&Y->inds[m], nfib))) break;
            e = cudaMemcpyAsync(Y->inds[m].data, g_ws.sinds[m].ptr, (size_t)nfib * 4, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        }
        if (r) break;
        e = cudaMemcpyAsync(Y->values.values, g_ws.out.ptr, yb, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        Y->nnz = nfib;
    } while (0);
    sptgb_unlock();
    return r;
}

int sptSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U, sptIndex const mode) {
    return sptCudaSparseTensorMulMatrix(Y, X, U, mode);
}

int sptOmpSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U, sptIndex const mode) {
    return sptCudaSparseTensorMulMatrix(Y, X, U, mode);
}

int sptCudaSparseTensorMulMatrixOneKernel(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U,
                                          sptIndex const mode, sptIndex const impl_num, sptNnzIndex const smen_size) {
    (void)impl_num;
    (void)smen_size;
    return sptCudaSparseTensorMulMatrix(Y, X, U, mode);
}
