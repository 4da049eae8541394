/*
 * Page-locking of caller host arrays (extension; the reference has no such
 * call).  A tensor or matrix that a caller passes to many host-buffer calls
 * can be registered once; the copies of every later call then run as DMA
 * from page-locked memory instead of through the translation of pageable
 * pages.  Registration and release are all-or-nothing per object.
 */
#define _GNU_SOURCE
#include <cuda_runtime_api.h>
#include "devtensor.h"

typedef struct { void *p; size_t bytes; } span;

static int pin_spans(const span *sp, int n, const char *module) {
    SPTGB_CHECK(sptgb_ctx(), module);
    for (int i = 0; i < n; ++i) {
        if (!sp[i].p || !sp[i].bytes) continue;
        const cudaError_t e = cudaHostRegister(sp[i].p, sp[i].bytes, cudaHostRegisterPortable);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();   /* reported here; not left for the next launch check */
            for (int j = 0; j < i; ++j)
                if (sp[j].p && sp[j].bytes) cudaHostUnregister(sp[j].p);
            return sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        }
    }
    return 0;
}

static int unpin_spans(const span *sp, int n, const char *module) {
    SPTGB_CHECK(sptgb_ctx(), module);
    int r = 0;
    for (int i = 0; i < n; ++i) {
        if (!sp[i].p || !sp[i].bytes) continue;
        const cudaError_t e = cudaHostUnregister(sp[i].p);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            if (!r) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        }
    }
    return r;
}

static int tensor_spans(const sptSparseTensor *X, span *sp) {
    int n = 0;
    for (sptIndex m = 0; m < X->nmodes && m < SPTGB_MAX_MODES; ++m) {
        sp[n].p = X->inds[m].data;
        sp[n++].bytes = (size_t)X->nnz * sizeof(sptIndex);
    }
    sp[n].p = X->values.data;
    sp[n++].bytes = (size_t)X->nnz * sizeof(sptValue);
    return n;
}

static int bad_order(const sptSparseTensor *X, const char *module) {
    if (X->nmodes <= SPTGB_MAX_MODES) return 0;
    spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported order");
    return SPTERR_VALUE_ERROR;
}

int sptgbPinSparseTensor(const sptSparseTensor *X) {
    const char *module = "Pin SpTns";
    span sp[SPTGB_MAX_MODES + 1];
    if (bad_order(X, module)) return SPTERR_VALUE_ERROR;
    return pin_spans(sp, tensor_spans(X, sp), module);
}

int sptgbUnpinSparseTensor(const sptSparseTensor *X) {
    const char *module = "Unpin SpTns";
    span sp[SPTGB_MAX_MODES + 1];
    if (bad_order(X, module)) return SPTERR_VALUE_ERROR;
    return unpin_spans(sp, tensor_spans(X, sp), module);
}

int sptgbPinMatrix(const sptMatrix *M) {
    const span sp = {M->values, (size_t)M->cap * M->stride * sizeof(sptValue)};
    return pin_spans(&sp, 1, "Pin Mtx");
}

int sptgbUnpinMatrix(const sptMatrix *M) {
    const span sp = {M->values, (size_t)M->cap * M->stride * sizeof(sptValue)};
    return unpin_spans(&sp, 1, "Unpin Mtx");
}
