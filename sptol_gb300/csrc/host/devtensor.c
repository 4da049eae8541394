/*
 * Device-side tensor handling shared by the drop-in entry points:
 *   - the library workspace (grow-only device buffers, one lock),
 *   - the multi-pass stable device sort that reproduces the reference's
 *     sort orders (src/sptensor/sort.c:410-585),
 *   - the resident COO tensor of the extension API (sptgbCoo*),
 *   - the drop-in sort entry points, which sort a host tensor in place on
 *     the GPU.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

sptgb_workspace g_ws = {PTHREAD_MUTEX_INITIALIZER};

void sptgb_lock(void) { pthread_mutex_lock(&g_ws.lock); }
void sptgb_unlock(void) { pthread_mutex_unlock(&g_ws.lock); }

int sptgb_trace_on(void) {
    static int on = -1;
    if (on < 0) {
        const char *e = getenv("SPTGB_TRACE");
        on = (e && e[0] && e[0] != '0') ? 1 : 0;
    }
    return on;
}

double sptgb_wall(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

int sptgb_ws_sync_objects(void) {
    if (!g_ws.hflag) {
        void *h = NULL;
        SPTGB_CUDA(cudaMallocHost(&h, 16 * sizeof(unsigned int)), "SpTns GPU alloc");
        g_ws.hflag = (unsigned int *)h;
    }
    for (int i = 0; i < 4; ++i)
        if (!g_ws.ev[i]) SPTGB_CUDA(cudaEventCreateWithFlags(&g_ws.ev[i], cudaEventDisableTiming), "SpTns GPU init");
    for (int i = 0; i < 8; ++i)
        if (!g_ws.cev[i]) SPTGB_CUDA(cudaEventCreateWithFlags(&g_ws.cev[i], cudaEventDisableTiming), "SpTns GPU init");
    return 0;
}

int sptgb_bitwidth(uint64_t x) {
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

int sptgb_upload_tensor(const sptSparseTensor *X, sptgb_dbuf *inds, sptgb_dbuf *vals, const int *need,
                        cudaStream_t s) {
    const uint64_t n = X->nnz;
    for (sptIndex m = 0; m < X->nmodes; ++m) {
        if (need && !need[m]) continue;
        SPTGB_CHECK(sptgb_dbuf_reserve(&inds[m], n * sizeof(uint32_t)), "SpTns H2D");
        if (n) SPTGB_CUDA(cudaMemcpyAsync(inds[m].ptr, X->inds[m].data, n * sizeof(uint32_t),
                                          cudaMemcpyHostToDevice, s), "SpTns H2D");
    }
    SPTGB_CHECK(sptgb_dbuf_reserve(vals, n * sizeof(float)), "SpTns H2D");
    if (n) SPTGB_CUDA(cudaMemcpyAsync(vals->ptr, X->values.data, n * sizeof(float), cudaMemcpyHostToDevice, s),
                      "SpTns H2D");
    return 0;
}

int sptgb_validate(uint32_t *const *d_inds, const sptIndex *ndims, int nmodes, uint64_t n,
                   const uint32_t *sorted_check, int *unsorted_out, cudaStream_t s) {
    SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.flag, 2 * sizeof(unsigned int)), "SpTns validate");
    unsigned int *dflag = (unsigned int *)g_ws.flag.ptr;
    SPTGB_CUDA(sptgb_check_bounds((const uint32_t *const *)d_inds, ndims, nmodes, n, dflag, s), "SpTns validate");
    if (sorted_check) SPTGB_CUDA(sptgb_check_sorted(sorted_check, n, dflag + 1, s), "SpTns validate");
    unsigned int h[2] = {0, 0};
    SPTGB_CUDA(cudaMemcpyAsync(h, dflag, sizeof h, cudaMemcpyDeviceToHost, s), "SpTns validate");
    SPTGB_CUDA(cudaStreamSynchronize(s), "SpTns validate");
    if (h[0]) {
        spt_ComplainError("SpTns validate", SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                          "a coordinate is not smaller than its mode size");
        return SPTERR_VALUE_ERROR;
    }
    if (unsorted_out) *unsorted_out = sorted_check ? (int)h[1] : 1;
    return 0;
}

int sptgb_sort_perm(uint32_t *const *d_inds, int nmodes, uint64_t n, const sptgb_sortpass *passes, int npasses,
                    uint32_t **perm_out, cudaStream_t s) {
    for (int b = 0; b < 2; ++b) {
        SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.keys[b], (n ? n : 1) * sizeof(uint32_t)), "SpTns sort");
        SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.perm[b], (n ? n : 1) * sizeof(uint32_t)), "SpTns sort");
    }
    SPTGB_CHECK(sptgb_dbuf_reserve(&g_ws.rtmp, sptgb_radix_tmp_bytes(n)), "SpTns sort");
    uint32_t *keys[2] = {(uint32_t *)g_ws.keys[0].ptr, (uint32_t *)g_ws.keys[1].ptr};
    uint32_t *perm[2] = {(uint32_t *)g_ws.perm[0].ptr, (uint32_t *)g_ws.perm[1].ptr};
    int cur = 0;
    SPTGB_CUDA(sptgb_iota_u32(perm[0], n, 0, s), "SpTns sort");
    for (int p = 0; p < npasses; ++p) {
        if (passes[p].bits <= 0) continue;
        sptgb_keyspec ks;
        memset(&ks, 0, sizeof ks);
        for (int m = 0; m < nmodes; ++m) ks.inds[m] = d_inds[m];
        ks.nmodes = nmodes;
        ks.kind = passes[p].kind;
        ks.mode = passes[p].mode;
        ks.shift = passes[p].shift;
        ks.slice = passes[p].slice;
        SPTGB_CUDA(sptgb_make_keys(&ks, perm[cur], keys[0], n, s), "SpTns sort");
        uint32_t *kk[2] = {keys[0], keys[1]};
        uint32_t *vv[2] = {perm[cur], perm[cur ^ 1]};
        int which = 0;
        SPTGB_CUDA(sptgb_radix_sort_u32(kk, vv, n, passes[p].bits, g_ws.rtmp.ptr, &which, s), "SpTns sort");
        if (which) cur ^= 1;
    }
    *perm_out = perm[cur];
    return 0;
}

int sptgb_lex_passes(const sptIndex *ndims, const sptIndex *order, int nmodes, sptgb_sortpass *passes) {
    int np = 0;
    for (int i = nmodes - 1; i >= 0; --i) {
        const sptIndex m = order[i];
        sptgb_sortpass p = {0, (int)m, 0, 0, sptgb_bitwidth(ndims[m] ? ndims[m] - 1 : 0)};
        passes[np++] = p;
    }
    return np;
}

/* Passes of the HiCOO order: Morton key slices of the full coordinates
 * (least significant first), then the kernel coordinates idx >> sk_bits,
 * lexicographic (convert.c:160-226 = SortIndexRowBlock then per-kernel
 * SortIndexMorton). */
int sptgb_hicoo_passes(const sptIndex *ndims, int nmodes, int sk_bits, int with_kernels, sptgb_sortpass *passes) {
    int np = 0;
    int B = 0;
    for (int m = 0; m < nmodes; ++m) {
        const int b = sptgb_bitwidth(ndims[m] ? ndims[m] - 1 : 0);
        if (b > B) B = b;
    }
    if (nmodes == 3) {
        if (B > 24) B = 24;
        const int bits = 3 * B;
        for (int sl = 0; sl * 32 < bits; ++sl) {
            sptgb_sortpass p = {1, 0, 0, sl, bits - sl * 32 > 32 ? 32 : bits - sl * 32};
            passes[np++] = p;
        }
    } else if (nmodes == 4) {
        for (int sl = 0; sl * 8 < B; ++sl) {
            const int cb = B - sl * 8 > 8 ? 8 : B - sl * 8;
            sptgb_sortpass p = {2, 0, 0, sl, 4 * cb};
            passes[np++] = p;
        }
    }
    if (with_kernels) {
        for (int m = nmodes - 1; m >= 0; --m) {
            const int b = sptgb_bitwidth(ndims[m] ? (ndims[m] - 1) >> sk_bits : 0);
            sptgb_sortpass p = {0, m, sk_bits, 0, b};
            passes[np++] = p;
        }
    }
    return np;
}

/* Morton passes only (sptSparseTensorSortIndexMorton). */
static int morton_passes(const sptIndex *ndims, int nmodes, sptgb_sortpass *passes) {
    return sptgb_hicoo_passes(ndims, nmodes, 0, 0, passes);
}

int sptgb_gather_tensor(uint32_t *const *src_inds, const float *src_vals, uint32_t *const *dst_inds, float *dst_vals,
                        int nmodes, const uint32_t *perm, uint64_t n, cudaStream_t s) {
    for (int m = 0; m < nmodes; ++m)
        if (src_inds[m] && dst_inds[m])
            SPTGB_CUDA(sptgb_gather_u32(src_inds[m], perm, dst_inds[m], n, s), "SpTns gather");
    if (src_vals && dst_vals)
        SPTGB_CUDA(sptgb_gather_u32((const uint32_t *)src_vals, perm, (uint32_t *)dst_vals, n, s), "SpTns gather");
    return 0;
}

/* Sorts the nonzeros [begin, end) of a host tensor in place on the GPU. */
static int sort_host_range(sptSparseTensor *tsr, uint64_t begin, uint64_t end, const sptgb_sortpass *passes,
                           int npasses) {
    if (end <= begin + 1) return 0;
    SPTGB_CHECK(sptgb_ctx(), "SpTns sort");
    const cudaStream_t s = sptgb_stream();
    const uint64_t n = end - begin;
    const int N = (int)tsr->nmodes;
    if (N < 1 || N > SPTGB_MAX_MODES) {
        spt_ComplainError("SpTns sort", SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported tensor order");
        return SPTERR_VALUE_ERROR;
    }
    if (n >= 0xffffffffull) {
        spt_ComplainError("SpTns sort", SPTERR_VALUE_ERROR, __FILE__, __LINE__, "more than 2^32-2 nonzeros");
        return SPTERR_VALUE_ERROR;
    }
    sptgb_lock();
    int r = 0;
    uint32_t *din[SPTGB_MAX_MODES] = {0}, *dout[SPTGB_MAX_MODES] = {0};
    for (int m = 0; m < N && !r; ++m) {
        r = sptgb_dbuf_reserve(&g_ws.inds[m], n * sizeof(uint32_t));
        if (!r) r = sptgb_dbuf_reserve(&g_ws.sinds[m], n * sizeof(uint32_t));
        if (!r) {
            din[m] = (uint32_t *)g_ws.inds[m].ptr;
            dout[m] = (uint32_t *)g_ws.sinds[m].ptr;
            if (cudaMemcpyAsync(din[m], tsr->inds[m].data + begin, n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                s) != cudaSuccess)
                r = sptgb_cuda_fail(cudaGetLastError(), "SpTns sort", __FILE__, __LINE__);
        }
    }
    if (!r) r = sptgb_dbuf_reserve(&g_ws.vals, n * sizeof(float));
    if (!r) r = sptgb_dbuf_reserve(&g_ws.svals, n * sizeof(float));
    if (!r && cudaMemcpyAsync(g_ws.vals.ptr, tsr->values.data + begin, n * sizeof(float), cudaMemcpyHostToDevice,
                              s) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), "SpTns sort", __FILE__, __LINE__);
    uint32_t *perm = NULL;
    if (!r) r = sptgb_validate(din, tsr->ndims, N, n, NULL, NULL, s);
    if (!r) r = sptgb_sort_perm(din, N, n, passes, npasses, &perm, s);
    if (!r) r = sptgb_gather_tensor(din, (float *)g_ws.vals.ptr, dout, (float *)g_ws.svals.ptr, N, perm, n, s);
    for (int m = 0; m < N && !r; ++m)
        if (cudaMemcpyAsync(tsr->inds[m].data + begin, dout[m], n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), "SpTns sort", __FILE__, __LINE__);
    if (!r && cudaMemcpyAsync(tsr->values.data + begin, g_ws.svals.ptr, n * sizeof(float), cudaMemcpyDeviceToHost,
                              s) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), "SpTns sort", __FILE__, __LINE__);
    if (!r) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "SpTns sort", __FILE__, __LINE__);
    }
    sptgb_unlock();
    return r;
}

static int set_identity_order(sptSparseTensor *tsr) {
    int needsort = 0;
    for (sptIndex m = 0; m < tsr->nmodes; ++m)
        if (tsr->sortorder[m] != m) {
            tsr->sortorder[m] = m;
            needsort = 1;
        }
    return needsort;
}

/* sort.c:559-580 */
void sptSparseTensorSortIndex(sptSparseTensor *tsr, int force, int tk) {
    (void)tk;
    const int needsort = set_identity_order(tsr);
    if (!(needsort || force)) return;
    sptIndex order[SPTGB_MAX_MODES];
    for (sptIndex m = 0; m < tsr->nmodes; ++m) order[m] = m;
    sptgb_sortpass passes[SPTGB_MAX_MODES];
    const int np = sptgb_lex_passes(tsr->ndims, order, (int)tsr->nmodes, passes);
    sort_host_range(tsr, 0, tsr->nnz, passes, np);
}

/* sort.c:523-552 */
void sptSparseTensorSortIndexCustomOrder(sptSparseTensor *tsr, sptIndex const *mode_order, int force, int tk) {
    (void)tk;
    const sptIndex N = tsr->nmodes;
    if (!force && memcmp(tsr->sortorder, mode_order, N * sizeof(sptIndex)) == 0) return;
    sptgb_sortpass passes[SPTGB_MAX_MODES];
    const int np = sptgb_lex_passes(tsr->ndims, mode_order, (int)N, passes);
    sort_host_range(tsr, 0, tsr->nnz, passes, np);
    for (sptIndex m = 0; m < N; ++m) tsr->sortorder[m] = mode_order[m];
}

/* sort.c:588-618: all modes but `mode` in order, then `mode`. */
void sptSparseTensorSortIndexAtMode(sptSparseTensor *tsr, sptIndex const mode, int force, int tk) {
    (void)tk;
    const sptIndex N = tsr->nmodes;
    int needsort = 0;
    sptIndex order[SPTGB_MAX_MODES];
    sptIndex k = 0;
    for (sptIndex m = 0; m < N; ++m)
        if (m != mode) order[k++] = m;
    order[N - 1] = mode;
    for (sptIndex m = 0; m < N; ++m)
        if (tsr->sortorder[m] != order[m]) {
            tsr->sortorder[m] = order[m];
            needsort = 1;
        }
    if (!(needsort || force)) return;
    sptgb_sortpass passes[SPTGB_MAX_MODES];
    const int np = sptgb_lex_passes(tsr->ndims, order, (int)N, passes);
    sort_host_range(tsr, 0, tsr->nnz, passes, np);
}

/* sort.c:462-488.  Ties (nonzeros of the same kernel) keep their input
 * order; the reference's quicksort leaves them in an order that depends on
 * its partitioning, so only the kernel order itself is comparable. */
void sptSparseTensorSortIndexRowBlock(sptSparseTensor *tsr, int force, const sptNnzIndex begin,
                                      const sptNnzIndex end, const sptElementIndex sk_bits, int const tk) {
    (void)tk;
    const int needsort = set_identity_order(tsr);
    if (!(needsort || force)) return;
    sptgb_sortpass passes[SPTGB_MAX_MODES];
    int np = 0;
    for (int m = (int)tsr->nmodes - 1; m >= 0; --m) {
        const int b = sptgb_bitwidth(tsr->ndims[m] ? (tsr->ndims[m] - 1) >> sk_bits : 0);
        sptgb_sortpass p = {0, m, sk_bits, 0, b};
        passes[np++] = p;
    }
    sort_host_range(tsr, begin, end, passes, np);
}

/* sort.c:410-454 */
void sptSparseTensorSortIndexMorton(sptSparseTensor *tsr, int force, const sptNnzIndex begin,
                                    const sptNnzIndex end, const sptElementIndex sb_bits, int tk) {
    (void)tk;
    (void)sb_bits;
    const int needsort = set_identity_order(tsr);
    if (!(needsort || force)) return;
    if (tsr->nmodes != 3 && tsr->nmodes != 4) {
        printf("No support for more than 4th-order tensors yet.\n");
        return;
    }
    sptgb_sortpass passes[16];
    const int np = morton_passes(tsr->ndims, (int)tsr->nmodes, passes);
    sort_host_range(tsr, begin, end, passes, np);
}

/* sort.c:283-313: row-block order of kernels, Morton order inside each. */
int sptSparseTensorMixedOrder(sptSparseTensor *tsr, const sptElementIndex sb_bits, const sptElementIndex sk_bits,
                              int const tk) {
    (void)tk;
    (void)sb_bits;
    set_identity_order(tsr);
    sptgb_sortpass passes[24];
    const int np = sptgb_hicoo_passes(tsr->ndims, (int)tsr->nmodes, sk_bits, 1, passes);
    return sort_host_range(tsr, 0, tsr->nnz, passes, np);
}

/* -------------------------------------------- resident COO (sptgb.h) -- */
int sptgbCooCreate(sptgbCoo **out, const sptSparseTensor *X, void *stream) {
    *out = NULL;
    SPTGB_CHECK(sptgb_ctx(), "GPU COO create");
    const cudaStream_t s = (cudaStream_t)stream;
    if (X->nmodes < 2 || X->nmodes > SPTGB_MAX_MODES || X->nnz >= 0xffffffffull) {
        spt_ComplainError("GPU COO create", SPTERR_VALUE_ERROR, __FILE__, __LINE__, "unsupported tensor shape");
        return SPTERR_VALUE_ERROR;
    }
    sptgbCoo *t = (sptgbCoo *)calloc(1, sizeof *t);
    if (!t) return SPTERR_OS_ERROR;
    t->nmodes = X->nmodes;
    t->nnz = X->nnz;
    memcpy(t->ndims, X->ndims, X->nmodes * sizeof(sptIndex));
    const uint64_t n = X->nnz;
    int r = 0;
    for (sptIndex m = 0; m < X->nmodes && !r; ++m) {
        cudaError_t e = cudaMalloc((void **)&t->inds[m], (n ? n : 1) * sizeof(uint32_t));
        if (e == cudaSuccess && n)
            e = cudaMemcpyAsync(t->inds[m], X->inds[m].data, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU COO create", __FILE__, __LINE__);
    }
    if (!r) {
        cudaError_t e = cudaMalloc((void **)&t->vals, (n ? n : 1) * sizeof(float));
        if (e == cudaSuccess && n)
            e = cudaMemcpyAsync(t->vals, X->values.data, n * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU COO create", __FILE__, __LINE__);
    }
    t->bytes = (size_t)n * (X->nmodes + 1) * 4;
    if (!r) {
        sptgb_lock();
        r = sptgb_validate(t->inds, t->ndims, (int)t->nmodes, n, NULL, NULL, s);
        sptgb_unlock();
    }
    if (r) {
        sptgbCooFree(t);
        return r;
    }
    *out = t;
    return 0;
}

int sptgbCooPrepareMode(sptgbCoo *t, sptIndex mode, void *stream) {
    if (mode >= t->nmodes) return SPTERR_VALUE_ERROR;
    if (t->ready[mode]) return 0;
    SPTGB_CHECK(sptgb_ctx(), "GPU COO prepare");
    const cudaStream_t s = (cudaStream_t)stream;
    const uint64_t n = t->nnz;
    const int N = (int)t->nmodes;
    for (int m = 0; m < N; ++m)
        SPTGB_CUDA(cudaMalloc((void **)&t->minds[mode][m], (n ? n : 1) * sizeof(uint32_t)), "GPU COO prepare");
    SPTGB_CUDA(cudaMalloc((void **)&t->mvals[mode], (n ? n : 1) * sizeof(float)), "GPU COO prepare");
    t->bytes += (size_t)n * (N + 1) * 4;
    /* Order: mode first, the other modes ascending (CustomOrder). */
    sptIndex order[SPTGB_MAX_MODES];
    int k = 0;
    order[k++] = mode;
    for (int m = 0; m < N; ++m)
        if ((sptIndex)m != mode) order[k++] = (sptIndex)m;
    sptgb_sortpass passes[SPTGB_MAX_MODES];
    const int np = sptgb_lex_passes(t->ndims, order, N, passes);
    sptgb_lock();
    uint32_t *perm = NULL;
    int r = sptgb_sort_perm(t->inds, N, n, passes, np, &perm, s);
    if (!r) r = sptgb_gather_tensor(t->inds, t->vals, t->minds[mode], t->mvals[mode], N, perm, n, s);
    if (!r && N == 3) {
        /* records {row, idx_a, idx_b, value}, a < b the two other modes */
        const int a = mode == 0 ? 1 : 0, b = mode == 2 ? 1 : 2;
        cudaError_t e = cudaMalloc(&t->mrec[mode], (n ? n : 1) * 16);
        if (e == cudaSuccess)
            e = sptgb_pack_records(t->minds[mode][mode], t->minds[mode][a], t->minds[mode][b], t->mvals[mode],
                                   0xffffffffu, 0xffffffffu, NULL, t->mrec[mode], n, s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU COO prepare", __FILE__, __LINE__);
        t->bytes += (size_t)n * 16;
    }
    if (!r && N == 4) {
        /* records {row, idx_a, idx_b, idx_c}, a < b < c the other modes; the
         * values stay in the mode-sorted value array */
        uint32_t o[3];
        int k3 = 0;
        for (int m = 0; m < 4; ++m)
            if ((sptIndex)m != mode) o[k3++] = (uint32_t)m;
        cudaError_t e = cudaMalloc(&t->mrec[mode], (n ? n : 1) * 16);
        if (e == cudaSuccess)
            e = sptgb_pack_records4(t->minds[mode][mode], t->minds[mode][o[0]], t->minds[mode][o[1]],
                                    t->minds[mode][o[2]], 0xffffffffu, 0xffffffffu, 0xffffffffu, NULL,
                                    t->mrec[mode], n, s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU COO prepare", __FILE__, __LINE__);
        t->bytes += (size_t)n * 16;
    }
    if (!r) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU COO prepare", __FILE__, __LINE__);
    }
    sptgb_unlock();
    if (!r) t->ready[mode] = 1;
    return r;
}

static int coo_mttkrp(sptgbCoo *t, sptIndex mode, const sptIndex *mats_order, const void *const *d_mats,
                      sptIndex rank, sptIndex stride, float *d_out, void *stream, int bf16) {
    if (mode >= t->nmodes) return SPTERR_VALUE_ERROR;
    SPTGB_CHECK(sptgbCooPrepareMode(t, mode, stream), "GPU COO MTTKRP");
    const cudaStream_t s = (cudaStream_t)stream;
    sptgb_mttkrp_args a;
    memset(&a, 0, sizeof a);
    a.rows = t->minds[mode][mode];
    for (sptIndex i = 1; i < t->nmodes; ++i) {
        const sptIndex pm = mats_order[i];
        if (pm >= t->nmodes || pm == mode) return SPTERR_VALUE_ERROR;
        a.idx[i - 1] = t->minds[mode][pm];
        a.fac[i - 1] = d_mats[pm];
    }
    if ((t->nmodes == 3 || t->nmodes == 4) && t->mrec[mode]) {
        /* the records hold the other modes in ascending order */
        int k = 0;
        for (sptIndex m = 0; m < t->nmodes; ++m)
            if (m != mode) a.fac[k++] = d_mats[m];
        a.rec = t->mrec[mode];
    }
    a.vals = t->mvals[mode];
    a.out = d_out;
    a.nnz = t->nnz;
    a.out_rows = t->ndims[mode];
    a.nprod = t->nmodes - 1;
    a.rank = rank;
    a.stride = stride;
    a.bf16 = bf16;
    if (t->timing) {
        if (!t->ev0) {
            cudaEventCreate(&t->ev0);
            cudaEventCreate(&t->ev1);
        }
        cudaEventRecord(t->ev0, s);
    }
    SPTGB_CUDA(sptgb_mttkrp_coo(&a, s), "GPU COO MTTKRP");
    if (t->timing) {
        cudaEventRecord(t->ev1, s);
        cudaEventSynchronize(t->ev1);
        cudaEventElapsedTime(&t->last_ms, t->ev0, t->ev1);
    }
    return 0;
}

int sptgbCooMTTKRP(sptgbCoo *t, sptIndex mode, const sptIndex *mats_order, const float *const *d_mats,
                   sptIndex rank, sptIndex stride, float *d_out, void *stream) {
    return coo_mttkrp(t, mode, mats_order, (const void *const *)d_mats, rank, stride, d_out, stream, 0);
}

int sptgbCooMTTKRPBf16(sptgbCoo *t, sptIndex mode, const sptIndex *mats_order, const uint16_t *const *d_mats_bf16,
                       sptIndex rank, sptIndex stride, float *d_out, void *stream) {
    return coo_mttkrp(t, mode, mats_order, (const void *const *)d_mats_bf16, rank, stride, d_out, stream, 1);
}

int sptgbCooModeArrays(sptgbCoo *t, sptIndex mode, const uint32_t **inds, const float **vals, void *stream) {
    if (mode >= t->nmodes) return SPTERR_VALUE_ERROR;
    SPTGB_CHECK(sptgbCooPrepareMode(t, mode, stream), "GPU COO arrays");
    for (sptIndex m = 0; m < t->nmodes; ++m) inds[m] = t->minds[mode][m];
    *vals = t->mvals[mode];
    return 0;
}

sptNnzIndex sptgbCooNnz(const sptgbCoo *t) { return t->nnz; }
size_t sptgbCooDeviceBytes(const sptgbCoo *t) { return t->bytes; }
void sptgbCooSetTiming(sptgbCoo *t, int enable) { t->timing = enable; }
float sptgbCooLastKernelMs(const sptgbCoo *t) { return t->last_ms; }

void sptgbCooFree(sptgbCoo *t) {
    if (!t) return;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) {
        if (t->inds[m]) cudaFree(t->inds[m]);
        for (int k = 0; k < SPTGB_MAX_MODES; ++k)
            if (t->minds[m][k]) cudaFree(t->minds[m][k]);
        if (t->mvals[m]) cudaFree(t->mvals[m]);
        if (t->mrec[m]) cudaFree(t->mrec[m]);
    }
    if (t->vals) cudaFree(t->vals);
    if (t->ev0) cudaEventDestroy(t->ev0);
    if (t->ev1) cudaEventDestroy(t->ev1);
    free(t);
}
