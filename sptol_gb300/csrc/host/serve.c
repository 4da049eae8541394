/*
 * Batched and served CP-ALS (sptgbServer*, include/sptgb.h).
 *
 * A server owns one device arena of the HBM budget and a table of slots.  A
 * submitted job waits in a FIFO queue until a slot and enough arena space are
 * free; admission then uploads the tensor, builds its mode-sorted 16-byte
 * records on the device (the stable radix sort of the single-tensor path),
 * uploads the initial factors and computes their FP64 Grams and ||X||^2.
 * Every step runs one ALS iteration of all admitted jobs with one launch of a
 * CUDA graph (csrc/cuda/batch.cu: the kernels read device-side work lists, so
 * the graph is captured once and only the lists change with membership) and
 * then completes jobs that reached their iteration count: GetFinalLambda on
 * the device, factors, lambda and per-iteration fits copied into the job's
 * buffers, slot and arena space returned.
 *
 * The first capture times the MTTKRP of each rank group with unit lengths of
 * 64..512 nonzeros on the admitted jobs and keeps the fastest (the autotuner);
 * the chosen lengths are fixed in the captured graph.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

enum { NL_MT = 0, NL_ZR = 16, NL_ONE = 20, NL_DN = 24, NL_FIT = 28, NL_FITONE = 29, NLISTS = 30 };
enum { JOB_QUEUED = 0, JOB_ACTIVE = 1, JOB_DONE = 2, JOB_FAILED = -1 };

typedef struct {
    uint64_t ticket;
    const sptSparseTensor *X;
    sptIndex rank, niters;
    sptMatrix *init[4], *out[4];
    sptValue *lambda;
    double *fits;
    double t_submit, t_done;
    int state;
    int slot;
    size_t bytes;
} job_t;

typedef struct { uint64_t off, len; } span_t;

struct sptgbServer {
    size_t budget, used;
    uint32_t cap;
    char *arena;
    span_t *freel;
    uint32_t nfree, freecap;
    sptgb_slot *hs, *ds;
    int64_t *slot_job;          /* job index per slot, -1 when free */
    uint64_t *slot_off, *slot_len;
    uint32_t *slot_iters;
    job_t *jobs;
    uint64_t njobs, jobcap;
    uint64_t *queue;
    uint64_t nqueue, qcap;
    uint32_t *d_counts, *h_counts, *d_ids, *h_ids;
    uint64_t *d_pre, *h_pre;
    sptgb_step_lists L;
    uint32_t ul[4];
    int tuned;
    cudaStream_t cs;
    cudaGraphExec_t gexec;
    int have_graph;
    int changed;
    uint32_t nactive;
};

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

static size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

/* ------------------------------------------------------------- arena -- */
static int arena_alloc(sptgbServer *s, uint64_t len, uint64_t *off) {
    len = up256(len);
    for (uint32_t i = 0; i < s->nfree; ++i)
        if (s->freel[i].len >= len) {
            *off = s->freel[i].off;
            s->freel[i].off += len;
            s->freel[i].len -= len;
            if (s->freel[i].len == 0) {
                memmove(&s->freel[i], &s->freel[i + 1], (s->nfree - i - 1) * sizeof(span_t));
                --s->nfree;
            }
            s->used += len;
            return 0;
        }
    return SPTERR_NO_MORE;
}

static void arena_free(sptgbServer *s, uint64_t off, uint64_t len) {
    len = up256(len);
    s->used -= len;
    uint32_t i = 0;
    while (i < s->nfree && s->freel[i].off < off) ++i;
    if (s->nfree == s->freecap) {
        s->freecap = s->freecap ? 2 * s->freecap : 64;
        s->freel = (span_t *)realloc(s->freel, s->freecap * sizeof(span_t));
    }
    memmove(&s->freel[i + 1], &s->freel[i], (s->nfree - i) * sizeof(span_t));
    s->freel[i].off = off;
    s->freel[i].len = len;
    ++s->nfree;
    /* merge with the neighbours */
    if (i + 1 < s->nfree && s->freel[i].off + s->freel[i].len == s->freel[i + 1].off) {
        s->freel[i].len += s->freel[i + 1].len;
        memmove(&s->freel[i + 1], &s->freel[i + 2], (s->nfree - i - 2) * sizeof(span_t));
        --s->nfree;
    }
    if (i > 0 && s->freel[i - 1].off + s->freel[i - 1].len == s->freel[i].off) {
        s->freel[i - 1].len += s->freel[i].len;
        memmove(&s->freel[i], &s->freel[i + 1], (s->nfree - i - 1) * sizeof(span_t));
        --s->nfree;
    }
}

/* ------------------------------------------------------ slot layout -- */
typedef struct {
    size_t rec[4], val4[4], fac[4], M, gram[4], S, lambda, ws, fits, normX2, status, total;
} layout_t;

static void layout(const sptSparseTensor *X, uint32_t rank, uint32_t niters, layout_t *L) {
    const uint32_t N = X->nmodes, stride = ((rank - 1) / 8 + 1) * 8;
    const uint64_t n = X->nnz ? X->nnz : 1;
    size_t o = 0;
    uint32_t maxd = 1;
    memset(L, 0, sizeof *L);
    for (uint32_t m = 0; m < N; ++m) {
        L->rec[m] = o;
        o += up256(n * 16);
        if (N == 4) {
            L->val4[m] = o;
            o += up256(n * 4);
        }
    }
    for (uint32_t m = 0; m < N; ++m) {
        L->fac[m] = o;
        o += up256((size_t)(X->ndims[m] ? X->ndims[m] : 1) * stride * 4);
        if (X->ndims[m] > maxd) maxd = X->ndims[m];
    }
    L->M = o;
    o += up256((size_t)maxd * stride * 4);
    for (uint32_t m = 0; m < N; ++m) {
        L->gram[m] = o;
        o += up256((size_t)rank * rank * 8);
    }
    L->S = o;
    o += up256((size_t)rank * rank * 8);
    L->lambda = o;
    o += up256((size_t)rank * 4);
    L->ws = o;
    o += up256(sptgb_dense_ws_bytes((int)rank, 0));
    L->fits = o;
    o += up256((size_t)(niters ? niters : 1) * 8);
    L->normX2 = o;
    o += 256;
    L->status = o;
    o += 256;
    L->total = o;
}

static int group_of(uint32_t stride) {
    const uint32_t c4 = stride / 4;
    return c4 <= 2 ? 0 : c4 <= 4 ? 1 : c4 <= 8 ? 2 : 3;
}

/* ------------------------------------------------------------ lists -- */
static void lists_reset(sptgbServer *s) {
    memset(s->h_counts, 0, NLISTS * sizeof(uint32_t));
    for (int l = 0; l < NLISTS; ++l) s->h_pre[(size_t)l * (s->cap + 1)] = 0;
}

static void lists_add(sptgbServer *s, int l, uint32_t slot, uint64_t items) {
    if (items == 0) return;
    const uint32_t c = s->h_counts[l];
    uint64_t *pre = s->h_pre + (size_t)l * (s->cap + 1);
    s->h_ids[(size_t)l * s->cap + c] = slot;
    pre[c + 1] = pre[c] + items;
    s->h_counts[l] = c + 1;
}

static uint64_t dense_blocks(uint64_t rows, uint32_t per) {
    const uint64_t nb = sptgb_batch_max_blocks();
    uint64_t b = (rows + per - 1) / per;
    if (b > nb) b = nb;
    return b ? b : 1;
}

static void lists_build(sptgbServer *s) {
    lists_reset(s);
    const uint32_t tr = sptgb_batch_rows_per_block(), fr = sptgb_batch_fit_rows_per_block();
    const uint32_t zr = sptgb_batch_zero_rows();
    for (uint32_t i = 0; i < s->cap; ++i) {
        if (s->slot_job[i] < 0) continue;
        const sptgb_slot *d = &s->hs[i];
        const int g = group_of(d->stride);
        for (uint32_t m = 0; m < d->nmodes; ++m) {
            lists_add(s, NL_MT + 4 * (int)m + g, i, (d->nnz + s->ul[g] - 1) / s->ul[g]);
            lists_add(s, NL_ZR + (int)m, i, ((uint64_t)d->ndims[m] + zr - 1) / zr);
            lists_add(s, NL_ONE + (int)m, i, 1);
            lists_add(s, NL_DN + (int)m, i, dense_blocks(d->ndims[m], tr));
        }
        lists_add(s, NL_FIT, i, dense_blocks(d->ndims[d->nmodes - 1], fr));
        lists_add(s, NL_FITONE, i, 1);
    }
}

static int lists_upload(sptgbServer *s) {
    SPTGB_CUDA(cudaMemcpyAsync(s->d_counts, s->h_counts, NLISTS * sizeof(uint32_t), cudaMemcpyHostToDevice, s->cs),
               "GPU server lists");
    SPTGB_CUDA(cudaMemcpyAsync(s->d_ids, s->h_ids, (size_t)NLISTS * s->cap * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               s->cs),
               "GPU server lists");
    SPTGB_CUDA(cudaMemcpyAsync(s->d_pre, s->h_pre, (size_t)NLISTS * (s->cap + 1) * sizeof(uint64_t),
                               cudaMemcpyHostToDevice, s->cs),
               "GPU server lists");
    return 0;
}

static sptgb_wlist wl(sptgbServer *s, int l) {
    sptgb_wlist w = {s->d_counts + l, s->d_ids + (size_t)l * s->cap, s->d_pre + (size_t)l * (s->cap + 1)};
    return w;
}

/* ------------------------------------------------------ admission -- */
static int admit(sptgbServer *s, job_t *j, uint32_t slot) {
    const char *module = "GPU server admit";
    const sptSparseTensor *X = j->X;
    const uint32_t N = X->nmodes, R = j->rank, stride = ((R - 1) / 8 + 1) * 8;
    const uint64_t n = X->nnz;
    layout_t Lo;
    layout(X, R, j->niters, &Lo);
    char *base = s->arena + s->slot_off[slot];
    sptgb_slot *d = &s->hs[slot];
    memset(d, 0, sizeof *d);
    d->nmodes = N;
    d->rank = R;
    d->stride = stride;
    d->nnz = n;
    for (uint32_t m = 0; m < N; ++m) {
        d->ndims[m] = X->ndims[m];
        d->rec[m] = base + Lo.rec[m];
        d->val4[m] = N == 4 ? (const float *)(base + Lo.val4[m]) : NULL;
        d->fac[m] = (float *)(base + Lo.fac[m]);
        d->gram[m] = (double *)(base + Lo.gram[m]);
    }
    d->M = (float *)(base + Lo.M);
    d->S = (double *)(base + Lo.S);
    d->lambda = (float *)(base + Lo.lambda);
    d->ws = (double *)(base + Lo.ws);
    d->fits = (double *)(base + Lo.fits);
    d->normX2 = (double *)(base + Lo.normX2);
    d->status = (int *)(base + Lo.status);
    const cudaStream_t cs = s->cs;
    int r = 0;
    if (n) {
        sptgb_lock();
        uint32_t *din[SPTGB_MAX_MODES] = {0}, *dsrt[SPTGB_MAX_MODES] = {0};
        r = sptgb_upload_tensor(X, g_ws.inds, &g_ws.vals, NULL, cs);
        for (uint32_t m = 0; m < N && !r; ++m) {
            din[m] = (uint32_t *)g_ws.inds[m].ptr;
            r = sptgb_dbuf_reserve(&g_ws.sinds[m], n * 4);
            dsrt[m] = (uint32_t *)g_ws.sinds[m].ptr;
        }
        if (!r) r = sptgb_dbuf_reserve(&g_ws.svals, n * 4);
        if (!r) r = sptgb_validate(din, X->ndims, (int)N, n, NULL, NULL, cs);
        if (!r && sptgb_sumsq((const float *)g_ws.vals.ptr, n, d->normX2, d->ws, cs) != cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
        for (uint32_t m = 0; m < N && !r; ++m) {
            sptIndex order[4];
            uint32_t k = 0, o[3];
            order[k++] = m;
            for (uint32_t q = 0; q < N; ++q)
                if (q != m) order[k++] = q;
            for (uint32_t q = 0; q < N - 1; ++q) o[q] = order[q + 1];
            sptgb_sortpass passes[SPTGB_MAX_MODES];
            const int np = sptgb_lex_passes(X->ndims, order, (int)N, passes);
            uint32_t *perm = NULL;
            r = sptgb_sort_perm(din, (int)N, n, passes, np, &perm, cs);
            if (!r) r = sptgb_gather_tensor(din, (float *)g_ws.vals.ptr, dsrt, (float *)g_ws.svals.ptr, (int)N, perm, n, cs);
            if (r) break;
            cudaError_t e;
            if (N == 3) {
                e = sptgb_pack_records(dsrt[m], dsrt[o[0]], dsrt[o[1]], (const float *)g_ws.svals.ptr,
                                       (void *)d->rec[m], n, cs);
            } else {
                e = sptgb_pack_records4(dsrt[m], dsrt[o[0]], dsrt[o[1]], dsrt[o[2]], (void *)d->rec[m], n, cs);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync((void *)d->val4[m], g_ws.svals.ptr, n * 4, cudaMemcpyDeviceToDevice, cs);
            }
            if (e != cudaSuccess) r = sptgb_cuda_fail(e, module, __FILE__, __LINE__);
        }
        /* the workspace is reused by the next admission: finish with it first */
        if (!r && cudaStreamSynchronize(cs) != cudaSuccess) r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
        sptgb_unlock();
    } else {
        if (cudaMemsetAsync(d->normX2, 0, 8, cs) != cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    }
    for (uint32_t m = 0; m < N && !r; ++m) {
        const size_t bytes = (size_t)X->ndims[m] * stride * 4;
        if (bytes && cudaMemcpyAsync(d->fac[m], j->init[m]->values, bytes, cudaMemcpyHostToDevice, cs) != cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
        if (!r && sptgb_gram(d->fac[m], X->ndims[m], (int)R, (int)stride, d->gram[m], d->ws, cs) != cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    }
    if (!r && cudaMemsetAsync(d->status, 0, 16, cs) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    if (!r && cudaMemcpyAsync(&s->ds[slot], d, sizeof *d, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    return r;
}

static void release(sptgbServer *s, uint32_t slot) {
    arena_free(s, s->slot_off[slot], s->slot_len[slot]);
    s->slot_job[slot] = -1;
    s->changed = 1;
    --s->nactive;
}

/* GetFinalLambda, results into the job's buffers (matrix.c:557-573). */
static int retire(sptgbServer *s, uint32_t slot) {
    const char *module = "GPU server retire";
    job_t *j = &s->jobs[s->slot_job[slot]];
    const sptgb_slot *d = &s->hs[slot];
    int r = 0;
    for (uint32_t m = 0; m < d->nmodes && !r; ++m)
        if (sptgb_colnorm_scale(d->fac[m], d->ndims[m], (int)d->rank, (int)d->stride, d->lambda, d->ws, s->cs) !=
            cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    for (uint32_t m = 0; m < d->nmodes && !r; ++m) {
        const size_t bytes = (size_t)d->ndims[m] * d->stride * 4;
        if (bytes && cudaMemcpyAsync(j->out[m]->values, d->fac[m], bytes, cudaMemcpyDeviceToHost, s->cs) != cudaSuccess)
            r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    }
    if (!r && cudaMemcpyAsync(j->lambda, d->lambda, d->rank * 4, cudaMemcpyDeviceToHost, s->cs) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    if (!r && j->niters &&
        cudaMemcpyAsync(j->fits, d->fits, (size_t)j->niters * 8, cudaMemcpyDeviceToHost, s->cs) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    if (!r && cudaStreamSynchronize(s->cs) != cudaSuccess)
        r = sptgb_cuda_fail(cudaGetLastError(), module, __FILE__, __LINE__);
    j->t_done = now_s();
    j->state = r ? JOB_FAILED : JOB_DONE;
    release(s, slot);
    return r;
}

/* ------------------------------------------------------ autotuning -- */
static int autotune(sptgbServer *s) {
    static const uint32_t cand[4] = {64, 128, 256, 512};
    cudaEvent_t e0, e1;
    SPTGB_CUDA(cudaEventCreate(&e0), "GPU server tune");
    SPTGB_CUDA(cudaEventCreate(&e1), "GPU server tune");
    for (int g = 0; g < 4; ++g) {
        float best = 1e30f;
        uint32_t best_ul = s->ul[g];
        int present = 0;
        for (uint32_t i = 0; i < s->cap && !present; ++i)
            if (s->slot_job[i] >= 0 && group_of(s->hs[i].stride) == g && s->hs[i].nnz) present = 1;
        if (!present) continue;
        for (int c = 0; c < 4; ++c) {
            s->ul[g] = cand[c];
            lists_build(s);
            SPTGB_CHECK(lists_upload(s), "GPU server tune");
            const sptgb_wlist w = wl(s, NL_MT + g);
            float ms = 0.f, tot = 0.f;
            for (int rep = 0; rep < 3; ++rep) {
                cudaEventRecord(e0, s->cs);
                SPTGB_CUDA(sptgb_batch_mttkrp(s->ds, &w, 0, g, cand[c], s->cs), "GPU server tune");
                cudaEventRecord(e1, s->cs);
                SPTGB_CUDA(cudaEventSynchronize(e1), "GPU server tune");
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep) tot += ms;
            }
            if (tot < best) {
                best = tot;
                best_ul = cand[c];
            }
        }
        s->ul[g] = best_ul;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->tuned = 1;
    return 0;
}

static int capture(sptgbServer *s) {
    if (s->have_graph) {
        cudaGraphExecDestroy(s->gexec);
        s->have_graph = 0;
    }
    for (int m = 0; m < 4; ++m) {
        for (int g = 0; g < 4; ++g) s->L.mt[m][g] = wl(s, NL_MT + 4 * m + g);
        s->L.zr[m] = wl(s, NL_ZR + m);
        s->L.one[m] = wl(s, NL_ONE + m);
        s->L.dn[m] = wl(s, NL_DN + m);
    }
    for (int g = 0; g < 4; ++g) s->L.ul[g] = s->ul[g];
    s->L.fit = wl(s, NL_FIT);
    s->L.fit_one = wl(s, NL_FITONE);
    cudaGraph_t graph;
    SPTGB_CUDA(cudaStreamBeginCapture(s->cs, cudaStreamCaptureModeThreadLocal), "GPU server capture");
    cudaError_t e = sptgb_batch_step(s->ds, &s->L, s->cs);
    cudaError_t e2 = cudaStreamEndCapture(s->cs, &graph);
    if (e != cudaSuccess) return sptgb_cuda_fail(e, "GPU server capture", __FILE__, __LINE__);
    SPTGB_CUDA(e2, "GPU server capture");
    e = cudaGraphInstantiate(&s->gexec, graph, 0);
    cudaGraphDestroy(graph);
    SPTGB_CUDA(e, "GPU server capture");
    s->have_graph = 1;
    return 0;
}

/* ------------------------------------------------------------- API -- */
int sptgbServerCreate(sptgbServer **out, size_t hbm_budget_bytes, uint32_t max_slots) {
    *out = NULL;
    SPTGB_CHECK(sptgb_ctx(), "GPU server create");
    if (max_slots == 0 || hbm_budget_bytes < 4096) return SPTERR_VALUE_ERROR;
    sptgbServer *s = (sptgbServer *)calloc(1, sizeof *s);
    if (!s) return SPTERR_OS_ERROR;
    s->budget = up256(hbm_budget_bytes);
    s->cap = max_slots;
    int r = 0;
    cudaError_t e = cudaMalloc((void **)&s->arena, s->budget);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->ds, (size_t)s->cap * sizeof(sptgb_slot));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_counts, NLISTS * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_ids, (size_t)NLISTS * s->cap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_pre, (size_t)NLISTS * (s->cap + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU server create", __FILE__, __LINE__);
    s->hs = (sptgb_slot *)calloc(s->cap, sizeof(sptgb_slot));
    s->slot_job = (int64_t *)malloc(s->cap * sizeof(int64_t));
    s->slot_off = (uint64_t *)calloc(s->cap, sizeof(uint64_t));
    s->slot_len = (uint64_t *)calloc(s->cap, sizeof(uint64_t));
    s->slot_iters = (uint32_t *)calloc(s->cap, sizeof(uint32_t));
    s->h_counts = (uint32_t *)calloc(NLISTS, sizeof(uint32_t));
    s->h_ids = (uint32_t *)calloc((size_t)NLISTS * s->cap, sizeof(uint32_t));
    s->h_pre = (uint64_t *)calloc((size_t)NLISTS * (s->cap + 1), sizeof(uint64_t));
    if (!r && (!s->hs || !s->slot_job || !s->slot_off || !s->slot_len || !s->slot_iters || !s->h_counts || !s->h_ids ||
               !s->h_pre))
        r = SPTERR_OS_ERROR;
    if (r) {
        sptgbServerFree(s);
        return r;
    }
    for (uint32_t i = 0; i < s->cap; ++i) s->slot_job[i] = -1;
    s->freecap = 64;
    s->freel = (span_t *)malloc(s->freecap * sizeof(span_t));
    s->freel[0].off = 0;
    s->freel[0].len = s->budget;
    s->nfree = 1;
    for (int g = 0; g < 4; ++g) s->ul[g] = 256;
    s->changed = 1;
    *out = s;
    return 0;
}

int sptgbServerSubmit(sptgbServer *s, const sptSparseTensor *X, sptIndex rank, sptIndex niters, sptMatrix *const *init,
                      sptMatrix *const *out, sptValue *lambda, double *fits, uint64_t *ticket) {
    const char *module = "GPU server submit";
    if (X->nmodes < 3 || X->nmodes > 4 || rank < 1 || rank > 64 || X->nnz >= 0xffffffffull) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "order 3 or 4 and rank in [1, 64] required");
        return SPTERR_VALUE_ERROR;
    }
    const uint32_t stride = ((rank - 1) / 8 + 1) * 8;
    for (uint32_t m = 0; m < X->nmodes; ++m)
        if (init[m]->nrows != X->ndims[m] || init[m]->stride != stride || out[m]->cap < X->ndims[m] ||
            out[m]->stride != stride) {
            spt_ComplainError(module, SPTERR_SHAPE_MISMATCH, __FILE__, __LINE__, "factor matrix shape");
            return SPTERR_SHAPE_MISMATCH;
        }
    if (s->njobs == s->jobcap) {
        s->jobcap = s->jobcap ? 2 * s->jobcap : 256;
        s->jobs = (job_t *)realloc(s->jobs, s->jobcap * sizeof(job_t));
    }
    if (s->nqueue == s->qcap) {
        s->qcap = s->qcap ? 2 * s->qcap : 256;
        s->queue = (uint64_t *)realloc(s->queue, s->qcap * sizeof(uint64_t));
    }
    job_t *j = &s->jobs[s->njobs];
    memset(j, 0, sizeof *j);
    j->ticket = s->njobs;
    j->X = X;
    j->rank = rank;
    j->niters = niters;
    for (uint32_t m = 0; m < X->nmodes; ++m) {
        j->init[m] = init[m];
        j->out[m] = out[m];
    }
    j->lambda = lambda;
    j->fits = fits;
    j->t_submit = now_s();
    j->state = JOB_QUEUED;
    j->slot = -1;
    layout_t Lo;
    layout(X, rank, niters, &Lo);
    j->bytes = Lo.total;
    s->queue[s->nqueue++] = s->njobs;
    *ticket = s->njobs++;
    return 0;
}

int sptgbServerStep(sptgbServer *s, uint32_t *active, uint32_t *queued) {
    const char *module = "GPU server step";
    SPTGB_CHECK(sptgb_ctx(), module);
    /* admit queued jobs that fit, in submission order */
    uint64_t keep = 0;
    for (uint64_t qi = 0; qi < s->nqueue; ++qi) {
        const uint64_t ji = s->queue[qi];
        job_t *j = &s->jobs[ji];
        int slot = -1;
        for (uint32_t i = 0; i < s->cap; ++i)
            if (s->slot_job[i] < 0) {
                slot = (int)i;
                break;
            }
        uint64_t off = 0;
        if (j->bytes > s->budget) {
            spt_ComplainError(module, SPTERR_NO_MORE, __FILE__, __LINE__, "job larger than the HBM budget");
            j->state = JOB_FAILED;
            j->t_done = now_s();
            continue;
        }
        if (slot < 0 || arena_alloc(s, j->bytes, &off) != 0) {
            s->queue[keep++] = ji;
            continue;
        }
        s->slot_off[slot] = off;
        s->slot_len[slot] = j->bytes;
        s->slot_job[slot] = (int64_t)ji;
        s->slot_iters[slot] = 0;
        ++s->nactive;
        j->slot = slot;
        j->state = JOB_ACTIVE;
        s->changed = 1;
        const int r = admit(s, j, (uint32_t)slot);
        if (r) {
            j->state = JOB_FAILED;
            j->t_done = now_s();
            release(s, (uint32_t)slot);
            continue;
        }
        if (j->niters == 0) SPTGB_CHECK(retire(s, (uint32_t)slot), module);
    }
    s->nqueue = keep;
    if (s->nactive > 0) {
        if (!s->tuned) {
            SPTGB_CHECK(autotune(s), module);
            s->changed = 1;
            if (s->have_graph) {
                cudaGraphExecDestroy(s->gexec);
                s->have_graph = 0;
            }
        }
        if (s->changed) {
            lists_build(s);
            SPTGB_CHECK(lists_upload(s), module);
            s->changed = 0;
        }
        if (!s->have_graph) SPTGB_CHECK(capture(s), module);
        SPTGB_CUDA(cudaGraphLaunch(s->gexec, s->cs), module);
        for (uint32_t i = 0; i < s->cap; ++i) {
            if (s->slot_job[i] < 0) continue;
            if (++s->slot_iters[i] >= s->jobs[s->slot_job[i]].niters) SPTGB_CHECK(retire(s, i), module);
        }
    }
    if (active) *active = s->nactive;
    if (queued) *queued = (uint32_t)s->nqueue;
    return 0;
}

int sptgbServerDone(sptgbServer *s, uint64_t ticket, double *submit_s, double *done_s) {
    if (ticket >= s->njobs) return SPTERR_VALUE_ERROR;
    const job_t *j = &s->jobs[ticket];
    if (submit_s) *submit_s = j->t_submit;
    if (done_s) *done_s = j->t_done;
    if (j->state == JOB_FAILED) return -1;
    return j->state == JOB_DONE ? 1 : 0;
}

int sptgbServerDrain(sptgbServer *s) {
    uint32_t a = 0, q = 0;
    do {
        SPTGB_CHECK(sptgbServerStep(s, &a, &q), "GPU server drain");
    } while (a > 0 || q > 0);
    return 0;
}

size_t sptgbServerBytesInUse(const sptgbServer *s) { return s->used; }

uint32_t sptgbServerUnitLength(const sptgbServer *s, int group) { return group >= 0 && group < 4 ? s->ul[group] : 0; }

void sptgbServerFree(sptgbServer *s) {
    if (!s) return;
    if (s->have_graph) cudaGraphExecDestroy(s->gexec);
    if (s->cs) cudaStreamSynchronize(s->cs);
    if (s->arena) cudaFree(s->arena);
    if (s->ds) cudaFree(s->ds);
    if (s->d_counts) cudaFree(s->d_counts);
    if (s->d_ids) cudaFree(s->d_ids);
    if (s->d_pre) cudaFree(s->d_pre);
    if (s->cs) cudaStreamDestroy(s->cs);
    free(s->hs);
    free(s->slot_job);
    free(s->slot_off);
    free(s->slot_len);
    free(s->slot_iters);
    free(s->h_counts);
    free(s->h_ids);
    free(s->h_pre);
    free(s->freel);
    free(s->jobs);
    free(s->queue);
    free(s);
}
