/*
 * Batched and served CP-ALS (sptgbServer*, include/sptgb.h).
 *
 * A server owns one device arena of the HBM budget and a table of slots.  A
 * submitted job waits in a FIFO queue until a slot and enough arena space are
 * free.  Each step then
 *   1. admits, as one group, the queued jobs that fit: their nonzeros are
 *      staged back to back, bounds-checked, and sorted for every mode by one
 *      stable radix sort of (job, row) keys over the whole group; one kernel
 *      writes each job's 16-byte records into its slot; ||X||^2 and the Grams
 *      of the initial factors are computed for all new jobs by work-list
 *      kernels (csrc/cuda/batch.cu), with the same block decomposition as the
 *      single-tensor path;
 *   2. runs one ALS iteration of every admitted job with one launch of a CUDA
 *      graph: the kernels read device-side work lists, so the graph is
 *      captured once and only the lists change with membership;
 *   3. retires jobs that reached their iteration count: GetFinalLambda for all
 *      of them by work-list kernels, then factors, lambda and per-iteration
 *      fits copied into each job's buffers, slot and arena space returned.
 * Slot descriptors are written once at admission (the iteration counter lives
 * in the slot's status words), so membership changes never touch a running
 * job's state.
 *
 * The first time a rank group has admitted jobs, before their first
 * iteration, the autotuner picks the group's MTTKRP schedule: unit length
 * (64..512 nonzeros), record batch depth and the register budget (2 or 3
 * blocks per SM), timed on the admitted jobs of the group; the
 * choice is cached per process by (rank group, dominant order, nonzeros per
 * job rounded to a power of two), so a later server with jobs of the same
 * kind reuses it without timing.  The schedules are launch parameters of the
 * captured graph, which is captured again when a group gets its schedule.
 *
 * Staging buffers of an admission group (coordinates, values, sort keys and
 * permutations, about 40 bytes per nonzero) are outside the budget; a group
 * holds at most SERVE_GROUP_NNZ nonzeros unless a single job is larger.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

/* step lists (fixed positions, captured in the graph) */
enum { NL_MT = 0, NL_ZR = 16, NL_ONE = 20, NL_DN = 24, NL_FIT = 28, NL_FITONE = 29, NL_STEP = 30 };
/* admission lists: ids are group job indices for SQ/SQONE, slot ids for the rest */
enum { NL_SQ = NL_STEP, NL_SQONE = NL_STEP + 1, NL_GDN = NL_STEP + 2, NL_GONE = NL_STEP + 6, NL_ADM_END = NL_STEP + 10 };
/* retirement lists (slot ids) */
enum { NL_RDN = NL_ADM_END, NL_RONE = NL_ADM_END + 4, NLISTS = NL_ADM_END + 8 };
enum { JOB_QUEUED = 0, JOB_ACTIVE = 1, JOB_DONE = 2, JOB_FAILED = -1 };

#define SERVE_GROUP_NNZ (32ull << 20)
#define SERVE_GROUP_JOBS 4096u

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
    uint32_t sched[4];           /* MTTKRP schedule bits per rank group (sptgb_step_lists.sched) */
    int tuned_from_cache[4];     /* 1: the group's schedule came from the process cache, 0: timed, -1: no jobs */
    cudaStream_t cs;
    cudaStream_t as;             /* admission: uploads, checks, sorts of new slots, overlapping the step on cs */
    cudaGraphExec_t gexec;
    int have_graph;
    int persistent;              /* the step graph holds one persistent kernel (1) or the kernel sequence (0) */
    uint32_t graph_kernels;      /* kernels in the step graph */
    sptgb_grid_bar *bar;         /* its grid barrier (device) */
    int changed;
    uint32_t nactive;
    /* admission group */
    uint32_t *grp;               /* job indices */
    sptgb_adm_job *h_gjobs;
    uint64_t *h_goffs;
    unsigned int *h_gerr;
    sptgb_dbuf st_ind[4], st_val, keys[2], perm[2], rtmp, d_gjobs, d_goffs, d_gerr;
    uint32_t *ret;               /* retiring slots */
    uint64_t *fin;               /* completion queue: tickets in completion order */
    uint64_t nfin, fincap, finread;
    /* SPTGB_TRACE=1: wall time per phase, printed by sptgbServerFree */
    int trace;
    double t_select, t_admit_host, t_admit_h2d, t_admit_dev, t_step, t_retire;
    uint64_t n_groups, n_steps, n_retire_calls;
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
        s->freecap *= 2;
        s->freel = (span_t *)realloc(s->freel, s->freecap * sizeof(span_t));
    }
    memmove(&s->freel[i + 1], &s->freel[i], (s->nfree - i) * sizeof(span_t));
    s->freel[i].off = off;
    s->freel[i].len = len;
    ++s->nfree;
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
    size_t rec[4], val4[4], fac[4], M, gram[4], S, lambda, ws, fits, status, normX2, total;
} layout_t;

static uint32_t stride_of(uint32_t rank) { return ((rank - 1) / 8 + 1) * 8; }

static void layout(const sptSparseTensor *X, uint32_t rank, uint32_t niters, layout_t *L) {
    const uint32_t N = X->nmodes, stride = stride_of(rank);
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
    L->status = o;
    o += 256;
    L->normX2 = o;
    o += 256;
    L->total = o;
}

static int group_of(uint32_t stride) {
    const uint32_t c4 = stride / 4;
    return c4 <= 2 ? 0 : c4 <= 4 ? 1 : c4 <= 8 ? 2 : 3;
}

/* ------------------------------------------------------------ lists -- */
static void list_clear(sptgbServer *s, int l) {
    s->h_counts[l] = 0;
    s->h_pre[(size_t)l * (s->cap + 1)] = 0;
}

static void list_add(sptgbServer *s, int l, uint32_t id, uint64_t items) {
    if (items == 0) return;
    const uint32_t c = s->h_counts[l];
    uint64_t *pre = s->h_pre + (size_t)l * (s->cap + 1);
    s->h_ids[(size_t)l * s->cap + c] = id;
    pre[c + 1] = pre[c] + items;
    s->h_counts[l] = c + 1;
}

/* Uploads lists [l0, l1). */
static int lists_upload(sptgbServer *s, int l0, int l1, cudaStream_t st) {
    const char *module = "GPU server lists";
    SPTGB_CUDA(cudaMemcpyAsync(s->d_counts + l0, s->h_counts + l0, (size_t)(l1 - l0) * 4, cudaMemcpyHostToDevice, st),
               module);
    SPTGB_CUDA(cudaMemcpyAsync(s->d_ids + (size_t)l0 * s->cap, s->h_ids + (size_t)l0 * s->cap,
                               (size_t)(l1 - l0) * s->cap * 4, cudaMemcpyHostToDevice, st),
               module);
    SPTGB_CUDA(cudaMemcpyAsync(s->d_pre + (size_t)l0 * (s->cap + 1), s->h_pre + (size_t)l0 * (s->cap + 1),
                               (size_t)(l1 - l0) * (s->cap + 1) * 8, cudaMemcpyHostToDevice, st),
               module);
    return 0;
}

static sptgb_wlist wl(sptgbServer *s, int l) {
    sptgb_wlist w = {s->d_counts + l, s->d_ids + (size_t)l * s->cap, s->d_pre + (size_t)l * (s->cap + 1)};
    return w;
}

static uint64_t clamp_blocks(uint64_t rows, uint32_t per) {
    const uint64_t nb = sptgb_batch_max_blocks();
    uint64_t b = (rows + per - 1) / per;
    if (b > nb) b = nb;
    return b ? b : 1;
}

/* Row blocks of a slot's solve for mode m: eight TR-row tiles each (enough
 * to amortise the per-block setup, small enough to balance many slots over
 * the persistent grid), at most the partial space NBLK.  The split depends
 * only on the slot's own shape, so a job's arithmetic does not change with
 * the mix it runs in. */
static uint64_t solve_items(uint64_t rows, uint32_t tr) { return clamp_blocks(rows, 8 * tr); }

static void step_lists_build(sptgbServer *s) {
    for (int l = 0; l < NL_STEP; ++l) list_clear(s, l);
    const uint32_t fr = sptgb_batch_fit_rows_per_block();
    const uint32_t zr = sptgb_batch_zero_rows();
    for (uint32_t i = 0; i < s->cap; ++i) {
        if (s->slot_job[i] < 0 || s->jobs[s->slot_job[i]].state != JOB_ACTIVE) continue;
        const sptgb_slot *d = &s->hs[i];
        const int g = group_of(d->stride);
        for (uint32_t m = 0; m < d->nmodes; ++m) {
            list_add(s, NL_MT + 4 * (int)m + g, i, (d->nnz + s->ul[g] - 1) / s->ul[g]);
            list_add(s, NL_ZR + (int)m, i, ((uint64_t)d->ndims[m] + zr - 1) / zr);
            list_add(s, NL_ONE + (int)m, i, 1);
            list_add(s, NL_DN + (int)m, i, solve_items(d->ndims[m], sptgb_batch_solve_tile_rows(d->rank)));
        }
        list_add(s, NL_FIT, i, clamp_blocks(d->ndims[d->nmodes - 1], fr));
        list_add(s, NL_FITONE, i, 1);
    }
}

/* ------------------------------------------------------ admission -- */
static void fill_descriptor(sptgbServer *s, uint32_t slot, const job_t *j) {
    const sptSparseTensor *X = j->X;
    const uint32_t N = X->nmodes;
    layout_t Lo;
    layout(X, j->rank, j->niters, &Lo);
    char *base = s->arena + s->slot_off[slot];
    sptgb_slot *d = &s->hs[slot];
    memset(d, 0, sizeof *d);
    d->nmodes = N;
    d->rank = j->rank;
    d->stride = stride_of(j->rank);
    d->nnz = X->nnz;
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
}

static int sort_group_mode(sptgbServer *s, const sptgb_adm_group *g, int mode, int jbits, int rowbits,
                           uint32_t **perm_out) {
    const char *module = "GPU server admit";
    const uint64_t n = g->total;
    uint32_t *keys[2] = {(uint32_t *)s->keys[0].ptr, (uint32_t *)s->keys[1].ptr};
    uint32_t *perm[2] = {(uint32_t *)s->perm[0].ptr, (uint32_t *)s->perm[1].ptr};
    int cur = 0;
    SPTGB_CUDA(sptgb_iota_u32(perm[0], n, 0, s->as), module);
    /* (job, row) in one key when it fits in 32 bits, else row then job */
    int kinds[2], bits[2], np = 0;
    if (jbits + rowbits <= 32) {
        kinds[np] = 0;
        bits[np++] = jbits + rowbits;
    } else {
        kinds[np] = 1;
        bits[np++] = rowbits;
        kinds[np] = 2;
        bits[np++] = jbits;
    }
    for (int p = 0; p < np; ++p) {
        if (bits[p] == 0) continue;
        SPTGB_CUDA(sptgb_adm_keys(g, mode, rowbits, kinds[p], p ? perm[cur] : NULL, keys[0], s->as), module);
        uint32_t *kk[2] = {keys[0], keys[1]};
        uint32_t *vv[2] = {perm[cur], perm[cur ^ 1]};
        int which = 0;
        SPTGB_CUDA(sptgb_radix_sort_u32(kk, vv, n, bits[p], s->rtmp.ptr, &which, s->as), module);
        if (which) cur ^= 1;
    }
    *perm_out = perm[cur];
    return 0;
}

static void release(sptgbServer *s, uint32_t slot) {
    arena_free(s, s->slot_off[slot], s->slot_len[slot]);
    s->slot_job[slot] = -1;
    s->changed = 1;
    --s->nactive;
}

static void push_completed(sptgbServer *s, uint64_t ticket) {
    if (s->nfin == s->fincap) {
        s->fincap = s->fincap ? 2 * s->fincap : 256;
        s->fin = (uint64_t *)realloc(s->fin, s->fincap * sizeof(uint64_t));
    }
    s->fin[s->nfin++] = ticket;
}

static void fail_job(sptgbServer *s, job_t *j) {
    push_completed(s, j->ticket);
    j->state = JOB_FAILED;
    j->t_done = now_s();
    if (j->slot >= 0) release(s, (uint32_t)j->slot);
    j->slot = -1;
}

/* Admits the group s->grp[0..G) (slots and arena space already reserved). */
static int admit_group(sptgbServer *s, uint32_t G) {
    const char *module = "GPU server admit";
    const cudaStream_t cs = s->as;   /* the step graph may be running on s->cs */
    uint64_t total = 0;
    uint32_t lo = s->cap, hi = 0;
    int maxN = 0, rowbits[4] = {0, 0, 0, 0};
    for (uint32_t q = 0; q < G; ++q) {
        job_t *j = &s->jobs[s->grp[q]];
        const sptSparseTensor *X = j->X;
        fill_descriptor(s, (uint32_t)j->slot, j);
        if ((uint32_t)j->slot < lo) lo = (uint32_t)j->slot;
        if ((uint32_t)j->slot > hi) hi = (uint32_t)j->slot;
        sptgb_adm_job *a = &s->h_gjobs[q];
        memset(a, 0, sizeof *a);
        a->off = total;
        a->n = X->nnz;
        a->slot = (uint32_t)j->slot;
        a->nmodes = X->nmodes;
        for (uint32_t m = 0; m < X->nmodes; ++m) {
            a->ndims[m] = X->ndims[m];
            const int b = sptgb_bitwidth(X->ndims[m] ? X->ndims[m] - 1 : 0);
            if (b > rowbits[m]) rowbits[m] = b;
        }
        if ((int)X->nmodes > maxN) maxN = (int)X->nmodes;
        s->h_goffs[q] = total;
        total += X->nnz;
    }
    s->h_goffs[G] = total;
    const int jbits = sptgb_bitwidth(G - 1);
    double t0 = s->trace ? now_s() : 0.0;

    /* descriptors of the new slots (a contiguous range; other slots in it are rewritten unchanged) */
    SPTGB_CUDA(cudaMemcpyAsync(&s->ds[lo], &s->hs[lo], (size_t)(hi - lo + 1) * sizeof(sptgb_slot),
                               cudaMemcpyHostToDevice, cs),
               module);

    /* staging */
    const uint64_t nn = total ? total : 1;
    for (int m = 0; m < maxN; ++m) SPTGB_CHECK(sptgb_dbuf_reserve(&s->st_ind[m], nn * 4), module);
    SPTGB_CHECK(sptgb_dbuf_reserve(&s->st_val, nn * 4), module);
    for (int b = 0; b < 2; ++b) {
        SPTGB_CHECK(sptgb_dbuf_reserve(&s->keys[b], nn * 4), module);
        SPTGB_CHECK(sptgb_dbuf_reserve(&s->perm[b], nn * 4), module);
    }
    SPTGB_CHECK(sptgb_dbuf_reserve(&s->rtmp, sptgb_radix_tmp_bytes(nn)), module);
    SPTGB_CHECK(sptgb_dbuf_reserve(&s->d_gjobs, (size_t)G * sizeof(sptgb_adm_job)), module);
    SPTGB_CHECK(sptgb_dbuf_reserve(&s->d_goffs, (size_t)(G + 1) * 8), module);
    SPTGB_CHECK(sptgb_dbuf_reserve(&s->d_gerr, (size_t)G * 4), module);
    for (uint32_t q = 0; q < G; ++q) {
        const job_t *j = &s->jobs[s->grp[q]];
        const sptSparseTensor *X = j->X;
        const uint64_t off = s->h_goffs[q], n = X->nnz;
        if (!n) continue;
        for (uint32_t m = 0; m < X->nmodes; ++m)
            SPTGB_CUDA(cudaMemcpyAsync((uint32_t *)s->st_ind[m].ptr + off, X->inds[m].data, n * 4,
                                       cudaMemcpyHostToDevice, cs),
                       module);
        SPTGB_CUDA(cudaMemcpyAsync((float *)s->st_val.ptr + off, X->values.data, n * 4, cudaMemcpyHostToDevice, cs),
                   module);
    }
    if (s->trace) {
        const double t1 = now_s();
        s->t_admit_host += t1 - t0;
        t0 = t1;
    }
    SPTGB_CUDA(cudaMemcpyAsync(s->d_gjobs.ptr, s->h_gjobs, (size_t)G * sizeof(sptgb_adm_job), cudaMemcpyHostToDevice,
                               cs),
               module);
    SPTGB_CUDA(cudaMemcpyAsync(s->d_goffs.ptr, s->h_goffs, (size_t)(G + 1) * 8, cudaMemcpyHostToDevice, cs), module);
    SPTGB_CUDA(cudaMemsetAsync(s->d_gerr.ptr, 0, (size_t)G * 4, cs), module);

    sptgb_adm_group g;
    memset(&g, 0, sizeof g);
    for (int m = 0; m < maxN; ++m) g.ind[m] = (const uint32_t *)s->st_ind[m].ptr;
    g.val = (const float *)s->st_val.ptr;
    g.offs = (const uint64_t *)s->d_goffs.ptr;
    g.jobs = (const sptgb_adm_job *)s->d_gjobs.ptr;
    g.njobs = G;
    g.total = total;
    g.err = (unsigned int *)s->d_gerr.ptr;
    SPTGB_CUDA(sptgb_adm_check(&g, cs), module);

    /* ||X||^2, lambda = 1, status = 0; initial factors and their Grams */
    for (int l = NL_STEP; l < NL_ADM_END; ++l) list_clear(s, l);
    for (uint32_t q = 0; q < G; ++q) {
        const sptgb_adm_job *a = &s->h_gjobs[q];
        list_add(s, NL_SQ, q, sptgb_sumsq_blocks(a->n));
        list_add(s, NL_SQONE, q, 1);
        for (uint32_t m = 0; m < a->nmodes; ++m) {
            list_add(s, NL_GDN + (int)m, a->slot, sptgb_gram_blocks(a->ndims[m]));
            list_add(s, NL_GONE + (int)m, a->slot, 1);
        }
    }
    SPTGB_CHECK(lists_upload(s, NL_STEP, NL_ADM_END, cs), module);
    const sptgb_wlist sq = wl(s, NL_SQ), sqone = wl(s, NL_SQONE);
    SPTGB_CUDA(sptgb_adm_normsq(s->ds, &g, &sq, &sqone, cs), module);
    for (uint32_t q = 0; q < G; ++q) {
        const job_t *j = &s->jobs[s->grp[q]];
        const sptgb_slot *d = &s->hs[j->slot];
        for (uint32_t m = 0; m < d->nmodes; ++m) {
            const size_t bytes = (size_t)d->ndims[m] * d->stride * 4;
            if (bytes)
                SPTGB_CUDA(cudaMemcpyAsync(d->fac[m], j->init[m]->values, bytes, cudaMemcpyHostToDevice, cs), module);
        }
    }
    for (int m = 0; m < maxN; ++m) {
        const sptgb_wlist dn = wl(s, NL_GDN + m), one = wl(s, NL_GONE + m);
        SPTGB_CUDA(sptgb_batch_gram(s->ds, &dn, &one, m, cs), module);
    }
    if (s->trace) {
        SPTGB_CUDA(cudaStreamSynchronize(cs), module);
        const double t1 = now_s();
        s->t_admit_h2d += t1 - t0;
        t0 = t1;
    }

    /* records, one sort of the whole group per mode */
    for (int m = 0; m < maxN && total; ++m) {
        uint32_t *perm = NULL;
        SPTGB_CHECK(sort_group_mode(s, &g, m, jbits, rowbits[m], &perm), module);
        SPTGB_CUDA(sptgb_adm_pack(&g, s->ds, m, perm, cs), module);
    }

    SPTGB_CUDA(cudaMemcpyAsync(s->h_gerr, s->d_gerr.ptr, (size_t)G * 4, cudaMemcpyDeviceToHost, cs), module);
    SPTGB_CUDA(cudaStreamSynchronize(cs), module);
    if (s->trace) {
        s->t_admit_dev += now_s() - t0;
        ++s->n_groups;
    }
    for (uint32_t q = 0; q < G; ++q) {
        job_t *j = &s->jobs[s->grp[q]];
        if (s->h_gerr[q]) {
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                              "a coordinate is not smaller than its mode size");
            fail_job(s, j);
        } else {
            j->state = JOB_ACTIVE;
        }
    }
    return 0;
}

/* ----------------------------------------------------- retirement -- */
/* GetFinalLambda (matrix.c:557-573) for every slot in s->ret[0..R), results
 * into the jobs' buffers, slots freed. */
static int retire(sptgbServer *s, uint32_t R) {
    const char *module = "GPU server retire";
    if (R == 0) return 0;
    const double t0 = s->trace ? now_s() : 0.0;
    for (int l = NL_RDN; l < NLISTS; ++l) list_clear(s, l);
    int maxN = 0;
    for (uint32_t r = 0; r < R; ++r) {
        const sptgb_slot *d = &s->hs[s->ret[r]];
        for (uint32_t m = 0; m < d->nmodes; ++m) {
            list_add(s, NL_RDN + (int)m, s->ret[r], sptgb_colnorm_blocks(d->ndims[m]));
            list_add(s, NL_RONE + (int)m, s->ret[r], 1);
        }
        if ((int)d->nmodes > maxN) maxN = (int)d->nmodes;
    }
    SPTGB_CHECK(lists_upload(s, NL_RDN, NLISTS, s->cs), module);
    for (int m = 0; m < maxN; ++m) {
        const sptgb_wlist dn = wl(s, NL_RDN + m), one = wl(s, NL_RONE + m);
        SPTGB_CUDA(sptgb_batch_final_lambda(s->ds, &dn, &one, m, s->cs), module);
    }
    for (uint32_t r = 0; r < R; ++r) {
        const sptgb_slot *d = &s->hs[s->ret[r]];
        job_t *j = &s->jobs[s->slot_job[s->ret[r]]];
        for (uint32_t m = 0; m < d->nmodes; ++m) {
            const size_t bytes = (size_t)d->ndims[m] * d->stride * 4;
            if (bytes)
                SPTGB_CUDA(cudaMemcpyAsync(j->out[m]->values, d->fac[m], bytes, cudaMemcpyDeviceToHost, s->cs), module);
        }
        SPTGB_CUDA(cudaMemcpyAsync(j->lambda, d->lambda, d->rank * 4, cudaMemcpyDeviceToHost, s->cs), module);
        if (j->niters)
            SPTGB_CUDA(cudaMemcpyAsync(j->fits, d->fits, (size_t)j->niters * 8, cudaMemcpyDeviceToHost, s->cs), module);
    }
    SPTGB_CUDA(cudaStreamSynchronize(s->cs), module);
    if (s->persistent) {
        sptgb_grid_bar hb;   /* a grid barrier of the persistent step whose bounded wait ran out */
        SPTGB_CUDA(cudaMemcpy(&hb, s->bar, sizeof hb, cudaMemcpyDeviceToHost), module);
        if (hb.err) SPTGB_CUDA(cudaErrorLaunchTimeout, module);
    }
    const double t = now_s();
    for (uint32_t r = 0; r < R; ++r) {
        job_t *j = &s->jobs[s->slot_job[s->ret[r]]];
        j->t_done = t;
        j->state = JOB_DONE;
        j->slot = -1;
        push_completed(s, j->ticket);
        release(s, s->ret[r]);
    }
    if (s->trace) {
        s->t_retire += now_s() - t0;
        ++s->n_retire_calls;
    }
    return 0;
}

/* ------------------------------------------------------ autotuning -- */
/* Schedules tuned in this process: [rank group][order 3 / 4][log2 of the
 * mean nonzeros per job]. */
#define TUNE_BUCKETS 40
typedef struct {
    uint32_t ul, sched;
    int valid;
} tune_entry;
static tune_entry g_tune[4][2][TUNE_BUCKETS];
static pthread_mutex_t g_tune_lock = PTHREAD_MUTEX_INITIALIZER;

/* Tunes every rank group that has admitted jobs and no schedule yet (a
 * group is tuned once, before the first iteration of its first jobs);
 * *ntuned = groups given a schedule by this call. */
static int autotune(sptgbServer *s, int *ntuned) {
    static const uint32_t cand_ul[4] = {64, 128, 256, 512};
    const char *module = "GPU server tune";
    *ntuned = 0;
    uint64_t nnz3[4] = {0, 0, 0, 0}, nnz4[4] = {0, 0, 0, 0}, jobs[4] = {0, 0, 0, 0};
    for (uint32_t i = 0; i < s->cap; ++i)
        if (s->slot_job[i] >= 0 && s->hs[i].nnz) {
            const int g = group_of(s->hs[i].stride);
            ++jobs[g];
            if (s->hs[i].nmodes == 3) nnz3[g] += s->hs[i].nnz;
            else nnz4[g] += s->hs[i].nnz;
        }
    int todo = 0;
    for (int g = 0; g < 4; ++g) todo |= jobs[g] && s->tuned_from_cache[g] < 0;
    if (!todo) return 0;
    cudaEvent_t e0, e1;
    SPTGB_CUDA(cudaEventCreate(&e0), module);
    SPTGB_CUDA(cudaEventCreate(&e1), module);
    for (int g = 0; g < 4; ++g) {
        if (!jobs[g] || s->tuned_from_cache[g] >= 0) continue;
        ++*ntuned;
        const int ord = nnz4[g] > nnz3[g];
        int bucket = 0;
        for (uint64_t mean = (nnz3[g] + nnz4[g]) / jobs[g]; mean > 1 && bucket < TUNE_BUCKETS - 1; mean >>= 1)
            ++bucket;
        pthread_mutex_lock(&g_tune_lock);
        const tune_entry hit = g_tune[g][ord][bucket];
        pthread_mutex_unlock(&g_tune_lock);
        if (hit.valid) {
            s->ul[g] = hit.ul;
            s->sched[g] = hit.sched;
            s->tuned_from_cache[g] = 1;
            continue;
        }
        float best = 1e30f;
        uint32_t best_ul = s->ul[g], best_sched = s->sched[g];
        for (int c = 0; c < 4; ++c) {
            s->ul[g] = cand_ul[c];
            step_lists_build(s);
            SPTGB_CHECK(lists_upload(s, 0, NL_STEP, s->cs), module);
            const sptgb_wlist w = wl(s, NL_MT + g);
            for (uint32_t sc = 0; sc < 4; ++sc) {
                float ms = 0.f, tot = 0.f;
                for (int rep = 0; rep < 3; ++rep) {
                    SPTGB_CUDA(cudaEventRecord(e0, s->cs), module);
                    SPTGB_CUDA(sptgb_batch_mttkrp(s->ds, &w, 0, g, cand_ul[c], sc, s->cs), module);
                    SPTGB_CUDA(cudaEventRecord(e1, s->cs), module);
                    SPTGB_CUDA(cudaEventSynchronize(e1), module);
                    SPTGB_CUDA(cudaEventElapsedTime(&ms, e0, e1), module);
                    if (rep) tot += ms;
                }
                if (tot < best) {
                    best = tot;
                    best_ul = cand_ul[c];
                    best_sched = sc;
                }
            }
        }
        s->ul[g] = best_ul;
        s->sched[g] = best_sched;
        s->tuned_from_cache[g] = 0;
        pthread_mutex_lock(&g_tune_lock);
        g_tune[g][ord][bucket] = (tune_entry){best_ul, best_sched, 1};
        pthread_mutex_unlock(&g_tune_lock);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s->trace)
        for (int g = 0; g < 4; ++g)
            if (jobs[g] && s->tuned_from_cache[g] >= 0)
                fprintf(stderr, "[sptgb server] rank <= %d: MTTKRP unit %u, %s record batches, %d blocks/SM (%s)\n",
                        8 << g, s->ul[g], (s->sched[g] & 1u) ? "deep" : "shallow", (s->sched[g] & 2u) ? 3 : 2,
                        s->tuned_from_cache[g] ? "cached" : "timed");
    return 0;
}

static int capture(sptgbServer *s) {
    const char *module = "GPU server capture";
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
    for (int g = 0; g < 4; ++g) {
        s->L.ul[g] = s->ul[g];
        s->L.sched[g] = s->sched[g];
    }
    s->L.fit = wl(s, NL_FIT);
    s->L.fit_one = wl(s, NL_FITONE);
    /* One ALS iteration of every admitted job: by default the sequence of
     * kernels (one per phase and lane group); SPTGB_STEP=persistent captures
     * one persistent cooperative kernel (sptgb_batch_step_persistent) as the
     * graph's only node instead, and falls back to the sequence on a device
     * without cooperative launch or a capture that refuses the node.  The
     * sequence is the default because it is faster on GB300: its MTTKRP
     * kernels run with the whole L1 (the fused kernel carries the solve's
     * shared memory in every phase) and admission kernels overlap it. */
    const char *mode = getenv("SPTGB_STEP");
    int persistent = mode && mode[0] == 'p';
    for (int attempt = 0; attempt < 2; ++attempt) {
        cudaGraph_t graph = NULL;
        SPTGB_CUDA(cudaStreamBeginCapture(s->cs, cudaStreamCaptureModeThreadLocal), module);
        const uint64_t c0 = sptgbLaunchCount();
        const cudaError_t e = persistent ? sptgb_batch_step_persistent(s->ds, &s->L, s->bar, s->cs)
                                         : sptgb_batch_step(s->ds, &s->L, s->cs);
        const uint64_t nk = sptgbLaunchCount() - c0;
        sptgb_uncount_launch(nk);
        const cudaError_t e2 = cudaStreamEndCapture(s->cs, &graph);
        cudaError_t e3 = cudaErrorUnknown;
        if (e == cudaSuccess && e2 == cudaSuccess) e3 = cudaGraphInstantiate(&s->gexec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess) {
            s->have_graph = 1;
            s->persistent = persistent;
            s->graph_kernels = (uint32_t)nk;
            return 0;
        }
        cudaGetLastError();
        if (!persistent) {
            SPTGB_CUDA(e != cudaSuccess ? e : (e2 != cudaSuccess ? e2 : e3), module);
        }
        persistent = 0;   /* retry with the kernel sequence */
    }
    return SPTERR_CUDA_ERROR;
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
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->bar, sizeof(sptgb_grid_bar));
    if (e == cudaSuccess) e = cudaMemset(s->bar, 0, sizeof(sptgb_grid_bar));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_counts, NLISTS * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_ids, (size_t)NLISTS * s->cap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->d_pre, (size_t)NLISTS * (s->cap + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->as, cudaStreamNonBlocking);
    if (e != cudaSuccess) r = sptgb_cuda_fail(e, "GPU server create", __FILE__, __LINE__);
    const uint32_t gcap = s->cap < SERVE_GROUP_JOBS ? s->cap : SERVE_GROUP_JOBS;
    s->hs = (sptgb_slot *)calloc(s->cap, sizeof(sptgb_slot));
    s->slot_job = (int64_t *)malloc(s->cap * sizeof(int64_t));
    s->slot_off = (uint64_t *)calloc(s->cap, sizeof(uint64_t));
    s->slot_len = (uint64_t *)calloc(s->cap, sizeof(uint64_t));
    s->slot_iters = (uint32_t *)calloc(s->cap, sizeof(uint32_t));
    s->h_counts = (uint32_t *)calloc(NLISTS, sizeof(uint32_t));
    s->h_ids = (uint32_t *)calloc((size_t)NLISTS * s->cap, sizeof(uint32_t));
    s->h_pre = (uint64_t *)calloc((size_t)NLISTS * (s->cap + 1), sizeof(uint64_t));
    s->grp = (uint32_t *)calloc(gcap, sizeof(uint32_t));
    s->h_gjobs = (sptgb_adm_job *)calloc(gcap, sizeof(sptgb_adm_job));
    s->h_goffs = (uint64_t *)calloc(gcap + 1, sizeof(uint64_t));
    s->h_gerr = (unsigned int *)calloc(gcap, sizeof(unsigned int));
    s->ret = (uint32_t *)calloc(s->cap, sizeof(uint32_t));
    s->freecap = 64;
    s->freel = (span_t *)malloc(s->freecap * sizeof(span_t));
    if (!r && (!s->hs || !s->slot_job || !s->slot_off || !s->slot_len || !s->slot_iters || !s->h_counts || !s->h_ids ||
               !s->h_pre || !s->grp || !s->h_gjobs || !s->h_goffs || !s->h_gerr || !s->ret || !s->freel))
        r = SPTERR_OS_ERROR;
    if (r) {
        sptgbServerFree(s);
        return r;
    }
    for (uint32_t i = 0; i < s->cap; ++i) s->slot_job[i] = -1;
    s->freel[0].off = 0;
    s->freel[0].len = s->budget;
    s->nfree = 1;
    for (int g = 0; g < 4; ++g) {
        s->ul[g] = 256;
        s->sched[g] = 1;   /* deep batches, 2 blocks per SM until tuned */
        s->tuned_from_cache[g] = -1;
    }
    s->changed = 1;
    const char *tr = getenv("SPTGB_TRACE");
    s->trace = tr && tr[0] && tr[0] != '0';
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
    const uint32_t stride = stride_of(rank);
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
    double t0 = 0.0;
    /* 1. one ALS iteration of every job admitted by an earlier call, launched
     *    first: this call's admission (its own stream, new slots only) runs on
     *    the host and the copy engines while the graph runs */
    uint32_t R = 0;
    if (s->nactive > 0) {
        int ntuned = 0;
        SPTGB_CHECK(autotune(s, &ntuned), module);
        if (ntuned) {
            s->changed = 1;
            if (s->have_graph) {   /* the schedules are launch parameters of the captured step */
                cudaGraphExecDestroy(s->gexec);
                s->have_graph = 0;
            }
        }
        if (s->changed) {
            step_lists_build(s);
            SPTGB_CHECK(lists_upload(s, 0, NL_STEP, s->cs), module);
            s->changed = 0;
        }
        if (!s->have_graph) SPTGB_CHECK(capture(s), module);
        if (s->trace) t0 = now_s();
        SPTGB_CUDA(cudaGraphLaunch(s->gexec, s->cs), module);
        sptgb_count_launch(s->graph_kernels);
        if (s->trace) {
            SPTGB_CUDA(cudaStreamSynchronize(s->cs), module);
            s->t_step += now_s() - t0;
            ++s->n_steps;
        }
        /* the slots in this step that reach their iteration count retire
         * after it (slots admitted below start at the next step) */
        for (uint32_t i = 0; i < s->cap; ++i) {
            if (s->slot_job[i] < 0) continue;
            if (++s->slot_iters[i] >= s->jobs[s->slot_job[i]].niters) s->ret[R++] = i;
        }
    }
    /* 2. admission group: queued jobs that fit, in submission order */
    if (s->trace) t0 = now_s();
    const uint32_t gcap = s->cap < SERVE_GROUP_JOBS ? s->cap : SERVE_GROUP_JOBS;
    uint32_t G = 0;
    uint64_t gnnz = 0, keep = 0;
    uint32_t next_free = 0;
    for (uint64_t qi = 0; qi < s->nqueue; ++qi) {
        const uint64_t ji = s->queue[qi];
        job_t *j = &s->jobs[ji];
        if (j->bytes > s->budget) {
            spt_ComplainError(module, SPTERR_NO_MORE, __FILE__, __LINE__, "job larger than the HBM budget");
            fail_job(s, j);
            continue;
        }
        while (next_free < s->cap && s->slot_job[next_free] >= 0) ++next_free;
        uint64_t off = 0;
        if (G == gcap || next_free == s->cap || (G > 0 && gnnz + j->X->nnz > SERVE_GROUP_NNZ) ||
            arena_alloc(s, j->bytes, &off) != 0) {
            s->queue[keep++] = ji;
            continue;
        }
        const uint32_t slot = next_free;
        s->slot_off[slot] = off;
        s->slot_len[slot] = j->bytes;
        s->slot_job[slot] = (int64_t)ji;
        s->slot_iters[slot] = 0;
        ++s->nactive;
        j->slot = (int)slot;
        s->grp[G++] = (uint32_t)ji;
        gnnz += j->X->nnz;
        s->changed = 1;
    }
    s->nqueue = keep;
    if (s->trace) s->t_select += now_s() - t0;
    if (G) {
        const int r = admit_group(s, G);
        if (r) {
            for (uint32_t q = 0; q < G; ++q)
                if (s->jobs[s->grp[q]].state == JOB_QUEUED) fail_job(s, &s->jobs[s->grp[q]]);
            cudaStreamSynchronize(s->cs);   /* nothing of this call outlives it on error */
            return r;
        }
        /* jobs with no iterations finish at once */
        for (uint32_t q = 0; q < G; ++q) {
            const job_t *j = &s->jobs[s->grp[q]];
            if (j->state == JOB_ACTIVE && j->niters == 0) s->ret[R++] = (uint32_t)j->slot;
        }
    }
    /* 3. retirement (after the step: retire() runs on the step's stream) */
    SPTGB_CHECK(retire(s, R), module);
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

uint32_t sptgbServerCompleted(sptgbServer *s, uint64_t *tickets, uint32_t max) {
    uint32_t n = 0;
    while (n < max && s->finread < s->nfin) tickets[n++] = s->fin[s->finread++];
    if (s->finread == s->nfin) s->finread = s->nfin = 0;
    return n;
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
int sptgbServerPersistent(const sptgbServer *s) { return s->persistent; }
uint32_t sptgbServerStepKernels(const sptgbServer *s) { return s->have_graph ? s->graph_kernels : 0; }

int sptgbServerSchedule(const sptgbServer *s, int group, uint32_t *unit_len, uint32_t *deep, uint32_t *blocks_per_sm,
                        int *from_cache) {
    if (group < 0 || group > 3) return SPTERR_VALUE_ERROR;
    *unit_len = s->ul[group];
    *deep = s->sched[group] & 1u;
    *blocks_per_sm = (s->sched[group] & 2u) ? 3u : 2u;
    *from_cache = s->tuned_from_cache[group];
    return 0;
}

int sptgbGridBarrierSelfTest(int missing, int *err, unsigned int *rounds) {
    const char *module = "GPU barrier self-test";
    SPTGB_CHECK(sptgb_ctx(), module);
    SPTGB_CUDA(sptgb_grid_barrier_selftest(missing, err, rounds), module);
    return 0;
}

void sptgbServerFree(sptgbServer *s) {
    if (!s) return;
    if (s->trace)
        fprintf(stderr,
                "[sptgb server] select %.3f s | admit: host %.3f s, h2d+normsq+grams %.3f s, sort+pack %.3f s "
                "(%llu groups) | steps %.3f s (%llu) | retire %.3f s (%llu)\n",
                s->t_select, s->t_admit_host, s->t_admit_h2d, s->t_admit_dev, (unsigned long long)s->n_groups,
                s->t_step, (unsigned long long)s->n_steps, s->t_retire, (unsigned long long)s->n_retire_calls);
    if (s->cs) cudaStreamSynchronize(s->cs);
    if (s->have_graph) cudaGraphExecDestroy(s->gexec);
    if (s->arena) cudaFree(s->arena);
    if (s->ds) cudaFree(s->ds);
    if (s->bar) cudaFree(s->bar);
    if (s->d_counts) cudaFree(s->d_counts);
    if (s->d_ids) cudaFree(s->d_ids);
    if (s->d_pre) cudaFree(s->d_pre);
    for (int m = 0; m < 4; ++m) sptgb_dbuf_release(&s->st_ind[m]);
    sptgb_dbuf_release(&s->st_val);
    for (int b = 0; b < 2; ++b) {
        sptgb_dbuf_release(&s->keys[b]);
        sptgb_dbuf_release(&s->perm[b]);
    }
    sptgb_dbuf_release(&s->rtmp);
    sptgb_dbuf_release(&s->d_gjobs);
    sptgb_dbuf_release(&s->d_goffs);
    sptgb_dbuf_release(&s->d_gerr);
    if (s->cs) cudaStreamDestroy(s->cs);
    if (s->as) cudaStreamDestroy(s->as);
    free(s->hs);
    free(s->slot_job);
    free(s->slot_off);
    free(s->slot_len);
    free(s->slot_iters);
    free(s->h_counts);
    free(s->h_ids);
    free(s->h_pre);
    free(s->grp);
    free(s->h_gjobs);
    free(s->h_goffs);
    free(s->h_gerr);
    free(s->ret);
    free(s->freel);
    free(s->jobs);
    free(s->queue);
    free(s->fin);
    free(s);
}
