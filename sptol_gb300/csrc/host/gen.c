/*
 * Seeded synthetic sparse tensors and factor matrices.
 *
 * Random numbers: SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) used as a
 * counter-based generator, value i of stream (seed, id) = mix(base + (i+1)*
 * golden gamma), so every draw is computable independently and the output
 * does not depend on the thread count.
 *   uniform index in [0, n): multiply-shift of the high 32 bits;
 *   U[0,1): top 24 bits (exact in float);
 *   normal: Box-Muller from two 53-bit uniforms;
 *   truncated Zipf(s) on ranks 1..n (index = rank-1): inverse CDF over the
 *   exact normalised table of k^-s, searched through a 2^16-bucket guide.
 * Tensor construction:
 *   merge_duplicates = 1: `count` draws, coordinates sorted lexicographically,
 *     duplicate coordinates merged by summing their values in draw order;
 *   merge_duplicates = 0: draws are deduplicated and topped up with further
 *     draws (each round draws exactly the number still missing, so no round
 *     overshoots) until exactly `count` unique coordinates exist; values are
 *     then drawn per unique coordinate in sorted position order.
 * Coordinates are packed into one key (mode 0 most significant): 64 bits
 * when the bit widths of all modes sum to at most 64, else 128 bits, sorted
 * by the low 64 bits and then stably by the high bits.
 */
#define _GNU_SOURCE
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include "../sptgb_internal.h"
#include "../../../include/sptgb.h"

#define GAMMA 0x9E3779B97F4A7C15ULL

static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline uint64_t stream_base(uint64_t seed, uint64_t id) { return mix64(seed ^ mix64(id * GAMMA + 0x632BE59BD9B4E019ULL)); }
static inline uint64_t rng_at(uint64_t base, uint64_t i) { return mix64(base + GAMMA * (i + 1)); }
static inline uint32_t uniform_index(uint64_t r, uint32_t n) { return (uint32_t)(((r >> 32) * (uint64_t)n) >> 32); }
static inline float u01f(uint64_t r) { return (float)((r >> 40) * (1.0 / 16777216.0)); }
static inline double u01d(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }
static inline double normal_at(uint64_t base, uint64_t i) {
    const double u1 = ((double)(rng_at(base, 2 * i) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
    const double u2 = u01d(rng_at(base, 2 * i + 1));
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

typedef struct {
    double *cdf;     /* cdf[k] = P(index <= k), k in [0, n) */
    uint32_t *guide; /* guide[j] = first k with cdf[k] > j / G */
    uint32_t n;
} zipf_table;
#define ZG 65536

static int zipf_build(zipf_table *z, uint32_t n, double s) {
    z->n = n;
    z->cdf = (double *)malloc((size_t)n * sizeof(double));
    z->guide = (uint32_t *)malloc((ZG + 1) * sizeof(uint32_t));
    if (!z->cdf || !z->guide) return SPTERR_OS_ERROR;
    double acc = 0.0;
    for (uint32_t k = 0; k < n; ++k) {
        acc += pow((double)k + 1.0, -s);
        z->cdf[k] = acc;
    }
    for (uint32_t k = 0; k < n; ++k) z->cdf[k] /= acc;
    z->cdf[n - 1] = 1.0;
    uint32_t k = 0;
    for (uint32_t j = 0; j <= ZG; ++j) {
        const double t = (double)j / ZG;
        while (k < n - 1 && z->cdf[k] <= t) ++k;
        z->guide[j] = k;
    }
    return 0;
}

static inline uint32_t zipf_sample(const zipf_table *z, double u) {
    const uint32_t j = (uint32_t)(u * ZG);
    uint32_t lo = z->guide[j], hi = z->guide[j + 1 <= ZG ? j + 1 : ZG];
    if (hi < lo) hi = lo;
    /* first k in [lo, hi] with cdf[k] > u */
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (z->cdf[mid] > u) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

static void zipf_free(zipf_table *z) {
    free(z->cdf);
    free(z->guide);
}

/* Parallel stable LSD radix sort of u64 keys (optionally carrying u32
 * payloads) over the low `bits` bits, 11-bit digits. */
static int radix_sort_u64(uint64_t *keys, uint32_t *pay, uint64_t n, int bits) {
    if (n < 2 || bits <= 0) return 0;
    uint64_t *k2 = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint32_t *p2 = pay ? (uint32_t *)malloc(n * sizeof(uint32_t)) : NULL;
    if (!k2 || (pay && !p2)) {
        free(k2);
        free(p2);
        return SPTERR_OS_ERROR;
    }
    const int D = 11, B = 1 << D;
    const int T = omp_get_max_threads();
    uint64_t *hist = (uint64_t *)malloc((size_t)T * B * sizeof(uint64_t));
    uint64_t *ka = keys, *kb = k2;
    uint32_t *pa = pay, *pb = p2;
    for (int shift = 0; shift < bits; shift += D) {
        memset(hist, 0, (size_t)T * B * sizeof(uint64_t));
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num();
            const uint64_t lo = n * t / T, hi = n * (t + 1) / T;
            uint64_t *h = hist + (size_t)t * B;
            for (uint64_t i = lo; i < hi; ++i) h[(ka[i] >> shift) & (B - 1)]++;
        }
        uint64_t run = 0;
        for (int d = 0; d < B; ++d)
            for (int t = 0; t < T; ++t) {
                const uint64_t c = hist[(size_t)t * B + d];
                hist[(size_t)t * B + d] = run;
                run += c;
            }
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num();
            const uint64_t lo = n * t / T, hi = n * (t + 1) / T;
            uint64_t *h = hist + (size_t)t * B;
            for (uint64_t i = lo; i < hi; ++i) {
                const uint64_t pos = h[(ka[i] >> shift) & (B - 1)]++;
                kb[pos] = ka[i];
                if (pa) pb[pos] = pa[i];
            }
        }
        uint64_t *tk = ka;
        ka = kb;
        kb = tk;
        uint32_t *tp = pa;
        pa = pb;
        pb = tp;
    }
    if (ka != keys) {
        memcpy(keys, ka, n * sizeof(uint64_t));
        if (pay) memcpy(pay, pa, n * sizeof(uint32_t));
    }
    free(hist);
    free(k2);
    free(p2);
    return 0;
}

typedef struct {
    const sptgbGenSpec *spec;
    int bits[SPTGB_MAX_MODES];
    int shift[SPTGB_MAX_MODES];
    int total_bits;
    uint64_t base[SPTGB_MAX_MODES];
    zipf_table z[SPTGB_MAX_MODES];
} gen_ctx;

static void draw_keys(const gen_ctx *g, uint64_t first, uint64_t count, uint64_t *keys) {
    const sptgbGenSpec *sp = g->spec;
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < count; ++i) {
        uint64_t key = 0;
        for (sptIndex m = 0; m < sp->nmodes; ++m) {
            const uint64_t r = rng_at(g->base[m], first + i);
            uint32_t c;
            if (sp->coord_dist[m] == SPTGB_DIST_ZIPF) c = zipf_sample(&g->z[m], u01d(r));
            else c = uniform_index(r, sp->ndims[m]);
            key |= (uint64_t)c << g->shift[m];
        }
        keys[i] = key;
    }
}

/* Removes adjacent duplicates of a sorted array; returns the new length. */
static uint64_t unique_sorted(uint64_t *a, uint64_t n) {
    if (n == 0) return 0;
    uint64_t w = 1;
    for (uint64_t i = 1; i < n; ++i)
        if (a[i] != a[w - 1]) a[w++] = a[i];
    return w;
}

typedef unsigned __int128 u128;

static void draw_keys128(const gen_ctx *g, uint64_t first, uint64_t count, u128 *keys) {
    const sptgbGenSpec *sp = g->spec;
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < count; ++i) {
        u128 key = 0;
        for (sptIndex m = 0; m < sp->nmodes; ++m) {
            const uint64_t r = rng_at(g->base[m], first + i);
            uint32_t c;
            if (sp->coord_dist[m] == SPTGB_DIST_ZIPF) c = zipf_sample(&g->z[m], u01d(r));
            else c = uniform_index(r, sp->ndims[m]);
            key |= (u128)c << g->shift[m];
        }
        keys[i] = key;
    }
}

/* Stable sort of 128-bit keys (and u32 payloads): the 64-bit sort on the low
 * halves, then on the high halves, carrying a permutation. */
static int radix_sort_u128(u128 *keys, uint32_t *pay, uint64_t n, int bits) {
    if (n < 2 || bits <= 0) return 0;
    uint64_t *half = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint32_t *perm = (uint32_t *)malloc(n * sizeof(uint32_t));
    u128 *tk = (u128 *)malloc(n * sizeof(u128));
    uint32_t *tp = pay ? (uint32_t *)malloc(n * sizeof(uint32_t)) : NULL;
    int r = (!half || !perm || !tk || (pay && !tp)) ? SPTERR_OS_ERROR : 0;
    if (!r) {
#pragma omp parallel for schedule(static)
        for (uint64_t i = 0; i < n; ++i) {
            half[i] = (uint64_t)keys[i];
            perm[i] = (uint32_t)i;
        }
        r = radix_sort_u64(half, perm, n, bits < 64 ? bits : 64);
    }
    if (!r && bits > 64) {
#pragma omp parallel for schedule(static)
        for (uint64_t i = 0; i < n; ++i) half[i] = (uint64_t)(keys[perm[i]] >> 64);
        r = radix_sort_u64(half, perm, n, bits - 64);
    }
    if (!r) {
#pragma omp parallel for schedule(static)
        for (uint64_t i = 0; i < n; ++i) {
            tk[i] = keys[perm[i]];
            if (pay) tp[i] = pay[perm[i]];
        }
        memcpy(keys, tk, n * sizeof(u128));
        if (pay) memcpy(pay, tp, n * sizeof(uint32_t));
    }
    free(half);
    free(perm);
    free(tk);
    free(tp);
    return r;
}

/* Unique coordinates (merge_duplicates = 0) with keys wider than 64 bits:
 * the same draw-sort-dedupe-top-up rounds as the 64-bit path. */
static int unique_keys128(const gen_ctx *g, uint64_t target, int tb, u128 **out) {
    u128 *keys = (u128 *)malloc((target ? target : 1) * sizeof(u128));
    u128 *fresh = (u128 *)malloc((target ? target : 1) * sizeof(u128));
    u128 *merged = (u128 *)malloc((target ? target : 1) * sizeof(u128));
    if (!keys || !fresh || !merged) {
        free(keys);
        free(fresh);
        free(merged);
        return SPTERR_OS_ERROR;
    }
    uint64_t have = 0, drawn = 0;
    int r = 0;
    while (have < target) {
        const uint64_t need = target - have;
        draw_keys128(g, drawn, need, fresh);
        drawn += need;
        r = radix_sort_u128(fresh, NULL, need, tb);
        if (r) break;
        uint64_t nf = need ? 1 : 0;
        for (uint64_t i = 1; i < need; ++i)
            if (fresh[i] != fresh[nf - 1]) fresh[nf++] = fresh[i];
        uint64_t i = 0, j = 0, w = 0;
        while (i < have || j < nf) {
            if (j >= nf || (i < have && keys[i] < fresh[j])) merged[w++] = keys[i++];
            else if (i >= have || fresh[j] < keys[i]) merged[w++] = fresh[j++];
            else {
                merged[w++] = keys[i++];
                ++j;
            }
        }
        u128 *t = keys;
        keys = merged;
        merged = t;
        have = w;
    }
    free(fresh);
    free(merged);
    if (r) {
        free(keys);
        return r;
    }
    *out = keys;
    return 0;
}

int sptgbGenerate(sptSparseTensor *X, const sptgbGenSpec *sp) {
    const char *module = "SpTns generate";
    if (sp->nmodes < 1 || sp->nmodes > SPTGB_MAX_MODES) return SPTERR_VALUE_ERROR;
    gen_ctx g;
    memset(&g, 0, sizeof g);
    g.spec = sp;
    int tb = 0;
    for (int m = (int)sp->nmodes - 1; m >= 0; --m) {
        if (sp->ndims[m] == 0) return SPTERR_VALUE_ERROR;
        uint32_t x = sp->ndims[m] - 1;
        int b = 0;
        while (x) {
            ++b;
            x >>= 1;
        }
        g.bits[m] = b;
        g.shift[m] = tb;
        tb += b;
    }
    g.total_bits = tb;
    if (tb > 128 || (tb > 64 && sp->merge_duplicates)) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                          tb > 128 ? "mode bit widths exceed 128" : "merged duplicates need at most 64 key bits");
        return SPTERR_VALUE_ERROR;
    }
    uint64_t space = 1;
    for (sptIndex m = 0; m < sp->nmodes; ++m) {
        g.base[m] = stream_base(sp->seed, 1 + m);
        if (sp->coord_dist[m] == SPTGB_DIST_ZIPF && zipf_build(&g.z[m], sp->ndims[m], sp->zipf_s[m]))
            return SPTERR_OS_ERROR;
        space = (space > UINT64_MAX / sp->ndims[m]) ? UINT64_MAX : space * sp->ndims[m];
    }
    if (!sp->merge_duplicates && sp->count > space) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "more unique nonzeros than coordinates");
        return SPTERR_VALUE_ERROR;
    }
    uint64_t *keys = NULL;
    u128 *wkeys = NULL;
    float *vals = NULL;
    uint64_t nnz = 0;
    int r = 0;
    if (tb > 64) {
        r = unique_keys128(&g, sp->count, tb, &wkeys);
        nnz = sp->count;
        if (!r) {
            vals = (float *)malloc((nnz ? nnz : 1) * sizeof(float));
            if (!vals) r = SPTERR_OS_ERROR;
        }
    } else if (sp->merge_duplicates) {
        const uint64_t n = sp->count;
        keys = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
        uint32_t *order = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
        vals = (float *)malloc((n ? n : 1) * sizeof(float));
        if (!keys || !order || !vals) return SPTERR_OS_ERROR;
        draw_keys(&g, 0, n, keys);
        for (uint64_t i = 0; i < n; ++i) order[i] = (uint32_t)i;
        r = radix_sort_u64(keys, order, n, tb);
        const uint64_t vbase = stream_base(sp->seed, 100);
        uint64_t w = 0;
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t rv = rng_at(vbase, order[i]);
            float v = sp->value_dist == SPTGB_VAL_UPM1 ? 2.0f * u01f(rv) - 1.0f : u01f(rv);
            if (w > 0 && keys[w - 1] == keys[i]) {
                vals[w - 1] += v;
            } else {
                keys[w] = keys[i];
                vals[w] = v;
                ++w;
            }
        }
        nnz = w;
        free(order);
    } else {
        const uint64_t target = sp->count;
        uint64_t have = 0, drawn = 0;
        keys = (uint64_t *)malloc((target ? target : 1) * sizeof(uint64_t));
        uint64_t *fresh = (uint64_t *)malloc((target ? target : 1) * sizeof(uint64_t));
        uint64_t *merged = (uint64_t *)malloc((target ? target : 1) * sizeof(uint64_t));
        if (!keys || !fresh || !merged) return SPTERR_OS_ERROR;
        while (have < target) {
            const uint64_t need = target - have;
            draw_keys(&g, drawn, need, fresh);
            drawn += need;
            r = radix_sort_u64(fresh, NULL, need, tb);
            if (r) break;
            uint64_t nf = unique_sorted(fresh, need);
            /* fresh \ keys, merged with keys */
            uint64_t i = 0, j = 0, w = 0;
            while (i < have || j < nf) {
                if (j >= nf || (i < have && keys[i] < fresh[j])) merged[w++] = keys[i++];
                else if (i >= have || fresh[j] < keys[i]) merged[w++] = fresh[j++];
                else {
                    merged[w++] = keys[i++];
                    ++j;
                }
            }
            uint64_t *t = keys;
            keys = merged;
            merged = t;
            have = w;
        }
        free(fresh);
        free(merged);
        nnz = have;
        vals = (float *)malloc((nnz ? nnz : 1) * sizeof(float));
        if (!vals) return SPTERR_OS_ERROR;
    }
    for (sptIndex m = 0; m < sp->nmodes; ++m) zipf_free(&g.z[m]);
    if (r) {
        free(keys);
        free(wkeys);
        free(vals);
        return r;
    }

    r = sptNewSparseTensor(X, sp->nmodes, sp->ndims);
    if (r) return r;
    for (sptIndex m = 0; m < sp->nmodes; ++m)
        if ((r = sptResizeIndexVector(&X->inds[m], nnz))) return r;
    if ((r = sptResizeValueVector(&X->values, nnz))) return r;
    X->nnz = nnz;
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < nnz; ++i)
        for (sptIndex m = 0; m < sp->nmodes; ++m)
            X->inds[m].data[i] = wkeys ? (uint32_t)((wkeys[i] >> g.shift[m]) & ((1ULL << g.bits[m]) - 1))
                                       : (uint32_t)((keys[i] >> g.shift[m]) & ((1ULL << g.bits[m]) - 1));

    if (sp->merge_duplicates) {
        memcpy(X->values.data, vals, nnz * sizeof(float));
    } else {
        const uint64_t vbase = stream_base(sp->seed, 100);
        if (sp->value_dist == SPTGB_VAL_PLANTED) {
            const sptIndex R = sp->planted_rank ? sp->planted_rank : 1;
            float *A[SPTGB_MAX_MODES];
            for (sptIndex m = 0; m < sp->nmodes; ++m) {
                A[m] = (float *)malloc((size_t)sp->ndims[m] * R * sizeof(float));
                const uint64_t fb = stream_base(sp->planted_seed, 200 + m);
#pragma omp parallel for schedule(static)
                for (uint64_t e = 0; e < (uint64_t)sp->ndims[m] * R; ++e) A[m][e] = u01f(rng_at(fb, e));
            }
            const uint64_t nb = stream_base(sp->seed, 300);
#pragma omp parallel for schedule(static)
            for (uint64_t i = 0; i < nnz; ++i) {
                double v = 0.0;
                for (sptIndex rr = 0; rr < R; ++rr) {
                    double p = 1.0;
                    for (sptIndex m = 0; m < sp->nmodes; ++m)
                        p *= A[m][(size_t)X->inds[m].data[i] * R + rr];
                    v += p;
                }
                v += sp->noise_sigma * normal_at(nb, i);
                X->values.data[i] = (float)v;
            }
            for (sptIndex m = 0; m < sp->nmodes; ++m) free(A[m]);
        } else {
#pragma omp parallel for schedule(static)
            for (uint64_t i = 0; i < nnz; ++i) {
                float v;
                if (sp->value_dist == SPTGB_VAL_LOGNORMAL) v = (float)exp(normal_at(vbase, i));
                else if (sp->value_dist == SPTGB_VAL_UPM1) v = 2.0f * u01f(rng_at(vbase, i)) - 1.0f;
                else v = u01f(rng_at(vbase, i));
                X->values.data[i] = v;
            }
        }
    }
    free(keys);
    free(wkeys);
    free(vals);
    return 0;
}

int sptgbFillMatrix(sptMatrix *mtx, uint64_t seed, uint64_t stream_id, float lo, float hi) {
    const uint64_t base = stream_base(seed, 1000 + stream_id);
    const sptIndex nr = mtx->nrows, nc = mtx->ncols, st = mtx->stride;
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < nr; ++i)
        for (sptIndex j = 0; j < st; ++j)
            mtx->values[i * st + j] = j < nc ? lo + (hi - lo) * u01f(rng_at(base, i * nc + j)) : 0.0f;
    return 0;
}
