/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of ParTI!'s sparse MTTKRP / CP-ALS path, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline arm as the checker.
 * The library (libParTI.so) never links, loads or calls this code.
 *
 * Every function restates one reference routine, cited by file:line of the
 * ParTI! sources.  Parity pinning: tests/golden/ holds outputs of the
 * reference itself (compiled from its own sources by oracle/Makefile, target
 * `ref`), and tests/test_oracle_golden.py checks these functions against them.
 *
 * Interfaces use flat arrays: inds[m] points at the nnz mode-m coordinates,
 * factor matrices are row-major with `stride` floats per row.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_MODES 8

/* ------------------------------------------------------------- sorting --
 * Merge sort of a permutation under a comparison; the reference's orders are
 * total on unique coordinates, so any correct sort yields its permutation. */
typedef int (*orc_cmp)(const void *ctx, uint64_t a, uint64_t b);

static void msort(uint64_t *p, uint64_t *tmp, uint64_t n, orc_cmp cmp, const void *ctx) {
    if (n < 2) return;
    const uint64_t h = n / 2;
    msort(p, tmp, h, cmp, ctx);
    msort(p + h, tmp, n - h, cmp, ctx);
    uint64_t i = 0, j = h, k = 0;
    while (i < h && j < n) tmp[k++] = cmp(ctx, p[j], p[i]) < 0 ? p[j++] : p[i++];
    while (i < h) tmp[k++] = p[i++];
    while (j < n) tmp[k++] = p[j++];
    memcpy(p, tmp, n * sizeof *p);
}

typedef struct {
    uint32_t nmodes;
    const uint32_t *const *inds;
    const uint32_t *order;
    int sk_bits;
} sort_ctx;

/* sort.c:629-646 (with the mode order of SortIndexCustomOrder, :523-552). */
static int cmp_lex(const void *c, uint64_t a, uint64_t b) {
    const sort_ctx *s = (const sort_ctx *)c;
    for (uint32_t i = 0; i < s->nmodes; ++i) {
        const uint32_t m = s->order[i];
        const uint32_t x = s->inds[m][a], y = s->inds[m][b];
        if (x < y) return -1;
        if (x > y) return 1;
    }
    return 0;
}

/* The same orders through packed keys, for inputs of 10^8 nonzeros: each
 * nonzero gets a 192-bit key (w[0] most significant) whose unsigned order is
 * the comparison order above, and (key, position) pairs are merge-sorted in
 * parallel (ties keep input order, as msort does).  orc_sort_keyed_check
 * (tests/test_oracle_sorts.py) checks both paths give one permutation. */
typedef struct {
    uint64_t w[3];
    uint64_t i;
} keyed;

static inline int keyed_less(const keyed *a, const keyed *b) {
    for (int k = 0; k < 3; ++k)
        if (a->w[k] != b->w[k]) return a->w[k] < b->w[k];
    return a->i < b->i;
}

static void keyed_merge(const keyed *a, uint64_t na, const keyed *b, uint64_t nb, keyed *out) {
    uint64_t i = 0, j = 0, k = 0;
    while (i < na && j < nb) out[k++] = keyed_less(&b[j], &a[i]) ? b[j++] : a[i++];
    while (i < na) out[k++] = a[i++];
    while (j < nb) out[k++] = b[j++];
}

static void keyed_msort_seq(keyed *a, keyed *tmp, uint64_t n) {
    if (n < 2) return;
    if (n <= 16) {
        for (uint64_t i = 1; i < n; ++i) {
            keyed x = a[i];
            uint64_t j = i;
            while (j > 0 && keyed_less(&x, &a[j - 1])) {
                a[j] = a[j - 1];
                --j;
            }
            a[j] = x;
        }
        return;
    }
    const uint64_t h = n / 2;
    keyed_msort_seq(a, tmp, h);
    keyed_msort_seq(a + h, tmp + h, n - h);
    keyed_merge(a, h, a + h, n - h, tmp);
    memcpy(a, tmp, n * sizeof *a);
}

/* T sorted runs (one per thread), then log2(T) rounds of pairwise merges. */
static int keyed_sort(keyed *a, uint64_t n) {
    keyed *tmp = (keyed *)malloc((n ? n : 1) * sizeof *tmp);
    if (!tmp) return 1;
    int T = omp_get_max_threads();
    if (T < 1) T = 1;
    if ((uint64_t)T > n / 4096 + 1) T = (int)(n / 4096 + 1);
    uint64_t *cut = (uint64_t *)malloc((T + 1) * sizeof *cut);
    for (int t = 0; t <= T; ++t) cut[t] = n * (uint64_t)t / (uint64_t)T;
#pragma omp parallel for schedule(dynamic, 1) num_threads(T)
    for (int t = 0; t < T; ++t) keyed_msort_seq(a + cut[t], tmp + cut[t], cut[t + 1] - cut[t]);
    keyed *src = a, *dst = tmp;
    for (int width = 1; width < T; width *= 2) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int t = 0; t < T; t += 2 * width) {
            const int m = t + width < T ? t + width : T, e = t + 2 * width < T ? t + 2 * width : T;
            keyed_merge(src + cut[t], cut[m] - cut[t], src + cut[m], cut[e] - cut[m], dst + cut[t]);
        }
        keyed *x = src;
        src = dst;
        dst = x;
    }
    if (src != a) memcpy(a, src, n * sizeof *a);
    free(cut);
    free(tmp);
    return 0;
}

static int bits_of(uint32_t v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

/* Appends the low `bits` bits of v (bits <= 32) below the `used` bits
 * already placed in the 192-bit key w (w[0] most significant). */
static inline void key_push(uint64_t *w, int *used, uint64_t v, int bits) {
    if (bits == 0) return;
    const int lo = 192 - *used - bits;   /* bit index of v's bit 0, from the least significant end */
    const int q = 2 - lo / 64, off = lo % 64;
    w[q] |= v << off;
    if (off + bits > 64) w[q - 1] |= v >> (64 - off);
    *used += bits;
}

static int orc_sort_lex_keyed(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const uint32_t *order,
                              uint64_t *perm) {
    int bits[ORC_MAX_MODES], total = 0;
    for (uint32_t k = 0; k < nmodes; ++k) {
        uint32_t mx = 0;
        const uint32_t *a = inds[order[k]];
#pragma omp parallel for reduction(max : mx)
        for (uint64_t x = 0; x < nnz; ++x) mx = a[x] > mx ? a[x] : mx;
        bits[k] = bits_of(mx);
        total += bits[k];
    }
    if (total > 192) return -1;
    keyed *a = (keyed *)malloc((nnz ? nnz : 1) * sizeof *a);
    if (!a) return 1;
#pragma omp parallel for schedule(static)
    for (uint64_t x = 0; x < nnz; ++x) {
        keyed e = {{0, 0, 0}, x};
        int used = 0;
        for (uint32_t k = 0; k < nmodes; ++k) key_push(e.w, &used, inds[order[k]][x], bits[k]);
        a[x] = e;
    }
    int r = keyed_sort(a, nnz);
#pragma omp parallel for schedule(static)
    for (uint64_t x = 0; x < nnz; ++x) perm[x] = a[x].i;
    free(a);
    return r;
}

int orc_sort_lex(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const uint32_t *order, uint64_t *perm) {
    if (nnz >= (1u << 20)) {
        const int r = orc_sort_lex_keyed(nmodes, nnz, inds, order, perm);
        if (r >= 0) return r;
    }
    uint64_t *tmp = (uint64_t *)malloc((nnz ? nnz : 1) * sizeof *tmp);
    if (!tmp) return 1;
    for (uint64_t i = 0; i < nnz; ++i) perm[i] = i;
    sort_ctx c = {nmodes, inds, order, 0};
    msort(perm, tmp, nnz, cmp_lex, &c);
    free(tmp);
    return 0;
}

/* Byte-spread tables of sort.c:55-164 as a computation: bit i of the byte
 * goes to bit 3i (z), 3i+1 (y), 3i+2 (x). */
static uint32_t spread3(uint32_t byte) {
    uint32_t r = 0;
    for (int i = 0; i < 8; ++i) r |= ((byte >> i) & 1u) << (3 * i);
    return r;
}

/* sort.c:754-795: the 128-bit key built byte by byte from the top; the
 * highest byte's contribution is shifted past bit 127. */
static unsigned __int128 morton3(uint32_t x, uint32_t y, uint32_t z) {
    unsigned __int128 k;
    k = (unsigned __int128)((spread3((z >> 24) & 0xFF)) | (spread3((y >> 24) & 0xFF) << 1) |
                            (spread3((x >> 24) & 0xFF) << 2));
    k = (k << 72) | (spread3((z >> 16) & 0xFF) | (spread3((y >> 16) & 0xFF) << 1) | (spread3((x >> 16) & 0xFF) << 2));
    k = (k << 48) | (spread3((z >> 8) & 0xFF) | (spread3((y >> 8) & 0xFF) << 1) | (spread3((x >> 8) & 0xFF) << 2));
    k = (k << 24) | (spread3(z & 0xFF) | (spread3(y & 0xFF) << 1) | (spread3(x & 0xFF) << 2));
    return k;
}

/* sort.c:852-917: every coordinate bit i to bit 4i; key = w | z<<1 | y<<2 | x<<3. */
static unsigned __int128 spread4(uint32_t v) {
    unsigned __int128 r = 0;
    for (int i = 0; i < 32; ++i) r |= (unsigned __int128)((v >> i) & 1u) << (4 * i);
    return r;
}
static unsigned __int128 morton4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
    return spread4(w) | (spread4(z) << 1) | (spread4(y) << 2) | (spread4(x) << 3);
}

/* Row-block compare (sort.c:713-737) then Morton compare (sort.c:748-995):
 * the order left by spt_PreprocessSparseTensor (hicoo/convert.c:160-226). */
static int cmp_hicoo(const void *c, uint64_t a, uint64_t b) {
    const sort_ctx *s = (const sort_ctx *)c;
    for (uint32_t m = 0; m < s->nmodes; ++m) {
        const uint32_t x = s->inds[m][a] >> s->sk_bits, y = s->inds[m][b] >> s->sk_bits;
        if (x < y) return -1;
        if (x > y) return 1;
    }
    unsigned __int128 ka = 0, kb = 0;
    if (s->nmodes == 3) {
        ka = morton3(s->inds[0][a], s->inds[1][a], s->inds[2][a]);
        kb = morton3(s->inds[0][b], s->inds[1][b], s->inds[2][b]);
    } else if (s->nmodes == 4) {
        ka = morton4(s->inds[0][a], s->inds[1][a], s->inds[2][a], s->inds[3][a]);
        kb = morton4(s->inds[0][b], s->inds[1][b], s->inds[2][b], s->inds[3][b]);
    }
    return ka < kb ? -1 : (ka > kb ? 1 : 0);
}

/* HiCOO order through keys: w[0] the kernel coordinates (idx >> sk_bits,
 * mode 0 most significant), w[1..2] the Morton key of morton3 / morton4. */
static int orc_sort_hicoo_keyed(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, int sk_bits,
                                uint64_t *perm) {
    if (nmodes != 3 && nmodes != 4) return -1;
    int bits[ORC_MAX_MODES], total = 0;
    for (uint32_t m = 0; m < nmodes; ++m) {
        uint32_t mx = 0;
        const uint32_t *a = inds[m];
#pragma omp parallel for reduction(max : mx)
        for (uint64_t x = 0; x < nnz; ++x) mx = a[x] > mx ? a[x] : mx;
        bits[m] = bits_of(mx >> sk_bits);
        total += bits[m];
    }
    if (total > 64) return -1;
    keyed *a = (keyed *)malloc((nnz ? nnz : 1) * sizeof *a);
    if (!a) return 1;
#pragma omp parallel for schedule(static)
    for (uint64_t x = 0; x < nnz; ++x) {
        keyed e = {{0, 0, 0}, x};
        uint64_t kk = 0;
        for (uint32_t m = 0; m < nmodes; ++m) kk = (kk << bits[m]) | (uint64_t)(inds[m][x] >> sk_bits);
        const unsigned __int128 mk = nmodes == 3 ? morton3(inds[0][x], inds[1][x], inds[2][x])
                                                 : morton4(inds[0][x], inds[1][x], inds[2][x], inds[3][x]);
        e.w[0] = kk;
        e.w[1] = (uint64_t)(mk >> 64);
        e.w[2] = (uint64_t)mk;
        a[x] = e;
    }
    int r = keyed_sort(a, nnz);
#pragma omp parallel for schedule(static)
    for (uint64_t x = 0; x < nnz; ++x) perm[x] = a[x].i;
    free(a);
    return r;
}

/* Both paths on one input (test hook): 0 when they give one permutation. */
int orc_sort_keyed_check(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const uint32_t *order,
                         int sk_bits) {
    uint64_t *p1 = (uint64_t *)malloc((nnz ? nnz : 1) * 8), *p2 = (uint64_t *)malloc((nnz ? nnz : 1) * 8);
    uint64_t *tmp = (uint64_t *)malloc((nnz ? nnz : 1) * 8);
    int bad = 0;
    for (uint64_t i = 0; i < nnz; ++i) p1[i] = i;
    if (order) {
        sort_ctx c = {nmodes, inds, order, 0};
        msort(p1, tmp, nnz, cmp_lex, &c);
        bad = orc_sort_lex_keyed(nmodes, nnz, inds, order, p2) != 0;
    } else {
        sort_ctx c = {nmodes, inds, NULL, sk_bits};
        msort(p1, tmp, nnz, cmp_hicoo, &c);
        bad = orc_sort_hicoo_keyed(nmodes, nnz, inds, sk_bits, p2) != 0;
    }
    for (uint64_t i = 0; i < nnz && !bad; ++i) bad = p1[i] != p2[i];
    free(p1);
    free(p2);
    free(tmp);
    return bad;
}

int orc_sort_hicoo(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, int sk_bits, uint64_t *perm) {
    if (nnz >= (1u << 20)) {
        const int r = orc_sort_hicoo_keyed(nmodes, nnz, inds, sk_bits, perm);
        if (r >= 0) return r;
    }
    uint64_t *tmp = (uint64_t *)malloc((nnz ? nnz : 1) * sizeof *tmp);
    if (!tmp) return 1;
    for (uint64_t i = 0; i < nnz; ++i) perm[i] = i;
    sort_ctx c = {nmodes, inds, NULL, sk_bits};
    msort(perm, tmp, nnz, cmp_hicoo, &c);
    free(tmp);
    return 0;
}

/* ---------------------------------------------------------- HiCOO build --
 * hicoo/convert.c:103-146 (kschr), :237-288 (kernel pointers), :300-497
 * (blocks, chunks, elements), on a COO already in HiCOO order.  Outputs
 * (caller-sized: nb <= nnz, nk <= nnz, ncptr <= nb + nk + 1, kschr
 * nmodes * nk entries, kschr_len sum over modes of ceil(ndims/2^sk)). */
typedef struct {
    uint64_t nb, nk, ncptr, max_nnzb;
    uint64_t *bptr, *kptr, *cptr;
    uint32_t *binds;   /* [nmodes][nb] */
    uint8_t *einds;    /* [nmodes][nnz] */
    uint32_t *nkiters; /* [nmodes] */
    uint32_t *kschr_len;
    uint32_t *kschr;
} orc_hicoo;

int orc_hicoo_build(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, const uint32_t *const *inds, int sb_bits,
                    int sk_bits, orc_hicoo *h) {
    const uint64_t sc = 1ull << 14;
    if (nnz == 0) return 1;
    /* kernel starts (convert.c:237-288) */
    uint64_t *kstart = (uint64_t *)malloc((nnz + 1) * sizeof *kstart);
    uint64_t nk = 0;
    for (uint64_t z = 0; z < nnz; ++z) {
        int diff = (z == 0);
        for (uint32_t m = 0; m < nmodes && z; ++m) diff |= (inds[m][z] >> sk_bits) != (inds[m][z - 1] >> sk_bits);
        if (diff) kstart[nk++] = z;
    }
    kstart[nk] = nnz;
    /* kschr (convert.c:117-143) */
    uint32_t *row_off = (uint32_t *)calloc(ORC_MAX_MODES, sizeof(uint32_t));
    uint64_t tot_rows = 0;
    for (uint32_t m = 0; m < nmodes; ++m) {
        row_off[m] = (uint32_t)tot_rows;
        tot_rows += ((uint64_t)ndims[m] + (1ull << sk_bits) - 1) >> sk_bits;
    }
    memset(h->kschr_len, 0, tot_rows * sizeof(uint32_t));
    for (uint64_t k = 0; k < nk; ++k)
        for (uint32_t m = 0; m < nmodes; ++m) h->kschr_len[row_off[m] + (inds[m][kstart[k]] >> sk_bits)]++;
    /* entries in kernel order within each kernel row */
    uint64_t *fill = (uint64_t *)calloc(tot_rows + 1, sizeof(uint64_t));
    for (uint64_t r = 0; r < tot_rows; ++r) fill[r + 1] = fill[r] + h->kschr_len[r];
    for (uint64_t k = 0; k < nk; ++k)
        for (uint32_t m = 0; m < nmodes; ++m) {
            const uint64_t r = row_off[m] + (inds[m][kstart[k]] >> sk_bits);
            h->kschr[fill[r]++] = (uint32_t)k;
        }
    for (uint32_t m = 0; m < nmodes; ++m) {
        uint32_t mx = 0;
        const uint64_t kn = ((uint64_t)ndims[m] + (1ull << sk_bits) - 1) >> sk_bits;
        for (uint64_t i = 0; i < kn; ++i)
            if (h->kschr_len[row_off[m] + i] > mx) mx = h->kschr_len[row_off[m] + i];
        h->nkiters[m] = mx;
    }
    /* element / block / chunk emission (convert.c:372-472) */
    uint64_t nb = 1, ne = 0, chunk = 0, nc = 0;
    uint32_t prior[ORC_MAX_MODES];
    for (uint32_t m = 0; m < nmodes; ++m) {
        prior[m] = inds[m][0] >> sb_bits;
        h->binds[(uint64_t)m * nnz + 0] = prior[m];
    }
    h->bptr[0] = 0;
    uint64_t nbptr = 1;
    for (uint64_t k = 0; k < nk; ++k) {
        const uint64_t nb_tmp = k == 0 ? 0 : nb;
        h->kptr[k] = nb_tmp;
        h->cptr[nc++] = nb_tmp;
        chunk = 0;
        for (uint64_t z = kstart[k]; z < kstart[k + 1]; ++z) {
            int same = 1;
            uint32_t blk[ORC_MAX_MODES];
            for (uint32_t m = 0; m < nmodes; ++m) {
                blk[m] = inds[m][z] >> sb_bits;
                h->einds[(uint64_t)m * nnz + z] = (uint8_t)(inds[m][z] - (blk[m] << sb_bits));
                same &= blk[m] == prior[m];
            }
            if (same) {
                ++ne;
            } else {
                h->bptr[nbptr++] = (uint64_t)(uint32_t)z;
                for (uint32_t m = 0; m < nmodes; ++m) {
                    h->binds[(uint64_t)m * nnz + nb] = blk[m];
                    prior[m] = blk[m];
                }
                if (chunk + ne >= sc) {
                    h->cptr[nc++] = nb;
                    chunk = 0;
                } else {
                    chunk += ne;
                }
                ++nb;
                ne = 1;
            }
        }
    }
    h->kptr[nk] = nbptr;
    h->cptr[nc++] = nbptr;
    h->bptr[nbptr] = nnz;
    h->nb = nb;
    h->nk = nk;
    h->ncptr = nc;
    uint64_t mx = h->bptr[1] - h->bptr[0];
    for (uint64_t b = 0; b < nb; ++b)
        if (h->bptr[b + 1] - h->bptr[b] > mx) mx = h->bptr[b + 1] - h->bptr[b];
    h->max_nnzb = mx;
    /* binds were written with a row length of nnz; compact to nb */
    for (uint32_t m = 1; m < nmodes; ++m) memmove(h->binds + (uint64_t)m * nb, h->binds + (uint64_t)m * nnz, nb * 4);
    free(kstart);
    free(row_off);
    free(fill);
    return 0;
}

/* ------------------------------------------------------------- MTTKRP --
 * mttkrp.c:39-115 (order >= 4) and :118-177 (3-D): per nonzero the product
 * entry * F[o1][i1] * F[o2][i2] ... (left to right), added to the output
 * row in nonzero order, FP32. */
void orc_mttkrp_f32(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const float *vals,
                    const float *const *mats, uint32_t stride, uint32_t R, const uint32_t *mats_order, uint32_t mode,
                    uint32_t out_rows, float *out) {
    memset(out, 0, (size_t)out_rows * stride * sizeof(float));
    float scratch[1024];
    for (uint64_t x = 0; x < nnz; ++x) {
        const float entry = vals[x];
        const uint32_t o1 = mats_order[1];
        const float *r1 = mats[o1] + (size_t)inds[o1][x] * stride;
        for (uint32_t r = 0; r < R; ++r) scratch[r] = entry * r1[r];
        for (uint32_t i = 2; i < nmodes; ++i) {
            const uint32_t oi = mats_order[i];
            const float *ri = mats[oi] + (size_t)inds[oi][x] * stride;
            for (uint32_t r = 0; r < R; ++r) scratch[r] *= ri[r];
        }
        float *o = out + (size_t)inds[mode][x] * stride;
        for (uint32_t r = 0; r < R; ++r) o[r] += scratch[r];
    }
}

/* Same loop in FP64 (products and sums), the precision reference. */
void orc_mttkrp_f64(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const float *vals,
                    const float *const *mats, uint32_t stride, uint32_t R, const uint32_t *mats_order, uint32_t mode,
                    uint32_t out_rows, double *out) {
    memset(out, 0, (size_t)out_rows * stride * sizeof(double));
    double scratch[1024];
    for (uint64_t x = 0; x < nnz; ++x) {
        const double entry = vals[x];
        const uint32_t o1 = mats_order[1];
        const float *r1 = mats[o1] + (size_t)inds[o1][x] * stride;
        for (uint32_t r = 0; r < R; ++r) scratch[r] = entry * (double)r1[r];
        for (uint32_t i = 2; i < nmodes; ++i) {
            const uint32_t oi = mats_order[i];
            const float *ri = mats[oi] + (size_t)inds[oi][x] * stride;
            for (uint32_t r = 0; r < R; ++r) scratch[r] *= (double)ri[r];
        }
        double *o = out + (size_t)inds[mode][x] * stride;
        for (uint32_t r = 0; r < R; ++r) o[r] += scratch[r];
    }
}

/* orc_mttkrp_f64 over threads: static schedule over nonzeros into
 * per-thread FP64 outputs, added in thread order (the FP64 checker for
 * tensors too large for one core). */
void orc_omp_mttkrp_f64(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const float *vals,
                        const float *const *mats, uint32_t stride, uint32_t R, const uint32_t *mats_order, uint32_t mode,
                        uint32_t out_rows, double *out, int tk) {
    const size_t csz = (size_t)out_rows * stride;
    double *copies = (double *)calloc((size_t)tk * csz, sizeof(double));
    if (!copies) return;
#pragma omp parallel num_threads(tk)
    {
        const int t = omp_get_thread_num();
        const uint64_t lo = nnz * (uint64_t)t / (uint64_t)tk, hi = nnz * (uint64_t)(t + 1) / (uint64_t)tk;
        double *cp = copies + (size_t)t * csz;
        double scratch[1024];
        for (uint64_t x = lo; x < hi; ++x) {
            const double entry = vals[x];
            const uint32_t o1 = mats_order[1];
            const float *r1 = mats[o1] + (size_t)inds[o1][x] * stride;
            for (uint32_t r = 0; r < R; ++r) scratch[r] = entry * (double)r1[r];
            for (uint32_t i = 2; i < nmodes; ++i) {
                const uint32_t oi = mats_order[i];
                const float *ri = mats[oi] + (size_t)inds[oi][x] * stride;
                for (uint32_t r = 0; r < R; ++r) scratch[r] *= (double)ri[r];
            }
            double *o = cp + (size_t)inds[mode][x] * stride;
            for (uint32_t r = 0; r < R; ++r) o[r] += scratch[r];
        }
    }
#pragma omp parallel for schedule(static) num_threads(tk)
    for (uint64_t i = 0; i < csz; ++i) {
        double acc = 0.0;
        for (int t = 0; t < tk; ++t) acc += copies[(size_t)t * csz + i];
        out[i] = acc;
    }
    free(copies);
}

/* mttkrp_omp.c:401-476: privatised per-thread outputs, static schedule over
 * nonzeros, then a row-parallel reduction over threads. */
void orc_omp_mttkrp_reduce(uint32_t nmodes, uint64_t nnz, const uint32_t *const *inds, const float *vals,
                           const float *const *mats, uint32_t stride, uint32_t R, const uint32_t *mats_order,
                           uint32_t mode, uint32_t out_rows, float *out, int tk, float *copies) {
    memset(out, 0, (size_t)out_rows * stride * sizeof(float));
    const size_t csz = (size_t)out_rows * stride;
    memset(copies, 0, (size_t)tk * csz * sizeof(float));
#pragma omp parallel for schedule(static) num_threads(tk)
    for (uint64_t x = 0; x < nnz; ++x) {
        float *cp = copies + (size_t)omp_get_thread_num() * csz;
        float scratch[1024];
        const float entry = vals[x];
        const uint32_t o1 = mats_order[1];
        const float *r1 = mats[o1] + (size_t)inds[o1][x] * stride;
        for (uint32_t r = 0; r < R; ++r) scratch[r] = entry * r1[r];
        for (uint32_t i = 2; i < nmodes; ++i) {
            const uint32_t oi = mats_order[i];
            const float *ri = mats[oi] + (size_t)inds[oi][x] * stride;
            for (uint32_t r = 0; r < R; ++r) scratch[r] *= ri[r];
        }
        float *o = cp + (size_t)inds[mode][x] * stride;
        for (uint32_t r = 0; r < R; ++r) o[r] += scratch[r];
    }
#pragma omp parallel for schedule(static) num_threads(tk)
    for (uint32_t i = 0; i < out_rows; ++i)
        for (int t = 0; t < tk; ++t)
            for (uint32_t r = 0; r < R; ++r) out[(size_t)i * stride + r] += copies[(size_t)t * csz + (size_t)i * stride + r];
}

/* hicoo/mttkrp.c:53-144: kernels -> blocks -> elements, coordinates
 * (binds << sb_bits) + einds. */
void orc_mttkrp_hicoo_f32(uint32_t nmodes, uint64_t nb, const uint64_t *bptr, const uint32_t *const *binds,
                          const uint8_t *const *einds, const float *vals, int sb_bits, const float *const *mats,
                          uint32_t stride, uint32_t R, const uint32_t *mats_order, uint32_t mode, uint32_t out_rows,
                          float *out) {
    memset(out, 0, (size_t)out_rows * stride * sizeof(float));
    float scratch[1024];
    uint32_t c[ORC_MAX_MODES];
    for (uint64_t b = 0; b < nb; ++b) {
        for (uint64_t z = bptr[b]; z < bptr[b + 1]; ++z) {
            for (uint32_t m = 0; m < nmodes; ++m) c[m] = (binds[m][b] << sb_bits) + einds[m][z];
            const float entry = vals[z];
            const uint32_t o1 = mats_order[1];
            const float *r1 = mats[o1] + (size_t)c[o1] * stride;
            for (uint32_t r = 0; r < R; ++r) scratch[r] = entry * r1[r];
            for (uint32_t i = 2; i < nmodes; ++i) {
                const uint32_t oi = mats_order[i];
                const float *ri = mats[oi] + (size_t)c[oi] * stride;
                for (uint32_t r = 0; r < R; ++r) scratch[r] *= ri[r];
            }
            float *o = out + (size_t)c[mode] * stride;
            for (uint32_t r = 0; r < R; ++r) o[r] += scratch[r];
        }
    }
}

/* hicoo/mttkrp_omp.c:1214-1296 (3-D MatrixTiling_Scheduled_Reduce): a dynamic
 * parallel loop (chunk 1, mttkrp_omp.c:22) over the schedule iterations
 * i < nkiters; in iteration i, kernel i of every kernel row (kschr[mode][k][i],
 * kernel rows in order), its blocks in order, the elements of a block in
 * order, each thread summing into its own output copy; then the copies are
 * added row by row in thread order.  The kernel rows of `mode` are given
 * flattened: kernel ids ks_ids[ks_off[k] .. ks_off[k+1]). */
void orc_omp_mttkrp_hicoo_reduce(uint32_t nmodes, const uint64_t *bptr, const uint32_t *const *binds,
                                 const uint8_t *const *einds, const float *vals, int sb_bits, const uint64_t *kptr,
                                 uint32_t nkrows, const uint64_t *ks_off, const uint32_t *ks_ids, uint32_t nkiters,
                                 const float *const *mats, uint32_t stride, uint32_t R, const uint32_t *mats_order,
                                 uint32_t mode, uint32_t out_rows, float *out, int tk, float *copies) {
    if (nmodes != 3) return;
    memset(out, 0, (size_t)out_rows * stride * sizeof(float));
    const size_t csz = (size_t)out_rows * stride;
    memset(copies, 0, (size_t)tk * csz * sizeof(float));
    const uint32_t m1 = mats_order[1], m2 = mats_order[2];
#pragma omp parallel for schedule(dynamic, 1) num_threads(tk)
    for (uint32_t i = 0; i < nkiters; ++i) {
        float *cp = copies + (size_t)omp_get_thread_num() * csz;
        for (uint32_t k = 0; k < nkrows; ++k) {
            if (i >= ks_off[k + 1] - ks_off[k]) continue;
            const uint32_t kid = ks_ids[ks_off[k] + i];
            for (uint64_t b = kptr[kid]; b < kptr[kid + 1]; ++b) {
                float *bo = cp + (size_t)(binds[mode][b] << sb_bits) * stride;
                const float *b1 = mats[m1] + (size_t)(binds[m1][b] << sb_bits) * stride;
                const float *b2 = mats[m2] + (size_t)(binds[m2][b] << sb_bits) * stride;
                for (uint64_t z = bptr[b]; z < bptr[b + 1]; ++z) {
                    const float entry = vals[z];
                    float *o = bo + (size_t)einds[mode][z] * stride;
                    const float *r1 = b1 + (size_t)einds[m1][z] * stride;
                    const float *r2 = b2 + (size_t)einds[m2][z] * stride;
                    for (uint32_t r = 0; r < R; ++r) o[r] += entry * r1[r] * r2[r];
                }
            }
        }
    }
#pragma omp parallel for schedule(static) num_threads(tk)
    for (uint32_t i = 0; i < out_rows; ++i)
        for (int t = 0; t < tk; ++t)
            for (uint32_t r = 0; r < R; ++r) out[(size_t)i * stride + r] += copies[(size_t)t * csz + (size_t)i * stride + r];
}

/* -------------------------------------------------------------- CP-ALS --
 * cpd.c:32-137 restated in FP64 with a correct fit:
 *   Grams A^T A (full), per iteration and mode: MTTKRP, solve with the
 *   Hadamard of the other Grams (Cholesky; Gaussian elimination with partial
 *   pivoting when not positive definite, as matrix_solver.c:48-80 falls back
 *   from spotrf_ to sgesv_), 2-norm at iteration 0 else max-norm clamped to
 *   >= 1 (matrix.c:390-554), new Gram; then
 *   fit = 1 - r / ||X|| with r = sqrt(res) if res > 0 else res,
 *   res = ||X||^2 + ||K||^2 - 2 <X,K> (ktensor.c:102-120), ||K||^2 from full
 *   symmetric Grams, <X,K> from the last mode's MTTKRP (ktensor.c:173-257);
 *   GetFinalLambda (matrix.c:557-573) at the end.
 * Factors enter and leave as FP32 arrays of ndims[m] x stride. */
/* Threads of the FP64 CP-ALS restatement (orc_set_threads); 1 keeps the
 * sequential loops that the reference trace is pinned with.  Row solves are
 * independent per row; with more threads the Gram and MTTKRP sums are split
 * into per-thread partials added in thread order. */
static int orc_threads = 1;
void orc_set_threads(int t) { orc_threads = t < 1 ? 1 : t; }

static int solve_rows_f64(double *H, int R, double *X, uint64_t nrows, int ld) {
    /* Cholesky H = L L^T in place (lower). */
    double *L = (double *)malloc((size_t)R * R * sizeof(double));
    memcpy(L, H, (size_t)R * R * sizeof(double));
    int spd = 1;
    for (int k = 0; k < R && spd; ++k) {
        double d = L[k * R + k];
        for (int j = 0; j < k; ++j) d -= L[k * R + j] * L[k * R + j];
        if (!(d > 0.0)) {
            spd = 0;
            break;
        }
        L[k * R + k] = sqrt(d);
        for (int i = k + 1; i < R; ++i) {
            double s = L[i * R + k];
            for (int j = 0; j < k; ++j) s -= L[i * R + j] * L[k * R + j];
            L[i * R + k] = s / L[k * R + k];
        }
    }
    if (spd) {
#pragma omp parallel for schedule(static) num_threads(orc_threads)
        for (uint64_t i = 0; i < nrows; ++i) {
            double *x = X + i * ld;
            for (int r = 0; r < R; ++r) {
                double s = x[r];
                for (int j = 0; j < r; ++j) s -= L[r * R + j] * x[j];
                x[r] = s / L[r * R + r];
            }
            for (int r = R - 1; r >= 0; --r) {
                double s = x[r];
                for (int j = r + 1; j < R; ++j) s -= L[j * R + r] * x[j];
                x[r] = s / L[r * R + r];
            }
        }
        free(L);
        return 0;
    }
    /* LU with partial pivoting of H, solve H x = m per row.  An exactly zero
     * pivot leaves the rows unsolved, as sgesv_ returns with info > 0 and the
     * right-hand sides untouched (matrix_solver.c:66-80). */
    int *piv = (int *)malloc(R * sizeof(int));
    memcpy(L, H, (size_t)R * R * sizeof(double));
    int zero_pivot = 0;
    for (int k = 0; k < R; ++k) {
        int p = k;
        for (int i = k + 1; i < R; ++i)
            if (fabs(L[i * R + k]) > fabs(L[p * R + k])) p = i;
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < R; ++j) {
                double t = L[k * R + j];
                L[k * R + j] = L[p * R + j];
                L[p * R + j] = t;
            }
        if (L[k * R + k] != 0.0)
            for (int i = k + 1; i < R; ++i) {
                L[i * R + k] /= L[k * R + k];
                for (int j = k + 1; j < R; ++j) L[i * R + j] -= L[i * R + k] * L[k * R + j];
            }
        else
            zero_pivot = 1;
    }
    if (zero_pivot) {
        free(piv);
        free(L);
        return 2;
    }
#pragma omp parallel for schedule(static) num_threads(orc_threads)
    for (uint64_t i = 0; i < nrows; ++i) {
        double *x = X + i * ld;
        for (int k = 0; k < R; ++k) {
            double t = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = t;
        }
        for (int r = 0; r < R; ++r)
            for (int j = 0; j < r; ++j) x[r] -= L[r * R + j] * x[j];
        for (int r = R - 1; r >= 0; --r) {
            for (int j = r + 1; j < R; ++j) x[r] -= L[r * R + j] * x[j];
            x[r] /= L[r * R + r];
        }
    }
    free(piv);
    free(L);
    return 1;
}

static void gram_f64(const double *A, uint64_t nrows, int R, int ld, double *G) {
    memset(G, 0, (size_t)R * R * sizeof(double));
    if (orc_threads == 1) {
        for (uint64_t i = 0; i < nrows; ++i)
            for (int p = 0; p < R; ++p)
                for (int q = p; q < R; ++q) G[p * R + q] += A[i * ld + p] * A[i * ld + q];
    } else {
        const int tk = orc_threads;
        double *part = (double *)calloc((size_t)tk * R * R, sizeof(double));
#pragma omp parallel num_threads(tk)
        {
            const int t = omp_get_thread_num();
            double *g = part + (size_t)t * R * R;
            for (uint64_t i = nrows * (uint64_t)t / tk; i < nrows * (uint64_t)(t + 1) / tk; ++i)
                for (int p = 0; p < R; ++p)
                    for (int q = p; q < R; ++q) g[p * R + q] += A[i * ld + p] * A[i * ld + q];
        }
        for (int t = 0; t < tk; ++t)
            for (int e = 0; e < R * R; ++e) G[e] += part[(size_t)t * R * R + e];
        free(part);
    }
    for (int p = 0; p < R; ++p)
        for (int q = 0; q < p; ++q) G[p * R + q] = G[q * R + p];
}

int orc_cpd_als_f64(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, const uint32_t *const *inds,
                    const float *vals, uint32_t R, uint32_t niters, double tol, float *const *factors, uint32_t stride,
                    float *lambda_out, double *fits, uint32_t *iters_done) {
    double *A[ORC_MAX_MODES], *G[ORC_MAX_MODES];
    uint32_t maxd = 0;
    for (uint32_t m = 0; m < nmodes; ++m) {
        A[m] = (double *)malloc((size_t)ndims[m] * R * sizeof(double));
        for (uint64_t i = 0; i < ndims[m]; ++i)
            for (uint32_t r = 0; r < R; ++r) A[m][i * R + r] = factors[m][i * stride + r];
        G[m] = (double *)malloc((size_t)R * R * sizeof(double));
        gram_f64(A[m], ndims[m], (int)R, (int)R, G[m]);
        if (ndims[m] > maxd) maxd = ndims[m];
    }
    double *M = (double *)malloc((size_t)maxd * R * sizeof(double));
    double *H = (double *)malloc((size_t)R * R * sizeof(double));
    double *lam = (double *)malloc(R * sizeof(double));
    double *sc = (double *)malloc(1024 * sizeof(double));
    double normX2 = 0.0;
    for (uint64_t x = 0; x < nnz; ++x) normX2 += (double)vals[x] * vals[x];
    double oldfit = 0.0;
    uint32_t done = 0;
    for (uint32_t it = 0; it < niters; ++it) {
        for (uint32_t m = 0; m < nmodes; ++m) {
            uint32_t order[ORC_MAX_MODES];
            order[0] = m;
            for (uint32_t i = 1; i < nmodes; ++i) order[i] = (m + i) % nmodes;
            memset(M, 0, (size_t)ndims[m] * R * sizeof(double));
            if (orc_threads == 1) {
                for (uint64_t x = 0; x < nnz; ++x) {
                    for (uint32_t r = 0; r < R; ++r) sc[r] = vals[x] * A[order[1]][(size_t)inds[order[1]][x] * R + r];
                    for (uint32_t i = 2; i < nmodes; ++i)
                        for (uint32_t r = 0; r < R; ++r) sc[r] *= A[order[i]][(size_t)inds[order[i]][x] * R + r];
                    double *o = M + (size_t)inds[m][x] * R;
                    for (uint32_t r = 0; r < R; ++r) o[r] += sc[r];
                }
            } else {
                const int tk = orc_threads;
                const size_t csz = (size_t)ndims[m] * R;
                double *cp = (double *)calloc((size_t)tk * csz, sizeof(double));
#pragma omp parallel num_threads(tk)
                {
                    const int t = omp_get_thread_num();
                    double *o0 = cp + (size_t)t * csz, s2[1024];
                    for (uint64_t x = nnz * (uint64_t)t / tk; x < nnz * (uint64_t)(t + 1) / tk; ++x) {
                        for (uint32_t r = 0; r < R; ++r)
                            s2[r] = vals[x] * A[order[1]][(size_t)inds[order[1]][x] * R + r];
                        for (uint32_t i = 2; i < nmodes; ++i)
                            for (uint32_t r = 0; r < R; ++r) s2[r] *= A[order[i]][(size_t)inds[order[i]][x] * R + r];
                        double *o = o0 + (size_t)inds[m][x] * R;
                        for (uint32_t r = 0; r < R; ++r) o[r] += s2[r];
                    }
                }
#pragma omp parallel for schedule(static) num_threads(tk)
                for (uint64_t i = 0; i < csz; ++i) {
                    double acc = 0.0;
                    for (int t = 0; t < tk; ++t) acc += cp[(size_t)t * csz + i];
                    M[i] = acc;
                }
                free(cp);
            }
            for (uint32_t e = 0; e < R * R; ++e) {
                double v = 1.0;
                for (uint32_t k = 1; k < nmodes; ++k) v *= G[(m + k) % nmodes][e];
                H[e] = v;
            }
            memcpy(A[m], M, (size_t)ndims[m] * R * sizeof(double));
            solve_rows_f64(H, (int)R, A[m], ndims[m], (int)R);
            for (uint32_t r = 0; r < R; ++r) lam[r] = 0.0;
            if (it == 0) {
                for (uint64_t i = 0; i < ndims[m]; ++i)
                    for (uint32_t r = 0; r < R; ++r) lam[r] += A[m][i * R + r] * A[m][i * R + r];
                for (uint32_t r = 0; r < R; ++r) lam[r] = sqrt(lam[r]);
            } else {
                for (uint64_t i = 0; i < ndims[m]; ++i)
                    for (uint32_t r = 0; r < R; ++r)
                        if (A[m][i * R + r] > lam[r]) lam[r] = A[m][i * R + r];
                for (uint32_t r = 0; r < R; ++r)
                    if (lam[r] < 1.0) lam[r] = 1.0;
            }
            for (uint64_t i = 0; i < ndims[m]; ++i)
                for (uint32_t r = 0; r < R; ++r) A[m][i * R + r] /= lam[r];
            gram_f64(A[m], ndims[m], (int)R, (int)R, G[m]);
        }
        /* fit (ktensor.c:102-257) with full Grams */
        double normK = 0.0;
        for (uint32_t p = 0; p < R; ++p)
            for (uint32_t q = 0; q < R; ++q) {
                double h = 1.0;
                for (uint32_t m = 0; m < nmodes; ++m) h *= G[m][p * R + q];
                normK += h * lam[p] * lam[q];
            }
        normK = fabs(normK);
        const uint32_t last = nmodes - 1;
        double inner = 0.0;
        for (uint32_t r = 0; r < R; ++r) {
            double acc = 0.0;
            for (uint64_t i = 0; i < ndims[last]; ++i) acc += A[last][i * R + r] * M[i * R + r];
            inner += acc * lam[r];
        }
        double res = normX2 + normK - 2.0 * inner;
        if (res > 0.0) res = sqrt(res);
        const double fit = 1.0 - res / sqrt(normX2);
        fits[it] = fit;
        done = it + 1;
        if (it > 0 && fabs(fit - oldfit) < tol) break;
        oldfit = fit;
    }
    /* GetFinalLambda */
    for (uint32_t m = 0; m < nmodes; ++m) {
        for (uint32_t r = 0; r < R; ++r) {
            double s = 0.0;
            for (uint64_t i = 0; i < ndims[m]; ++i) s += A[m][i * R + r] * A[m][i * R + r];
            s = sqrt(s);
            lam[r] *= s;
            for (uint64_t i = 0; i < ndims[m]; ++i) A[m][i * R + r] /= s;
        }
    }
    for (uint32_t m = 0; m < nmodes; ++m)
        for (uint64_t i = 0; i < ndims[m]; ++i)
            for (uint32_t r = 0; r < R; ++r) factors[m][i * stride + r] = (float)A[m][i * R + r];
    for (uint32_t r = 0; r < R; ++r) lambda_out[r] = (float)lam[r];
    *iters_done = done;
    for (uint32_t m = 0; m < nmodes; ++m) {
        free(A[m]);
        free(G[m]);
    }
    free(M);
    free(H);
    free(lam);
    free(sc);
    return 0;
}

/* The corrected fit of a Kruskal model against the tensor, in FP64, with
 * <X,K> summed exactly over the nonzeros. */
double orc_fit_exact(uint32_t nmodes, const uint32_t *ndims, uint64_t nnz, const uint32_t *const *inds,
                     const float *vals, uint32_t R, const float *const *factors, uint32_t stride, const float *lambda) {
    double normX2 = 0.0, inner = 0.0, normK = 0.0;
    for (uint64_t x = 0; x < nnz; ++x) {
        normX2 += (double)vals[x] * vals[x];
        double s = 0.0;
        for (uint32_t r = 0; r < R; ++r) {
            double p = lambda[r];
            for (uint32_t m = 0; m < nmodes; ++m) p *= factors[m][(size_t)inds[m][x] * stride + r];
            s += p;
        }
        inner += vals[x] * s;
    }
    double *G = (double *)calloc((size_t)R * R, sizeof(double));
    for (uint32_t p = 0; p < R * R; ++p) G[p] = 1.0;
    for (uint32_t m = 0; m < nmodes; ++m)
        for (uint32_t p = 0; p < R; ++p)
            for (uint32_t q = 0; q < R; ++q) {
                double g = 0.0;
                for (uint64_t i = 0; i < ndims[m]; ++i)
                    g += (double)factors[m][i * stride + p] * factors[m][i * stride + q];
                G[p * R + q] *= g;
            }
    for (uint32_t p = 0; p < R; ++p)
        for (uint32_t q = 0; q < R; ++q) normK += G[p * R + q] * lambda[p] * lambda[q];
    free(G);
    normK = fabs(normK);
    double res = normX2 + normK - 2.0 * inner;
    if (res > 0.0) res = sqrt(res);
    return 1.0 - res / sqrt(normX2);
}

/* load.c:31-84 then collect.c:29-49: the reference's fscanf reader (stops at
 * the first token that does not convert; an index below start_index is an
 * error, -1) and its zero removal by moving the last nonzero in.  inds[m]
 * and vals hold `cap` entries. */
int orc_load_tns(const char *path, uint32_t start_index, uint32_t *nmodes_out, uint32_t *ndims_out, uint64_t cap,
                 uint32_t *const *inds, float *vals, uint64_t *nnz_out) {
    FILE *fp = fopen(path, "r");
    if (!fp) return -2;
    uint32_t N = 0;
    if (fscanf(fp, "%u", &N) != 1 || N < 1 || N > ORC_MAX_MODES) {
        fclose(fp);
        return -3;
    }
    for (uint32_t m = 0; m < N; ++m)
        if (fscanf(fp, "%u", &ndims_out[m]) != 1) {
            fclose(fp);
            return -3;
        }
    *nmodes_out = N;
    uint64_t nnz = 0;
    int stop = 0, rc = 0;
    while (!stop) {
        uint32_t idx[ORC_MAX_MODES];
        for (uint32_t m = 0; m < N; ++m) {
            if (fscanf(fp, "%u", &idx[m]) != 1) {
                stop = 1;
                break;
            }
            if (idx[m] < start_index) {
                rc = -1;
                stop = 1;
                break;
            }
        }
        if (stop) break;
        double v;
        if (fscanf(fp, "%lf", &v) != 1) break;
        if (nnz < cap) {
            for (uint32_t m = 0; m < N; ++m) inds[m][nnz] = idx[m] - start_index;
            vals[nnz] = (float)v;
        }
        ++nnz;
    }
    fclose(fp);
    if (nnz > cap) return -4;
    uint64_t i = 0;
    while (i < nnz) {
        if (vals[i] == 0) {
            for (uint32_t m = 0; m < N; ++m) inds[m][i] = inds[m][nnz - 1];
            vals[i] = vals[nnz - 1];
            --nnz;
        } else {
            ++i;
        }
    }
    *nnz_out = nnz;
    return rc;
}

/* setinds.c:33-71 and mmul.c:37-97 on a tensor already sorted at `mode`
 * (mode last): fiber f starts where a coordinate other than `mode` differs
 * from the fiber's first nonzero; Y[f, k] accumulates v * U[i_mode, k] in
 * nonzero order.  fib[m] receive the fiber coordinates (m != mode).
 * Returns the number of fibers. */
uint64_t orc_ttm(uint32_t N, uint64_t nnz, const uint32_t *const *inds, const float *vals, uint32_t mode,
                 const float *U, uint32_t ustride, uint32_t ncols, uint32_t ystride, uint32_t *const *fib, float *Y) {
    uint64_t nf = 0, head = nnz;
    for (uint64_t i = 0; i < nnz; ++i) {
        int diff = head == nnz;
        for (uint32_t m = 0; m < N && !diff; ++m)
            if (m != mode && inds[m][i] != inds[m][head]) diff = 1;
        if (diff) {
            for (uint32_t m = 0; m < N; ++m)
                if (m != mode) fib[m][nf] = inds[m][i];
            for (uint32_t k = 0; k < ystride; ++k) Y[nf * ystride + k] = 0.f;
            head = i;
            ++nf;
        }
        const uint32_t r = inds[mode][i];
        float *y = Y + (nf - 1) * ystride;
        for (uint32_t k = 0; k < ncols; ++k) y[k] += vals[i] * U[(size_t)r * ustride + k];
    }
    return nf;
}
