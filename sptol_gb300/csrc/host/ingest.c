/*
 * Text tensor loading (sptLoadSparseTensor, src/sptensor/load.c:31-84) with
 * the body parsed on the GPU (csrc/cuda/ingest.cu).
 *
 * Format, as the reference reads it with fscanf: nmodes, then nmodes sizes,
 * then per nonzero nmodes 1-based (start_index-based) indices and a value;
 * whitespace of any kind separates tokens.  Reading stops at the first token
 * that does not parse (the incomplete nonzero is dropped); an index below
 * start_index is an error.  The values are read as double and stored as
 * float; finally zero values are removed by moving the last nonzero into
 * their place (collect.c:29-49), so the result equals the reference's.
 *
 * The file is read in one pass into host memory; the body is copied to the
 * device in chunks of at most 256 MiB (SPTGB_INGEST_CHUNK bytes when set)
 * that end at whitespace.  Value tokens
 * the device fast path does not handle (more than 19 significant digits,
 * exponents beyond +-22, hex, inf, nan, trailing bytes) are parsed on the host
 * with strtod, which implements fscanf's "%lf" conversion.
 *
 * sptgbLoadSparseTensorMerged (extension) additionally sorts the nonzeros
 * lexicographically on the device and sums duplicate coordinates in file
 * order, then drops zero sums (order kept).
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "devtensor.h"

#define CHUNK (256ull << 20)
#define SLOW_CAP0 (4ull << 20)

static int host_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

/* fscanf("%u"): skip whitespace, optional sign, decimal digits. */
static int header_u32(const char *b, size_t len, size_t *pos, uint32_t *out) {
    size_t p = *pos;
    while (p < len && host_space(b[p])) ++p;
    int neg = 0;
    if (p < len && (b[p] == '+' || b[p] == '-')) neg = b[p++] == '-';
    if (p >= len || !isdigit((unsigned char)b[p])) return -1;
    uint64_t v = 0;
    while (p < len && isdigit((unsigned char)b[p])) v = v * 10 + (uint64_t)(b[p++] - '0');
    *out = (uint32_t)(neg ? -(int64_t)v : (int64_t)v);
    *pos = p;
    return 0;
}

static int read_all(FILE *fp, char **out, size_t *len) {
    size_t cap = 1 << 20, n = 0;
    char *b = (char *)malloc(cap + 1);
    if (!b) return SPTERR_OS_ERROR;
    for (;;) {
        if (n == cap) {
            cap *= 2;
            char *nb = (char *)realloc(b, cap + 1);
            if (!nb) {
                free(b);
                return SPTERR_OS_ERROR;
            }
            b = nb;
        }
        const size_t got = fread(b + n, 1, cap - n, fp);
        n += got;
        if (got == 0) break;
    }
    b[n] = 0;
    *out = b;
    *len = n;
    return 0;
}

/* collect.c:29-49 */
static void collect_zeros(sptSparseTensor *t) {
    uint64_t i = 0, nnz = t->nnz;
    while (i < nnz) {
        if (t->values.data[i] == 0) {
            for (sptIndex m = 0; m < t->nmodes; ++m) t->inds[m].data[i] = t->inds[m].data[nnz - 1];
            t->values.data[i] = t->values.data[nnz - 1];
            --nnz;
        } else {
            ++i;
        }
    }
    t->nnz = nnz;
    for (sptIndex m = 0; m < t->nmodes; ++m) t->inds[m].len = nnz;
    t->values.len = nnz;
}

#define CU(expr)                                                          \
    do {                                                                  \
        cudaError_t _c = (expr);                                          \
        if (_c != cudaSuccess) {                                          \
            r = sptgb_cuda_fail(_c, module, __FILE__, __LINE__);          \
            goto out;                                                     \
        }                                                                 \
    } while (0)
#define HO(expr)                                                          \
    do {                                                                  \
        int _e = (expr);                                                  \
        if (_e) {                                                         \
            r = _e;                                                       \
            goto out;                                                     \
        }                                                                 \
    } while (0)

static int load_impl(sptSparseTensor *tsr, sptIndex start_index, FILE *fp, int merge) {
    const char *module = "SpTns Load";
    char *buf = NULL;
    size_t len = 0;
    int r = read_all(fp, &buf, &len);
    if (r) {
        spt_ComplainError(module, r, __FILE__, __LINE__, "read failed");
        return r;
    }
    size_t pos = 0;
    uint32_t N = 0;
    sptIndex ndims[SPTGB_MAX_MODES];
    if (header_u32(buf, len, &pos, &N) || N < 1 || N > SPTGB_MAX_MODES) {
        free(buf);
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "bad header (order 1..8)");
        return SPTERR_VALUE_ERROR;
    }
    for (uint32_t m = 0; m < N; ++m)
        if (header_u32(buf, len, &pos, &ndims[m])) {
            free(buf);
            spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__, "bad header");
            return SPTERR_VALUE_ERROR;
        }
    const char *body = buf + pos;
    const uint64_t L = len - pos;
    r = sptgb_ctx();
    if (r) {
        free(buf);
        return r;
    }
    const cudaStream_t s = sptgb_stream();
    sptgb_lock();
    uint64_t records = 0, nslow = 0, slow_cap = SLOW_CAP0;
    uint64_t *hslow = NULL;
    float *hvals = NULL;
    const uint64_t max_rec = (L / 2 + 2) / (N + 1) + 1;
    sptgb_ingest_out o;
    memset(&o, 0, sizeof o);
    o.nmodes = N;
    o.start_index = start_index;
    o.max_records = max_rec;
    for (uint32_t m = 0; m < N; ++m) {
        HO(sptgb_dbuf_reserve(&g_ws.inds[m], max_rec * 4));
        o.inds[m] = (uint32_t *)g_ws.inds[m].ptr;
    }
    HO(sptgb_dbuf_reserve(&g_ws.vals, max_rec * 4));
    o.vals = (float *)g_ws.vals.ptr;
    uint64_t chunk = CHUNK;
    const char *ce = getenv("SPTGB_INGEST_CHUNK");   /* bytes per device chunk (tests force small ones) */
    if (ce && atoll(ce) >= 64) chunk = (uint64_t)atoll(ce);
    const uint64_t cb = L < chunk ? (L ? L : 1) : chunk;
    HO(sptgb_dbuf_reserve(&g_ws.misc[0], cb + 16));
    HO(sptgb_dbuf_reserve(&g_ws.misc[1], (2 * cb + 2) * 4));
    HO(sptgb_dbuf_reserve(&g_ws.misc[2], (cb / 2 + 2) * 8));
    HO(sptgb_dbuf_reserve(&g_ws.misc[3], sptgb_scan_tmp_bytes(cb)));
    uint32_t *flags = (uint32_t *)g_ws.misc[1].ptr, *tpos = flags + cb, *dntok = tpos + cb + 1;
    uint64_t *starts = (uint64_t *)g_ws.misc[2].ptr;
    for (int attempt = 0; attempt < 2; ++attempt) {
        HO(sptgb_dbuf_reserve(&g_ws.misc[4], (4 + 2 * slow_cap) * 8));
        uint64_t *cnt = (uint64_t *)g_ws.misc[4].ptr;
        o.first_bad = cnt;
        o.first_below = cnt + 1;
        o.nslow = cnt + 2;
        o.slow_cap = slow_cap;
        o.slow_rec = cnt + 4;
        o.slow_off = cnt + 4 + slow_cap;
        CU(cudaMemsetAsync(cnt, 0xff, 16, s));
        CU(cudaMemsetAsync(cnt + 2, 0, 16, s));
        uint64_t off = 0, base_tok = 0;
        while (off < L) {
            uint64_t end = off + cb < L ? off + cb : L;
            if (end < L) {   /* end the chunk at whitespace */
                uint64_t e = end;
                while (e > off && !host_space(body[e - 1])) --e;
                if (e == off) {
                    r = SPTERR_VALUE_ERROR;
                    spt_ComplainError(module, r, __FILE__, __LINE__, "token longer than a chunk");
                    goto out;
                }
                end = e;
            }
            const uint64_t n = end - off;
            CU(cudaMemcpyAsync(g_ws.misc[0].ptr, body + off, n, cudaMemcpyHostToDevice, s));
            CU(sptgb_ingest_token_starts(g_ws.misc[0].ptr, n, flags, tpos, dntok, g_ws.misc[3].ptr, starts, s));
            uint32_t ntok = 0;
            CU(cudaMemcpyAsync(&ntok, dntok, 4, cudaMemcpyDeviceToHost, s));
            CU(cudaStreamSynchronize(s));
            o.base_off = off;
            CU(sptgb_ingest_parse(g_ws.misc[0].ptr, n, starts, ntok, base_tok, &o, s));
            base_tok += ntok;
            off = end;
        }
        uint64_t h[3];
        CU(cudaMemcpyAsync(h, cnt, 24, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        nslow = h[2];
        if (nslow > slow_cap && attempt == 0) {
            slow_cap = nslow;
            continue;
        }
        /* the first token that stops reading, in token order */
        uint64_t stop = base_tok - base_tok % (N + 1);   /* an incomplete last nonzero */
        if (h[0] < stop) stop = h[0];
        records = stop / (N + 1);
        hslow = (uint64_t *)malloc((nslow ? nslow : 1) * 16);
        if (!hslow) HO(SPTERR_OS_ERROR);
        if (nslow) {
            CU(cudaMemcpyAsync(hslow, cnt + 4, nslow * 8, cudaMemcpyDeviceToHost, s));
            CU(cudaMemcpyAsync(hslow + nslow, cnt + 4 + slow_cap, nslow * 8, cudaMemcpyDeviceToHost, s));
            CU(cudaStreamSynchronize(s));
        }
        /* host conversion of the remaining values, as fscanf("%lf") */
        for (uint64_t k = 0; k < nslow; ++k) {
            const uint64_t rec = hslow[k];
            const char *tok = body + hslow[nslow + k];
            char *endp = NULL;
            (void)strtod(tok, &endp);
            const char *tend = tok;
            while (tend < body + L && !host_space(*tend)) ++tend;
            if (endp == tok) {
                if (rec * (N + 1) + N < stop) stop = rec * (N + 1) + N;
            } else if (endp < tend) {
                if ((rec + 1) * (N + 1) < stop) stop = (rec + 1) * (N + 1);
            }
        }
        records = stop / (N + 1);
        if (h[1] < stop) {
            r = SPTERR_VALUE_ERROR;
            spt_ComplainError(module, r, __FILE__, __LINE__, "index < start_index");
            goto out;
        }
        break;
    }
    hvals = (float *)malloc((records ? records : 1) * sizeof(float));
    if (!hvals) HO(SPTERR_OS_ERROR);
    if (records) CU(cudaMemcpyAsync(hvals, o.vals, records * 4, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    for (uint64_t k = 0; k < nslow; ++k)
        if (hslow[k] < records) hvals[hslow[k]] = (float)strtod(body + hslow[nslow + k], NULL);

    uint64_t n_out = records;
    if (merge && records) {
        /* lexicographic device sort, duplicates summed in file order */
        CU(cudaMemcpyAsync(o.vals, hvals, records * 4, cudaMemcpyHostToDevice, s));
        sptIndex order[SPTGB_MAX_MODES];
        for (uint32_t m = 0; m < N; ++m) order[m] = m;
        sptgb_sortpass passes[SPTGB_MAX_MODES];
        const int np = sptgb_lex_passes(ndims, order, (int)N, passes);
        uint32_t *perm = NULL, *din[SPTGB_MAX_MODES], *dsrt[SPTGB_MAX_MODES];
        for (uint32_t m = 0; m < N; ++m) {
            din[m] = o.inds[m];
            HO(sptgb_dbuf_reserve(&g_ws.sinds[m], records * 4));
            dsrt[m] = (uint32_t *)g_ws.sinds[m].ptr;
        }
        HO(sptgb_dbuf_reserve(&g_ws.svals, records * 4));
        HO(sptgb_sort_perm(din, (int)N, records, passes, np, &perm, s));
        HO(sptgb_gather_tensor(din, o.vals, dsrt, (float *)g_ws.svals.ptr, (int)N, perm, records, s));
        HO(sptgb_dbuf_reserve(&g_ws.misc[1], (2 * records + 2) * 4));
        HO(sptgb_dbuf_reserve(&g_ws.misc[2], (records + 1) * 8));
        HO(sptgb_dbuf_reserve(&g_ws.misc[3], sptgb_scan_tmp_bytes(records)));
        uint32_t *gf = (uint32_t *)g_ws.misc[1].ptr, *gp = gf + records, *gn = gp + records + 1;
        uint64_t *gs = (uint64_t *)g_ws.misc[2].ptr;
        CU(sptgb_mark_groups((const uint32_t *const *)dsrt, (int)N, 0, records, gf, s));
        CU(sptgb_exclusive_scan_u32(gf, gp, records, gn, g_ws.misc[3].ptr, s));
        CU(sptgb_compact_starts(gf, gp, records, gs, s));
        uint32_t ng = 0;
        CU(cudaMemcpyAsync(&ng, gn, 4, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        CU(sptgb_segment_sums(gs, ng, records, (const float *)g_ws.svals.ptr, o.vals, s));
        for (uint32_t m = 0; m < N; ++m) CU(sptgb_compact_u32(gf, gp, dsrt[m], records, o.inds[m], s));
        n_out = ng;
        CU(cudaMemcpyAsync(hvals, o.vals, n_out * 4, cudaMemcpyDeviceToHost, s));
    }
    HO(sptNewSparseTensor(tsr, N, ndims));
    for (uint32_t m = 0; m < N; ++m) {
        HO(sptResizeIndexVector(&tsr->inds[m], n_out));
        if (n_out) CU(cudaMemcpyAsync(tsr->inds[m].data, o.inds[m], n_out * 4, cudaMemcpyDeviceToHost, s));
    }
    HO(sptResizeValueVector(&tsr->values, n_out));
    CU(cudaStreamSynchronize(s));
    if (n_out) memcpy(tsr->values.data, hvals, n_out * 4);
    tsr->nnz = n_out;
    if (!merge) {
        collect_zeros(tsr);
    } else {
        uint64_t w = 0;
        for (uint64_t i = 0; i < n_out; ++i)
            if (tsr->values.data[i] != 0) {
                for (uint32_t m = 0; m < N; ++m) tsr->inds[m].data[w] = tsr->inds[m].data[i];
                tsr->values.data[w++] = tsr->values.data[i];
            }
        tsr->nnz = w;
        for (uint32_t m = 0; m < N; ++m) tsr->inds[m].len = w;
        tsr->values.len = w;
        for (uint32_t m = 0; m < N; ++m) tsr->sortorder[m] = m;
    }
out:
    sptgb_unlock();
    free(hslow);
    free(hvals);
    free(buf);
    return r;
}

int sptLoadSparseTensor(sptSparseTensor *tsr, sptIndex start_index, FILE *fp) {
    return load_impl(tsr, start_index, fp, 0);
}

int sptgbLoadSparseTensorMerged(sptSparseTensor *tsr, sptIndex start_index, FILE *fp) {
    return load_impl(tsr, start_index, fp, 1);
}
