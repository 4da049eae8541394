/*
 * Host containers of the drop-in API: dynamic vectors, COO / HiCOO tensors,
 * dense matrices and Kruskal tensors.  Allocation, growth and ownership
 * follow the reference (src/vector/vector.c, src/sptensor/sptensor.c:30-107,
 * src/sptensor/hicoo/hicoo.c:29-172, src/matrix/matrix.c:37-112,
 * src/ktensor/ktensor.c:33-89) so that objects built by either library can be
 * freed by the other.  These are plain host bookkeeping; every numerical
 * operation on them lives in the GPU paths.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <omp.h>
#include <string.h>
#include "../sptgb_internal.h"
#include "../../../include/sptgb.h"

uint64_t sptgb_seed_next(void);

#define CHECK_OS(cond, module) do { if (cond) { \
        spt_ComplainError(module, SPTERR_OS_ERROR + errno, __FILE__, __LINE__, strerror(errno)); \
        return SPTERR_OS_ERROR + errno; } } while (0)

/* One definition per element type, same rules as vector.c: New clamps the
 * capacity to >= 2 and zero-fills; Append grows by half; Resize sets
 * cap = max(size, 2). */
#define DEFINE_VECTOR(VT, ET, NAME)                                                   \
    int sptNew##NAME(VT *vec, uint64_t len, uint64_t cap) {                          \
        if (cap < len) cap = len;                                                     \
        if (cap < 2) cap = 2;                                                         \
        vec->len = len;                                                               \
        vec->cap = cap;                                                               \
        vec->data = malloc(cap * sizeof *vec->data);                                 \
        CHECK_OS(!vec->data, #NAME " New");                                           \
        memset(vec->data, 0, cap * sizeof *vec->data);                                \
        return 0;                                                                     \
    }                                                                                 \
    int sptAppend##NAME(VT *vec, ET const value) {                                   \
        if (vec->cap <= vec->len) {                                                   \
            sptNnzIndex newcap = vec->cap + vec->cap / 2;                             \
            if (newcap < 2) newcap = 2;                                               \
            ET *nd = realloc(vec->data, newcap * sizeof *vec->data);                  \
            CHECK_OS(!nd, #NAME " Append");                                           \
            vec->cap = newcap;                                                        \
            vec->data = nd;                                                           \
        }                                                                             \
        vec->data[vec->len++] = value;                                                \
        return 0;                                                                     \
    }                                                                                 \
    int sptResize##NAME(VT *vec, sptNnzIndex const size) {                           \
        sptNnzIndex newcap = size < 2 ? 2 : size;                                     \
        if (newcap != vec->cap) {                                                     \
            ET *nd = realloc(vec->data, newcap * sizeof *vec->data);                  \
            CHECK_OS(!nd, #NAME " Resize");                                           \
            vec->cap = newcap;                                                        \
            vec->data = nd;                                                           \
        }                                                                             \
        vec->len = size;                                                              \
        return 0;                                                                     \
    }                                                                                 \
    void sptFree##NAME(VT *vec) {                                                     \
        vec->len = 0;                                                                 \
        vec->cap = 0;                                                                 \
        free(vec->data);                                                              \
        vec->data = NULL;                                                             \
    }

DEFINE_VECTOR(sptValueVector, sptValue, ValueVector)
DEFINE_VECTOR(sptIndexVector, sptIndex, IndexVector)
DEFINE_VECTOR(sptElementIndexVector, sptElementIndex, ElementIndexVector)
DEFINE_VECTOR(sptBlockIndexVector, sptBlockIndex, BlockIndexVector)
DEFINE_VECTOR(sptNnzIndexVector, sptNnzIndex, NnzIndexVector)

int sptConstantValueVector(sptValueVector *const vec, sptValue const val) {
    for (sptNnzIndex i = 0; i < vec->len; ++i) vec->data[i] = val;
    return 0;
}

int sptConstantIndexVector(sptIndexVector *const vec, sptIndex const num) {
    for (sptNnzIndex i = 0; i < vec->len; ++i) vec->data[i] = num;
    return 0;
}

int sptCopyValueVector(sptValueVector *dest, const sptValueVector *src, int const nt) {
    (void)nt;
    int r = sptNewValueVector(dest, src->len, src->len);
    if (r) return r;
    memcpy(dest->data, src->data, src->len * sizeof *src->data);
    return 0;
}

int sptCopyIndexVector(sptIndexVector *dest, const sptIndexVector *src, int const nt) {
    (void)nt;
    int r = sptNewIndexVector(dest, src->len, src->len);
    if (r) return r;
    memcpy(dest->data, src->data, src->len * sizeof *src->data);
    return 0;
}

sptNnzIndex sptMaxNnzIndexArray(sptNnzIndex const *indices, sptNnzIndex const size) {
    sptNnzIndex m = indices[0];
    for (sptNnzIndex i = 1; i < size; ++i)
        if (indices[i] > m) m = indices[i];
    return m;
}

sptIndex sptMaxIndexArray(sptIndex const *indices, sptNnzIndex const size) {
    sptIndex m = indices[0];
    for (sptNnzIndex i = 1; i < size; ++i)
        if (indices[i] > m) m = indices[i];
    return m;
}

/* Increasing sort by value.  The same Hoare-partition quicksort as
 * src/vector/array.c:66-117 so that ties between equal mode sizes resolve as
 * in the reference (sptGetBestModeOrder depends on it). */
static void pair_qsort(sptKeyValuePair *a, sptIndex l, sptIndex r) {
    if (r - l < 2) return;
    sptIndex i, j, p = (l + r) / 2;
    for (i = l, j = r - 1;; ++i, --j) {
        while (a[i].value < a[p].value) ++i;
        while (a[p].value < a[j].value) --j;
        if (i >= j) break;
        sptKeyValuePair t = a[i];
        a[i] = a[j];
        a[j] = t;
        if (i == p) p = j;
        else if (j == p) p = i;
    }
    pair_qsort(a, l, i);
    pair_qsort(a, i, r);
}

void sptPairArraySort(sptKeyValuePair *kvarray, sptIndex const length) { pair_qsort(kvarray, 0, length); }

/* src/sptensor/sort.c:193-227 */
void sptGetBestModeOrder(sptIndex *mode_order, sptIndex const mode, sptIndex const *ndims, sptIndex const nmodes) {
    sptKeyValuePair *kv = malloc(nmodes * sizeof *kv);
    for (sptIndex m = 0; m < nmodes; ++m) {
        kv[m].key = m;
        kv[m].value = ndims[m];
    }
    sptPairArraySort(kv, nmodes);
    sptIndex loc = 0;
    for (sptIndex m = 0; m < nmodes; ++m) {
        mode_order[m] = kv[m].key;
        if (kv[m].key == mode) loc = m;
    }
    if (loc != 0) {
        for (sptIndex m = loc; m >= 1; --m) mode_order[m] = mode_order[m - 1];
        mode_order[0] = mode;
    }
    free(kv);
}

/* src/sptensor/sort.c:239-274 (including its shift of the trailing entries) */
void sptGetWorstModeOrder(sptIndex *mode_order, sptIndex const mode, sptIndex const *ndims, sptIndex const nmodes) {
    sptKeyValuePair *kv = malloc(nmodes * sizeof *kv);
    for (sptIndex m = 0; m < nmodes; ++m) {
        kv[m].key = m;
        kv[m].value = ndims[m];
    }
    sptPairArraySort(kv, nmodes);
    sptIndex loc = 0;
    for (sptIndex m = 0; m < nmodes; ++m) mode_order[m] = kv[nmodes - 1 - m].key;
    for (sptIndex m = 0; m < nmodes; ++m)
        if (mode_order[m] == mode) loc = m;
    if (loc != nmodes - 1) {
        for (sptIndex m = loc; m + 1 < nmodes; ++m) mode_order[m] = mode_order[m + 1];
        mode_order[nmodes - 1] = mode;
    }
    free(kv);
}

/* ------------------------------------------------------ COO tensor -- */
int sptNewSparseTensor(sptSparseTensor *tsr, sptIndex nmodes, const sptIndex ndims[]) {
    tsr->nmodes = nmodes;
    tsr->sortorder = malloc(nmodes * sizeof tsr->sortorder[0]);
    CHECK_OS(!tsr->sortorder, "SpTns New");
    for (sptIndex i = 0; i < nmodes; ++i) tsr->sortorder[i] = i;
    tsr->ndims = malloc(nmodes * sizeof *tsr->ndims);
    CHECK_OS(!tsr->ndims, "SpTns New");
    memcpy(tsr->ndims, ndims, nmodes * sizeof *tsr->ndims);
    tsr->nnz = 0;
    tsr->inds = malloc(nmodes * sizeof *tsr->inds);
    CHECK_OS(!tsr->inds, "SpTns New");
    for (sptIndex i = 0; i < nmodes; ++i) {
        int r = sptNewIndexVector(&tsr->inds[i], 0, 0);
        if (r) return r;
    }
    return sptNewValueVector(&tsr->values, 0, 0);
}

/* status.c:24-34: the geometric-mean density nnz^(1/N) / ndims[m], multiplied over the modes. */
double sptSparseTensorDensity(sptSparseTensor const *const tsr) {
    const double root = pow((double)tsr->nnz, 1. / (double)tsr->nmodes);
    double density = 1.0;
    for (sptIndex m = 0; m < tsr->nmodes; ++m) density *= root / (double)tsr->ndims[m];
    return density;
}

/* status.c:38-58: the same lines, in the same format. */
void sptSparseTensorStatus(sptSparseTensor *tsr, FILE *fp) {
    fprintf(fp, "COO Sparse Tensor information (use sptIndex, sptValue))---------\n");
    fprintf(fp, "DIMS=%" PARTI_PRI_INDEX, tsr->ndims[0]);
    for (sptIndex m = 1; m < tsr->nmodes; ++m) fprintf(fp, "x%" PARTI_PRI_INDEX, tsr->ndims[m]);
    fprintf(fp, " NNZ=%" PARTI_PRI_NNZ_INDEX, tsr->nnz);
    fprintf(fp, " DENSITY=%e\n", sptSparseTensorDensity(tsr));
    fprintf(fp, "Average slice length (c): ");
    for (sptIndex m = 0; m + 1 < tsr->nmodes; ++m) fprintf(fp, "%.2lf , ", (double)tsr->nnz / tsr->ndims[m]);
    fprintf(fp, "%.2lf\n", (double)tsr->nnz / tsr->ndims[tsr->nmodes - 1]);
    char *b = sptBytesString(tsr->nnz * (sizeof(sptIndex) * tsr->nmodes + sizeof(sptValue)));
    fprintf(fp, "COO-STORAGE=%s\n", b ? b : "?");
    fprintf(fp, "\n");
    free(b);
}

static int cmp_nnz(const void *a, const void *b) {
    const sptNnzIndex x = *(const sptNnzIndex *)a, y = *(const sptNnzIndex *)b;
    return x < y ? -1 : x > y;
}

/* hicoo/status.c:28-118: the same lines, in the same format.  Block sizes
 * are bptr differences; the median is element (nb + 1) / 2 - 1 of the sorted
 * sizes, the geometric mean the product over blocks, in block order, of
 * (nnzb / sb)^(1 / nb).  A tensor without blocks prints zero statistics. */
void sptSparseTensorStatusHiCOO(sptSparseTensorHiCOO *hitsr, FILE *fp) {
    const sptIndex N = hitsr->nmodes;
    fprintf(fp, "HiCOO Sparse Tensor information ---------\n");
    fprintf(fp, "DIMS=%" PARTI_PRI_INDEX, hitsr->ndims[0]);
    for (sptIndex m = 1; m < N; ++m) fprintf(fp, "x%" PARTI_PRI_INDEX, hitsr->ndims[m]);
    fprintf(fp, " NNZ=%" PARTI_PRI_NNZ_INDEX "\n", hitsr->nnz);
    const sptIndex sb = (sptIndex)1 << hitsr->sb_bits, sk = (sptIndex)1 << hitsr->sk_bits;
    fprintf(fp, "sb=%" PARTI_PRI_INDEX " sk=%" PARTI_PRI_INDEX "\n", sb, sk);
    const sptNnzIndex nb = hitsr->bptr.len ? hitsr->bptr.len - 1 : 0;
    fprintf(fp, "nb=%" PARTI_PRI_NNZ_INDEX " nk=%" PARTI_PRI_NNZ_INDEX " nc=%" PARTI_PRI_NNZ_INDEX "\n", nb,
            hitsr->kptr.len ? hitsr->kptr.len - 1 : 0, hitsr->cptr.len ? hitsr->cptr.len - 1 : 0);
    sptNnzIndex bytes = hitsr->nnz * (sizeof(sptValue) + N * sizeof(sptElementIndex));
    bytes += (sptNnzIndex)hitsr->binds[0].len * N * sizeof(sptBlockIndex);
    bytes += (hitsr->bptr.len + hitsr->kptr.len + hitsr->cptr.len) * sizeof(sptNnzIndex);
    for (sptIndex m = 0; m < N; ++m) {
        const sptIndex kdim = (hitsr->ndims[m] + sk - 1) / sk;
        if (hitsr->kschr && hitsr->kschr[m])   /* absent before a conversion filled them */
            for (sptIndex i = 0; i < kdim; ++i) bytes += (sptNnzIndex)hitsr->kschr[m][i].len * sizeof(sptIndex);
        bytes += kdim * sizeof(sptIndexVector *);
    }
    bytes += N * sizeof(sptIndexVector **) + N * sizeof(sptIndex);
    char *b = sptBytesString(bytes);
    fprintf(fp, "HiCOO-STORAGE=%s\n", b ? b : "?");
    free(b);
    fprintf(fp, "SCHEDULE INFO [KERNEL]: \n");
    for (sptIndex m = 0; m < N; ++m)
        fprintf(fp, "SCHEDULE MODE %" PARTI_PRI_INDEX " : %" PARTI_PRI_INDEX " x %" PARTI_PRI_INDEX "\n", m,
                (hitsr->ndims[m] + sk - 1) / sk, hitsr->nkiters ? hitsr->nkiters[m] : 0);
    sptNnzIndex mx = 0, mn = 0, sum = 0, med = 0;
    double geo = 1.0;
    fprintf(fp, "block nnzs:\n");
    if (nb) {
        sptNnzIndex *sz = (sptNnzIndex *)malloc(nb * sizeof *sz);
        mx = mn = hitsr->bptr.data[1] - hitsr->bptr.data[0];
        for (sptNnzIndex i = 0; i < nb; ++i) {
            const sptNnzIndex n = hitsr->bptr.data[i + 1] - hitsr->bptr.data[i];
            if (n > mx) mx = n;
            if (n < mn) mn = n;
            sum += n;
            geo *= pow((double)n / sb, 1.0 / nb);
            if (sz) sz[i] = n;
        }
        if (sz) {
            qsort(sz, nb, sizeof *sz, cmp_nnz);
            med = sz[(nb + 1) / 2 - 1];
            free(sz);
        }
    }
    const sptNnzIndex aver = nb ? sum / nb : 0;
    fprintf(fp, "Nnzb: Max=%lu, Min=%lu, Aver=%lu\n", (unsigned long)mx, (unsigned long)mn, (unsigned long)aver);
    fprintf(fp, "cb: Max=%.3lf, Min=%.3lf, Aver=%.3lf\n", (double)mx / sb, (double)mn / sb, (double)aver / sb);
    fprintf(fp, "median cb: %.3lf, geometric mean cb: %.3lf\n", (double)med / sb, geo);
    fprintf(fp, "alpha_b: %lf\n", hitsr->nnz ? (double)nb / hitsr->nnz : 0.0);
    fprintf(fp, "\nParameter configuration --------\n");
    fprintf(fp, "Suggest B (sb) <= %.2lf / R. For cache efficiency\n", (double)L1_SIZE / N / sizeof(sptValue));
    fprintf(fp, "Suggest alpha_b in (0,1], small is better. For tensor storage\n");
    fprintf(fp, "Suggest cb > 1, large is better. For MTTKRP performance\n");
    fprintf(fp, "Suggest num_tasks should in [%d, %d] PAR_DEGREE: [%d, %d]. For parallel efficiency\n",
            PAR_MIN_DEGREE * NUM_CORES, PAR_MAX_DEGREE * NUM_CORES, PAR_MIN_DEGREE, PAR_MAX_DEGREE);
    fprintf(fp, "\n\n");
}

/* sort.c:371-380: for every position z, srand(z + 1), one rand() scaled to a
 * position, and a swap of the two nonzeros (all modes and the value); the C
 * library's rand() makes it the reference's permutation on the same libc. */
void sptGetRandomShuffleElements(sptSparseTensor *tsr) {
    const sptNnzIndex nnz = tsr->nnz;
    for (sptNnzIndex z = 0; z < nnz; ++z) {
        srand((unsigned)(z + 1));
        const sptValue u = (sptValue)rand() / (sptValue)RAND_MAX;
        const sptNnzIndex w = (sptNnzIndex)(u * nnz) % nnz;
        for (sptIndex m = 0; m < tsr->nmodes; ++m) {
            const sptIndex t = tsr->inds[m].data[z];
            tsr->inds[m].data[z] = tsr->inds[m].data[w];
            tsr->inds[m].data[w] = t;
        }
        const sptValue t = tsr->values.data[z];
        tsr->values.data[z] = tsr->values.data[w];
        tsr->values.data[w] = t;
    }
}

int sptCopySparseTensor(sptSparseTensor *dest, const sptSparseTensor *src, int const nt) {
    dest->nmodes = src->nmodes;
    dest->sortorder = malloc(src->nmodes * sizeof src->sortorder[0]);
    CHECK_OS(!dest->sortorder, "SpTns Copy");
    memcpy(dest->sortorder, src->sortorder, src->nmodes * sizeof src->sortorder[0]);
    dest->ndims = malloc(src->nmodes * sizeof *dest->ndims);
    CHECK_OS(!dest->ndims, "SpTns Copy");
    memcpy(dest->ndims, src->ndims, src->nmodes * sizeof *src->ndims);
    dest->nnz = src->nnz;
    dest->inds = malloc(src->nmodes * sizeof *dest->inds);
    CHECK_OS(!dest->inds, "SpTns Copy");
    for (sptIndex i = 0; i < src->nmodes; ++i) {
        int r = sptCopyIndexVector(&dest->inds[i], &src->inds[i], nt);
        if (r) return r;
    }
    return sptCopyValueVector(&dest->values, &src->values, nt);
}

void sptFreeSparseTensor(sptSparseTensor *tsr) {
    for (sptIndex i = 0; i < tsr->nmodes; ++i) sptFreeIndexVector(&tsr->inds[i]);
    free(tsr->sortorder);
    free(tsr->ndims);
    free(tsr->inds);
    sptFreeValueVector(&tsr->values);
    tsr->sortorder = NULL;
    tsr->ndims = NULL;
    tsr->inds = NULL;
    tsr->nmodes = 0;
}

/* ------------------------------------------------------ HiCOO tensor -- */
static sptIndex kernel_ndim(sptIndex ndim, sptElementIndex sk_bits) {
    const uint64_t sk = 1ull << sk_bits;
    return (sptIndex)(((uint64_t)ndim + sk - 1) / sk);
}

int sptNewSparseTensorHiCOO(sptSparseTensorHiCOO *h, const sptIndex nmodes, const sptIndex ndims[],
                            const sptNnzIndex nnz, const sptElementIndex sb_bits, const sptElementIndex sk_bits,
                            const sptElementIndex sc_bits) {
    int r;
    memset(h, 0, sizeof *h);
    h->nmodes = nmodes;
    h->sortorder = malloc(nmodes * sizeof h->sortorder[0]);
    CHECK_OS(!h->sortorder, "HiSpTns New");
    for (sptIndex i = 0; i < nmodes; ++i) h->sortorder[i] = i;
    h->ndims = malloc(nmodes * sizeof *h->ndims);
    CHECK_OS(!h->ndims, "HiSpTns New");
    memcpy(h->ndims, ndims, nmodes * sizeof *h->ndims);
    h->nnz = nnz;
    h->sb_bits = sb_bits;
    h->sk_bits = sk_bits;
    h->sc_bits = sc_bits;
    h->kschr = malloc(nmodes * sizeof *h->kschr);
    h->kschr_balanced = malloc(nmodes * sizeof *h->kschr_balanced);
    h->kschr_balanced_pos = malloc(nmodes * sizeof *h->kschr_balanced_pos);
    CHECK_OS(!h->kschr || !h->kschr_balanced || !h->kschr_balanced_pos, "HiSpTns New");
    for (sptIndex m = 0; m < nmodes; ++m) {
        const sptIndex kn = kernel_ndim(ndims[m], sk_bits);
        h->kschr[m] = malloc((kn ? kn : 1) * sizeof *h->kschr[m]);
        h->kschr_balanced[m] = malloc((kn ? kn : 1) * sizeof *h->kschr_balanced[m]);
        h->kschr_balanced_pos[m] = malloc((kn ? kn : 1) * sizeof *h->kschr_balanced_pos[m]);
        CHECK_OS(!h->kschr[m] || !h->kschr_balanced[m] || !h->kschr_balanced_pos[m], "HiSpTns New");
        for (sptIndex i = 0; i < kn; ++i) {
            if ((r = sptNewIndexVector(&h->kschr[m][i], 0, 0))) return r;
            if ((r = sptNewIndexVector(&h->kschr_balanced[m][i], 0, 0))) return r;
            if ((r = sptNewIndexVector(&h->kschr_balanced_pos[m][i], 0, 0))) return r;
        }
    }
    h->nkiters = malloc(nmodes * sizeof *h->nkiters);
    h->nkpars = malloc(nmodes * sizeof *h->nkpars);
    h->kschr_rest = malloc(nmodes * sizeof *h->kschr_rest);
    CHECK_OS(!h->nkiters || !h->nkpars || !h->kschr_rest, "HiSpTns New");
    for (sptIndex m = 0; m < nmodes; ++m) {
        h->nkiters[m] = 0;
        h->nkpars[m] = 0;
        if ((r = sptNewIndexVector(&h->kschr_rest[m], 0, 0))) return r;
    }
    if ((r = sptNewNnzIndexVector(&h->kptr, 0, 0))) return r;
    if ((r = sptNewNnzIndexVector(&h->cptr, 0, 0))) return r;
    if ((r = sptNewNnzIndexVector(&h->knnzs, 0, 0))) return r;
    if ((r = sptNewNnzIndexVector(&h->bptr, 0, 0))) return r;
    h->binds = malloc(nmodes * sizeof *h->binds);
    h->einds = malloc(nmodes * sizeof *h->einds);
    CHECK_OS(!h->binds || !h->einds, "HiSpTns New");
    for (sptIndex i = 0; i < nmodes; ++i) {
        if ((r = sptNewBlockIndexVector(&h->binds[i], 0, 0))) return r;
        if ((r = sptNewElementIndexVector(&h->einds[i], 0, 0))) return r;
    }
    return sptNewValueVector(&h->values, 0, 0);
}

void sptFreeSparseTensorHiCOO(sptSparseTensorHiCOO *h) {
    const sptIndex nmodes = h->nmodes;
    for (sptIndex m = 0; m < nmodes; ++m) {
        const sptIndex kn = kernel_ndim(h->ndims[m], h->sk_bits);
        for (sptIndex i = 0; i < kn; ++i) {
            sptFreeIndexVector(&h->kschr[m][i]);
            if (h->kschr_balanced) sptFreeIndexVector(&h->kschr_balanced[m][i]);
            if (h->kschr_balanced_pos) sptFreeIndexVector(&h->kschr_balanced_pos[m][i]);
        }
        free(h->kschr[m]);
        if (h->kschr_balanced) free(h->kschr_balanced[m]);
        if (h->kschr_balanced_pos) free(h->kschr_balanced_pos[m]);
        if (h->kschr_rest) sptFreeIndexVector(&h->kschr_rest[m]);
    }
    free(h->kschr);
    free(h->kschr_balanced);
    free(h->kschr_balanced_pos);
    free(h->kschr_rest);
    free(h->nkiters);
    free(h->nkpars);
    sptFreeNnzIndexVector(&h->kptr);
    sptFreeNnzIndexVector(&h->cptr);
    sptFreeNnzIndexVector(&h->knnzs);
    sptFreeNnzIndexVector(&h->bptr);
    for (sptIndex i = 0; i < nmodes; ++i) {
        sptFreeBlockIndexVector(&h->binds[i]);
        sptFreeElementIndexVector(&h->einds[i]);
    }
    free(h->binds);
    free(h->einds);
    sptFreeValueVector(&h->values);
    free(h->sortorder);
    free(h->ndims);
    memset(h, 0, sizeof *h);
}

/* ---------------------------------------------------- dense matrices -- */
int sptNewMatrix(sptMatrix *mtx, sptIndex const nrows, sptIndex const ncols) {
    mtx->nrows = nrows;
    mtx->ncols = ncols;
    mtx->cap = nrows != 0 ? nrows : 1;
    mtx->stride = ((ncols - 1) / 8 + 1) * 8;
    mtx->values = NULL;
    int r = posix_memalign((void **)&mtx->values, 8 * sizeof(sptValue),
                           (size_t)mtx->cap * mtx->stride * sizeof(sptValue));
    if (r != 0 || !mtx->values) {
        errno = r ? r : ENOMEM;
        CHECK_OS(1, "Mtx New");
    }
    return 0;
}

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Values uniform in [-3, 3] as sptRandomValue (src/base.c:43-50), drawn from
 * a seeded SplitMix64 stream instead of rand() seeded with time(NULL). */
int sptRandomizeMatrix(sptMatrix *mtx, sptIndex const nrows, sptIndex const ncols) {
    const uint64_t base = sptgb_seed_next();
    for (sptIndex i = 0; i < nrows; ++i)
        for (sptIndex j = 0; j < ncols; ++j) {
            const uint64_t z = mix64(base + 0x9E3779B97F4A7C15ULL * ((uint64_t)i * ncols + j + 1));
            float v = 3.0f * (float)((z >> 40) * (1.0 / 16777216.0));
            if (z & 1) v = -v;
            mtx->values[(size_t)i * mtx->stride + j] = v;
        }
    return 0;
}

sptValue sptRandomValue(void) {
    const uint64_t z = mix64(sptgb_seed_next());
    float v = 3.0f * (float)((z >> 40) * (1.0 / 16777216.0));
    return (z & 1) ? -v : v;
}

int sptIdentityMatrix(sptMatrix *mtx) {
    for (sptIndex i = 0; i < mtx->nrows; ++i)
        for (sptIndex j = 0; j < mtx->ncols; ++j) mtx->values[(size_t)i * mtx->stride + j] = (i == j) ? 1.f : 0.f;
    return 0;
}

int sptConstantMatrix(sptMatrix *const mtx, sptValue const val) {
    for (sptIndex i = 0; i < mtx->nrows; ++i)
        for (sptIndex j = 0; j < mtx->ncols; ++j) mtx->values[(size_t)i * mtx->stride + j] = val;
    return 0;
}

int sptCopyMatrix(sptMatrix *dest, const sptMatrix *src) {
    int r = sptNewMatrix(dest, src->nrows, src->ncols);
    if (r) return r;
    memcpy(dest->values, src->values, (size_t)dest->cap * dest->stride * sizeof(sptValue));
    return 0;
}

void sptFreeMatrix(sptMatrix *mtx) {
    free(mtx->values);
    mtx->values = NULL;
    mtx->nrows = 0;
    mtx->ncols = 0;
}

/* ------------------------------------------------ rank matrix (u8 cols) --
 * rankmatrix.c:38-133: the same row-major layout with 8-bit column count and
 * stride; padding columns are zeroed here (the reference leaves them
 * uninitialised). */
int sptNewRankMatrix(sptRankMatrix *mtx, sptIndex const nrows, sptElementIndex const ncols) {
    mtx->nrows = nrows;
    mtx->ncols = ncols;
    mtx->cap = nrows != 0 ? nrows : 1;
    mtx->stride = (sptElementIndex)(((ncols - 1) / 8 + 1) * 8);
    mtx->values = NULL;
    int r = posix_memalign((void **)&mtx->values, 8 * sizeof(sptValue),
                           (size_t)mtx->cap * mtx->stride * sizeof(sptValue));
    if (r != 0 || !mtx->values) {
        errno = r ? r : ENOMEM;
        CHECK_OS(1, "RankMtx New");
    }
    memset(mtx->values, 0, (size_t)mtx->cap * mtx->stride * sizeof(sptValue));
    return 0;
}

int sptRandomizeRankMatrix(sptRankMatrix *mtx, sptIndex const nrows, sptElementIndex const ncols) {
    const uint64_t base = sptgb_seed_next();
    for (sptIndex i = 0; i < nrows; ++i)
        for (sptElementIndex j = 0; j < ncols; ++j) {
            const uint64_t z = mix64(base + 0x9E3779B97F4A7C15ULL * ((uint64_t)i * ncols + j + 1));
            float v = 3.0f * (float)((z >> 40) * (1.0 / 16777216.0));
            if (z & 1) v = -v;
            mtx->values[(size_t)i * mtx->stride + j] = v;
        }
    return 0;
}

int sptConstantRankMatrix(sptRankMatrix *mtx, sptValue const val) {
    for (sptIndex i = 0; i < mtx->nrows; ++i)
        for (sptElementIndex j = 0; j < mtx->ncols; ++j) mtx->values[(size_t)i * mtx->stride + j] = val;
    return 0;
}

void sptFreeRankMatrix(sptRankMatrix *mtx) {
    free(mtx->values);
    mtx->values = NULL;
    mtx->nrows = 0;
    mtx->ncols = 0;
    mtx->cap = 0;
    mtx->stride = 0;
}

/* rankktensor.c:33-88 */
int sptNewRankKruskalTensor(sptRankKruskalTensor *k, sptIndex nmodes, const sptIndex ndims[], sptElementIndex rank) {
    k->nmodes = nmodes;
    k->rank = rank;
    k->ndims = malloc(nmodes * sizeof(sptIndex));
    CHECK_OS(!k->ndims, "RankKruskal New");
    for (sptIndex i = 0; i < nmodes; ++i) k->ndims[i] = ndims[i];
    k->lambda = malloc((rank ? rank : 1) * sizeof(sptValue));
    CHECK_OS(!k->lambda, "RankKruskal New");
    k->fit = 0.0;
    k->factors = NULL;
    return 0;
}

void sptFreeRankKruskalTensor(sptRankKruskalTensor *k) {
    k->rank = 0;
    k->fit = 0.0;
    free(k->ndims);
    free(k->lambda);
    if (k->factors) {
        for (sptIndex i = 0; i < k->nmodes; ++i)
            if (k->factors[i]) {
                sptFreeRankMatrix(k->factors[i]);
                free(k->factors[i]);
            }
        free(k->factors);
    }
    k->factors = NULL;
    k->nmodes = 0;
}

/* ---------------------------------------------------- Kruskal tensor -- */
int sptNewKruskalTensor(sptKruskalTensor *k, sptIndex nmodes, const sptIndex ndims[], sptIndex rank) {
    k->nmodes = nmodes;
    k->rank = rank;
    k->ndims = malloc(nmodes * sizeof(sptIndex));
    CHECK_OS(!k->ndims, "Kruskal New");
    for (sptIndex i = 0; i < nmodes; ++i) k->ndims[i] = ndims[i];
    k->lambda = malloc(rank * sizeof(sptValue));
    CHECK_OS(!k->lambda, "Kruskal New");
    k->fit = 0.0;
    k->factors = NULL;
    return 0;
}

void sptFreeKruskalTensor(sptKruskalTensor *k) {
    k->rank = 0;
    k->fit = 0.0;
    free(k->ndims);
    free(k->lambda);
    if (k->factors) {
        for (sptIndex i = 0; i < k->nmodes; ++i)
            if (k->factors[i]) {
                sptFreeMatrix(k->factors[i]);
                free(k->factors[i]);
            }
        free(k->factors);
    }
    k->factors = NULL;
    k->nmodes = 0;
}

/* ------------------------------------------------------ OpenMP lock pool -- */
/* locks.c:21-55: nlocks * padsize locks, lock i initialised at (i % nlocks) * padsize. */
sptMutexPool *SptMutexAllocCustom(sptIndex const num_locks, sptIndex const pad_size) {
    sptMutexPool *pool = (sptMutexPool *)malloc(sizeof *pool);
    if (!pool) return NULL;
    pool->nlocks = num_locks;
    pool->padsize = pad_size;
    omp_lock_t *locks = (omp_lock_t *)malloc((size_t)num_locks * pad_size * sizeof(omp_lock_t));
    if (!locks && num_locks) {
        free(pool);
        return NULL;
    }
    for (sptIndex l = 0; l < num_locks; ++l) omp_init_lock(locks + (size_t)l * pad_size);
    pool->locks = locks;
    pool->initialized = true;
    return pool;
}

sptMutexPool *sptMutexAlloc(void) { return SptMutexAllocCustom(1024, 16); }

void sptMutexFree(sptMutexPool *pool) {
    if (!pool) return;
    omp_lock_t *locks = (omp_lock_t *)pool->locks;
    for (sptIndex l = 0; l < pool->nlocks; ++l) omp_destroy_lock(locks + (size_t)l * pool->padsize);
    free(locks);
    free(pool);
}
