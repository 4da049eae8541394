/*
 * Text writers of the reference, same formats:
 *   sptDumpSparseTensor   src/sptensor/dump.c:29-52  (order, mode sizes, then
 *                         one line per nonzero: coordinates + start_index,
 *                         tab-separated, value with %f)
 *   sptDumpMatrix         src/matrix/dump.c:34-50    ("R x C matrix", rows of
 *                         %.2f values each followed by a tab, blank line)
 *   sptDumpKruskalTensor  src/ktensor/dump.c:24-51   (header, mode sizes, fit,
 *                         lambda, the factor matrices)
 *   sptDumpRankMatrix, sptDumpRankKruskalTensor  src/matrix/dump.c:60-76,
 *                         src/ktensor/dump.c:55-87 (the same formats)
 *   sptDump*Vector, sptDump*Array  src/vector/dump.c:32-176  ("<type> length:
 *                         n" line, then the entries each followed by a tab)
 *   sptDumpSparseTensorHiCOO  src/sptensor/hicoo/dump.c:28-72  (order, mode
 *                         sizes, nkiters, kschr per mode and kernel, kptr,
 *                         cptr, bptr, binds, einds, values)
 * sptDump[Rank]KruskalTensor prints one lambda entry per mode, as the reference
 * does, and skips factor pointers that are NULL (sptCpdAls leaves
 * factors[nmodes] NULL; the reference's writer would read the matrix it
 * freed there).
 */
#define _GNU_SOURCE
#include <inttypes.h>
#include <stdio.h>
#include "devtensor.h"

#define IO(expr, module)                                                                  \
    do {                                                                                  \
        if ((expr) < 0) {                                                                 \
            spt_ComplainError(module, SPTERR_OS_ERROR, __FILE__, __LINE__, "write failed"); \
            return SPTERR_OS_ERROR;                                                        \
        }                                                                                 \
    } while (0)

int sptDumpSparseTensor(const sptSparseTensor *tsr, sptIndex start_index, FILE *fp) {
    const char *module = "SpTns Dump";
    IO(fprintf(fp, "%" PRIu32 "\n", tsr->nmodes), module);
    for (sptIndex m = 0; m < tsr->nmodes; ++m) {
        if (m) IO(fputs(" ", fp), module);
        IO(fprintf(fp, "%" PRIu32, tsr->ndims[m]), module);
    }
    IO(fputs("\n", fp), module);
    for (sptNnzIndex i = 0; i < tsr->nnz; ++i) {
        for (sptIndex m = 0; m < tsr->nmodes; ++m)
            IO(fprintf(fp, "%" PRIu32 "\t", tsr->inds[m].data[i] + start_index), module);
        IO(fprintf(fp, "%f\n", (double)tsr->values.data[i]), module);
    }
    return 0;
}

int sptDumpMatrix(sptMatrix *mtx, FILE *fp) {
    const char *module = "Mtx Dump";
    IO(fprintf(fp, "%" PRIu32 " x %" PRIu32 " matrix\n", mtx->nrows, mtx->ncols), module);
    for (sptIndex i = 0; i < mtx->nrows; ++i) {
        for (sptIndex j = 0; j < mtx->ncols; ++j) IO(fprintf(fp, "%.2f\t", mtx->values[(size_t)i * mtx->stride + j]), module);
        IO(fprintf(fp, "\n"), module);
    }
    IO(fprintf(fp, "\n"), module);
    return 0;
}

int sptDumpKruskalTensor(sptKruskalTensor *ktsr, FILE *fp) {
    const char *module = "KruskalTns Dump";
    IO(fprintf(fp, "nmodes: %" PRIu32 ", rank: %" PRIu32 "\n", ktsr->nmodes, ktsr->rank), module);
    for (sptIndex m = 0; m < ktsr->nmodes; ++m) {
        if (m) IO(fputs(" ", fp), module);
        IO(fprintf(fp, "%" PRIu32, ktsr->ndims[m]), module);
    }
    IO(fputs("\n", fp), module);
    IO(fprintf(fp, "fit: %lf\n", ktsr->fit), module);
    IO(fprintf(fp, "lambda:\n"), module);
    for (sptIndex m = 0; m < ktsr->nmodes; ++m) IO(fprintf(fp, "%f ", (double)ktsr->lambda[m]), module);
    IO(fprintf(fp, "Factor matrices:\n"), module);
    for (sptIndex m = 0; m < ktsr->nmodes + 1; ++m) {
        if (!ktsr->factors || !ktsr->factors[m]) continue;
        const int r = sptDumpMatrix(ktsr->factors[m], fp);
        if (r) return r;
    }
    return 0;
}

#define DUMP_LIST(name, type, label, fmt, module)                                       \
    int name(type *data, sptNnzIndex len, FILE *fp) {                                    \
        IO(fprintf(fp, label " length: %" PRIu64 "\n", (uint64_t)len), module);        \
        for (sptNnzIndex i = 0; i < len; ++i) IO(fprintf(fp, fmt "\t", data[i]), module); \
        IO(fprintf(fp, "\n"), module);                                                  \
        return 0;                                                                         \
    }
static DUMP_LIST(dump_elements, const sptElementIndex, "sptElementIndexVector", "%" PRIu8, "EleIdxVec Dump")
static DUMP_LIST(dump_indices, const sptIndex, "sptIndexVector", "%" PRIu32, "IdxVec Dump")
static DUMP_LIST(dump_blocks, const sptBlockIndex, "sptBlockIndexVector", "%" PRIu32, "BlkIdxVec Dump")
static DUMP_LIST(dump_nnz, const sptNnzIndex, "sptNnzIndexVector", "%" PRIu64, "NnzIdxVec Dump")
static DUMP_LIST(dump_values, const sptValue, "sptValueVector", "%f", "ValVec Dump")
static DUMP_LIST(dump_index_array, const sptIndex, "sptIndex array", "%" PRIu32, "IdxArray Dump")
static DUMP_LIST(dump_nnz_array, const sptNnzIndex, "sptNnzIndex array", "%" PRIu64, "NnzIdxArray Dump")

int sptDumpElementIndexVector(sptElementIndexVector *vec, FILE *fp) { return dump_elements(vec->data, vec->len, fp); }
int sptDumpIndexVector(sptIndexVector *vec, FILE *fp) { return dump_indices(vec->data, vec->len, fp); }
int sptDumpBlockIndexVector(sptBlockIndexVector *vec, FILE *fp) { return dump_blocks(vec->data, vec->len, fp); }
int sptDumpNnzIndexVector(sptNnzIndexVector *vec, FILE *fp) { return dump_nnz(vec->data, vec->len, fp); }
int sptDumpValueIndexVector(sptValueVector *vec, FILE *fp) { return dump_values(vec->data, vec->len, fp); }
int sptDumpIndexArray(sptIndex *array, sptNnzIndex const n, FILE *fp) { return dump_index_array(array, n, fp); }
int sptDumpNnzIndexArray(sptNnzIndex *array, sptNnzIndex const n, FILE *fp) { return dump_nnz_array(array, n, fp); }

int sptDumpSparseTensorHiCOO(sptSparseTensorHiCOO *const hitsr, FILE *fp) {
    const char *module = "SpTns Dump";
    const sptIndex N = hitsr->nmodes;
    const uint64_t sk = (uint64_t)1 << hitsr->sk_bits;
    int r;
    IO(fprintf(fp, "%" PRIu32 "\n", N), module);
    for (sptIndex m = 0; m < N; ++m) {
        if (m) IO(fputs(" ", fp), module);
        IO(fprintf(fp, "%" PRIu32, hitsr->ndims[m]), module);
    }
    IO(fputs("\n", fp), module);
    IO(fprintf(fp, "nkiters:\n"), module);
    if ((r = sptDumpIndexArray(hitsr->nkiters, N, fp))) return r;
    IO(fprintf(fp, "kschr:\n"), module);
    for (sptIndex m = 0; m < N; ++m) {
        IO(fprintf(fp, "mode %" PRIu32 "\n", m), module);
        const uint64_t nk = ((uint64_t)hitsr->ndims[m] + sk - 1) / sk;
        for (uint64_t i = 0; i < nk; ++i)
            if ((r = sptDumpIndexVector(&hitsr->kschr[m][i], fp))) return r;
    }
    IO(fprintf(fp, "kptr:\n"), module);
    if ((r = sptDumpNnzIndexVector(&hitsr->kptr, fp))) return r;
    IO(fprintf(fp, "cptr:\n"), module);
    if ((r = sptDumpNnzIndexVector(&hitsr->cptr, fp))) return r;
    IO(fprintf(fp, "bptr:\n"), module);
    if ((r = sptDumpNnzIndexVector(&hitsr->bptr, fp))) return r;
    IO(fprintf(fp, "binds:\n"), module);
    for (sptIndex m = 0; m < N; ++m)
        if ((r = sptDumpBlockIndexVector(&hitsr->binds[m], fp))) return r;
    IO(fprintf(fp, "einds:\n"), module);
    for (sptIndex m = 0; m < N; ++m)
        if ((r = sptDumpElementIndexVector(&hitsr->einds[m], fp))) return r;
    IO(fprintf(fp, "values:\n"), module);
    return sptDumpValueIndexVector(&hitsr->values, fp);
}

int sptDumpRankMatrix(sptRankMatrix *mtx, FILE *fp) {
    const char *module = "RankMtx Dump";
    IO(fprintf(fp, "%" PRIu32 " x %" PRIu8 " matrix\n", mtx->nrows, mtx->ncols), module);
    for (sptIndex i = 0; i < mtx->nrows; ++i) {
        for (sptElementIndex j = 0; j < mtx->ncols; ++j)
            IO(fprintf(fp, "%.2f\t", mtx->values[(size_t)i * mtx->stride + j]), module);
        IO(fprintf(fp, "\n"), module);
    }
    IO(fprintf(fp, "\n"), module);
    return 0;
}

int sptDumpRankKruskalTensor(sptRankKruskalTensor *ktsr, FILE *fp) {
    const char *module = "KruskalTns Dump";
    IO(fprintf(fp, "nmodes: %" PRIu32 ", rank: %" PRIu8 "\n", ktsr->nmodes, ktsr->rank), module);
    for (sptIndex m = 0; m < ktsr->nmodes; ++m) {
        if (m) IO(fputs(" ", fp), module);
        IO(fprintf(fp, "%" PRIu32, ktsr->ndims[m]), module);
    }
    IO(fputs("\n", fp), module);
    IO(fprintf(fp, "fit: %lf\n", ktsr->fit), module);
    IO(fprintf(fp, "lambda:\n"), module);
    for (sptIndex m = 0; m < ktsr->nmodes; ++m) IO(fprintf(fp, "%f ", (double)ktsr->lambda[m]), module);
    IO(fprintf(fp, "Factor matrices:\n"), module);
    for (sptIndex m = 0; m < ktsr->nmodes + 1; ++m) {
        if (!ktsr->factors || !ktsr->factors[m]) continue;
        const int r = sptDumpRankMatrix(ktsr->factors[m], fp);
        if (r) return r;
    }
    return 0;
}
