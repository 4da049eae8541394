/*
 * Text writers of the reference, same formats:
 *   sptDumpSparseTensor   src/sptensor/dump.c:29-52  (order, mode sizes, then
 *                         one line per nonzero: coordinates + start_index,
 *                         tab-separated, value with %f)
 *   sptDumpMatrix         src/matrix/dump.c:34-50    ("R x C matrix", rows of
 *                         %.2f values each followed by a tab, blank line)
 *   sptDumpKruskalTensor  src/ktensor/dump.c:24-51   (header, mode sizes, fit,
 *                         lambda, the factor matrices)
 * sptDumpKruskalTensor prints one lambda entry per mode, as the reference
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
