/*
 * ParTI.h -- drop-in public header of the GB300-native sparse MTTKRP / CP-ALS
 * library.
 *
 * Everything a caller of ParTI!'s MTTKRP and CP-ALS path links against is
 * declared here with the same names, argument meaning and struct layouts as
 * ParTI! built with 32-bit indices, 32-bit values and 8-bit element indices
 * (reference: include/includes/types.h:30-94, include/includes/structs.h,
 * include/includes/macros.h:44-52, CMakeLists.txt:24-26).  The compute behind
 * every declared MTTKRP / sort / HiCOO / CP-ALS entry point runs on the GPU;
 * there is no CPU implementation of those operations in this library.
 *
 * Struct layouts are byte-identical to the reference so that objects built by
 * code compiled against ParTI!'s own header can be handed to this library.
 */
#ifndef PARTI_H
#define PARTI_H

#include <stddef.h>
#include <stdio.h>
#include <stdint.h>
#include <inttypes.h>
#include <math.h>      /* the reference's header includes it; its callers use pow() */
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- types --
 * Widths fixed at index 32 / value 32 / element 8 (types.h:30-94). */
typedef uint32_t sptIndex;
typedef uint32_t sptBlockIndex;
typedef float    sptValue;
typedef uint8_t  sptElementIndex;
typedef uint16_t sptBlockMatrixIndex;
typedef sptBlockIndex sptBlockNnzIndex;
typedef uint64_t sptNnzIndex;
#if defined(__SIZEOF_INT128__)
typedef unsigned __int128 sptMortonIndex;
#endif

#define PARTI_INDEX_TYPEWIDTH 32
#define PARTI_VALUE_TYPEWIDTH 32
#define PARTI_ELEMENT_INDEX_TYPEWIDTH 8
#define PARTI_INDEX_MAX UINT32_MAX
/* printf / scanf conversions of the types above (types.h:30-92); callers
 * such as examples/mttkrp.c read their options with them */
#define PARTI_PRI_INDEX PRIu32
#define PARTI_SCN_INDEX SCNu32
#define PARTI_PRI_BLOCK_INDEX PRIu32
#define PARTI_SCN_BLOCK_INDEX SCNu32
#define PARTI_PRI_VALUE "f"
#define PARTI_SCN_VALUE "f"
#define PARTI_PRI_ELEMENT_INDEX PRIu8
#define PARTI_SCN_ELEMENT_INDEX SCNu8
#define PARTI_PRI_BLOCKMATRIX_INDEX PRIu16
#define PARTI_SCN_BLOCKMATRIX_INDEX SCNu16
#define PARTI_PRI_BLOCKNNZ_INDEX PARTI_PRI_BLOCK_INDEX
#define PARTI_SCN_BLOCKNNZ_INDEX PARTI_SCN_BLOCK_INDEX
#define PARTI_PRI_NNZ_INDEX PRIu64
/* Tuning constants of the reference's CPU schedules (macros.h:23-28); its
 * HiCOO callers print them and pick a reduction schedule with them. */
#define NUM_CORES 32
#define L1_SIZE 32000
#define PAR_DEGREE_REDUCE 20
#define PAR_MAX_DEGREE 100
#define PAR_MIN_DEGREE 4
#define PARTI_SCN_NNZ_INDEX SCNu64

/* --------------------------------------------------------------- errors --
 * Same codes as SptError (macros.h:44-52).  CUDA failures are reported as
 * SPTERR_CUDA_ERROR + cudaError_t, as spt_CheckCudaError does
 * (src/error/error.h:81-86). */
typedef enum {
    SPTERR_NO_ERROR       = 0,
    SPTERR_UNKNOWN        = 1,
    SPTERR_SHAPE_MISMATCH = 2,
    SPTERR_VALUE_ERROR    = 3,
    SPTERR_ZERO_DIVISION  = 4,
    SPTERR_NO_MORE        = 99,
    SPTERR_OS_ERROR       = 0x10000,
    SPTERR_CUDA_ERROR     = 0x20000,
} SptError;

/* ----------------------------------------------------------- containers --
 * structs.h:23-203, same member order and types. */
typedef struct { sptNnzIndex len; sptNnzIndex cap; sptValue *data; } sptValueVector;
typedef struct { sptNnzIndex len; sptNnzIndex cap; sptIndex *data; } sptIndexVector;
typedef struct { sptNnzIndex len; sptNnzIndex cap; sptElementIndex *data; } sptElementIndexVector;
typedef struct { sptNnzIndex len; sptNnzIndex cap; sptBlockIndex *data; } sptBlockIndexVector;
typedef struct { sptNnzIndex len; sptNnzIndex cap; sptNnzIndex *data; } sptNnzIndexVector;

/* Dense row-major matrix; stride = ncols rounded up to 8 (matrix.c:37-56). */
typedef struct {
    sptIndex nrows;
    sptIndex ncols;
    sptIndex cap;
    sptIndex stride;
    sptValue *values;
} sptMatrix;

/* Dense matrix with a small column count (structs.h:76-82). */
typedef struct {
    sptIndex        nrows;
    sptElementIndex ncols;
    sptIndex        cap;
    sptElementIndex stride;
    sptValue        *values;
} sptRankMatrix;

/* COO sparse tensor (structs.h:113-120): inds[m].data[x] is the mode-m
 * coordinate of nonzero x, values.data[x] its value. */
typedef struct {
    sptIndex nmodes;
    sptIndex *sortorder;
    sptIndex *ndims;
    sptNnzIndex nnz;
    sptIndexVector *inds;
    sptValueVector values;
} sptSparseTensor;

/* HiCOO sparse tensor (structs.h:126-156). */
typedef struct {
    sptIndex            nmodes;
    sptIndex            *sortorder;
    sptIndex            *ndims;
    sptNnzIndex         nnz;
    sptElementIndex     sb_bits;
    sptElementIndex     sk_bits;
    sptElementIndex     sc_bits;
    sptNnzIndexVector   kptr;
    sptIndexVector      **kschr;
    sptIndex            *nkiters;
    sptNnzIndexVector   cptr;
    sptIndexVector      **kschr_balanced;
    sptIndexVector      **kschr_balanced_pos;
    sptIndex            *nkpars;
    sptIndexVector      *kschr_rest;
    sptNnzIndexVector   knnzs;
    sptNnzIndexVector   bptr;
    sptBlockIndexVector *binds;
    sptElementIndexVector *einds;
    sptValueVector      values;
} sptSparseTensorHiCOO;

/* Kruskal tensor, the CP-ALS result (structs.h:196-203). */
typedef struct {
    sptIndex nmodes;
    sptIndex rank;
    sptIndex *ndims;
    sptValue *lambda;
    double fit;
    sptMatrix **factors;
} sptKruskalTensor;

typedef struct {
    sptIndex nmodes;
    sptElementIndex rank;
    sptIndex *ndims;
    sptValue *lambda;
    double fit;
    sptRankMatrix **factors;
} sptRankKruskalTensor;

typedef struct { sptIndex key; sptIndex value; } sptKeyValuePair;

/* OpenMP lock pool (structs.h:228-238, locks.c:21-55): `locks` holds
 * nlocks * padsize omp_lock_t, lock i at (i % nlocks) * padsize.  Callers of
 * sptOmpMTTKRP_Lock create one; the library itself takes no lock in it. */
typedef struct {
    bool initialized;
    sptIndex nlocks;
    sptIndex padsize;
    void *locks;
} sptMutexPool;
sptMutexPool *sptMutexAlloc(void);
sptMutexPool *SptMutexAllocCustom(sptIndex const num_locks, sptIndex const pad_size);
void sptMutexFree(sptMutexPool *pool);

/* Semi-sparse tensor (structs.h:167-175): mode `mode` dense, the others
 * sparse; nnz dense fibers of `stride` values (ndims[mode] rounded up to 8),
 * inds[m] the fiber coordinates for m != mode (inds[mode] unused). */
typedef struct {
    sptIndex nmodes;
    sptIndex *ndims;
    sptIndex mode;
    sptNnzIndex nnz;
    sptIndexVector *inds;
    sptIndex stride;
    sptMatrix values;
} sptSemiSparseTensor;

/* Opaque timer (macros.h:38); this library's timers are CUDA events on the
 * library stream when use_cuda != 0, CLOCK_MONOTONIC otherwise. */
typedef struct sptTagTimer *sptTimer;

/* ------------------------------------------------------ error reporting --
 * Thread-local last error, as src/error/error.c:28-116. */
int  sptGetLastError(const char **module, const char **file, unsigned *line, const char **reason);
void sptClearLastError(void);

/* Assertion and helpers of include/includes/helper_funcs.h:35-51: sptAssert
 * prints the failed expression and aborts (spt_Panic, src/error/error.c:75);
 * sptBytesString returns a malloc'd "12.34MB"-style string (src/base.c:25). */
void  spt_Panic(const char *file, unsigned line, const char *expr);
#define sptAssert(expr) ((expr) ? (void)0 : spt_Panic(__FILE__, __LINE__, #expr))
char *sptBytesString(uint64_t const bytes);

/* ------------------------------------------------------------- timers -- */
int    sptNewTimer(sptTimer *timer, int use_cuda);
int    sptStartTimer(sptTimer timer);
int    sptStopTimer(sptTimer timer);
double sptElapsedTime(const sptTimer timer);
double sptPrintElapsedTime(const sptTimer timer, const char *name);
double sptPrintAverageElapsedTime(const sptTimer timer, const int niters, const char *name);
int    sptFreeTimer(sptTimer timer);
int    sptCudaSetDevice(int device);
int    sptCudaGetLastError(void);

/* ------------------------------------------------------------- vectors --
 * include/includes/vectors.h: same growth rule (cap += cap/2). */
sptNnzIndex sptMaxNnzIndexArray(sptNnzIndex const *indices, sptNnzIndex const size);
sptIndex    sptMaxIndexArray(sptIndex const *indices, sptNnzIndex const size);
void        sptPairArraySort(sptKeyValuePair *kvarray, sptIndex const length);

int  sptNewValueVector(sptValueVector *vec, uint64_t len, uint64_t cap);
int  sptConstantValueVector(sptValueVector *const vec, sptValue const val);
int  sptCopyValueVector(sptValueVector *dest, const sptValueVector *src, int const nt);
int  sptAppendValueVector(sptValueVector *vec, sptValue const value);
int  sptResizeValueVector(sptValueVector *vec, sptNnzIndex const size);
void sptFreeValueVector(sptValueVector *vec);

int  sptNewIndexVector(sptIndexVector *vec, uint64_t len, uint64_t cap);
int  sptConstantIndexVector(sptIndexVector *const vec, sptIndex const num);
int  sptCopyIndexVector(sptIndexVector *dest, const sptIndexVector *src, int const nt);
int  sptAppendIndexVector(sptIndexVector *vec, sptIndex const value);
int  sptResizeIndexVector(sptIndexVector *vec, sptNnzIndex const size);
void sptFreeIndexVector(sptIndexVector *vec);

int  sptNewElementIndexVector(sptElementIndexVector *vec, uint64_t len, uint64_t cap);
int  sptAppendElementIndexVector(sptElementIndexVector *vec, sptElementIndex const value);
int  sptResizeElementIndexVector(sptElementIndexVector *vec, sptNnzIndex const size);
void sptFreeElementIndexVector(sptElementIndexVector *vec);

int  sptNewBlockIndexVector(sptBlockIndexVector *vec, uint64_t len, uint64_t cap);
int  sptAppendBlockIndexVector(sptBlockIndexVector *vec, sptBlockIndex const value);
int  sptResizeBlockIndexVector(sptBlockIndexVector *vec, sptNnzIndex const size);
void sptFreeBlockIndexVector(sptBlockIndexVector *vec);

int  sptNewNnzIndexVector(sptNnzIndexVector *vec, uint64_t len, uint64_t cap);
int  sptAppendNnzIndexVector(sptNnzIndexVector *vec, sptNnzIndex const value);
int  sptResizeNnzIndexVector(sptNnzIndexVector *vec, sptNnzIndex const size);
void sptFreeNnzIndexVector(sptNnzIndexVector *vec);

/* ------------------------------------------------------- dense matrices --
 * include/includes/matrices.h (containers; the CP-ALS reductions run on the
 * GPU inside sptCpdAls). */
int  sptNewMatrix(sptMatrix *mtx, sptIndex const nrows, sptIndex const ncols);
int  sptResizeMatrix(sptMatrix *mtx, sptIndex const new_nrows);
int  sptRandomizeMatrix(sptMatrix *mtx, sptIndex const nrows, sptIndex const ncols);
int  sptIdentityMatrix(sptMatrix *mtx);
int  sptConstantMatrix(sptMatrix *const mtx, sptValue const val);
int  sptCopyMatrix(sptMatrix *dest, const sptMatrix *src);
void sptFreeMatrix(sptMatrix *mtx);
sptValue sptRandomValue(void);

/* ---------------------------------------------------- COO sparse tensor --
 * include/includes/sptensors.h. */
int    sptNewSparseTensor(sptSparseTensor *tsr, sptIndex nmodes, const sptIndex ndims[]);
int    sptCopySparseTensor(sptSparseTensor *dest, const sptSparseTensor *src, int const nt);
void   sptFreeSparseTensor(sptSparseTensor *tsr);
double SparseTensorFrobeniusNormSquared(sptSparseTensor const *const spten);

/* Host-side summaries and reorderings (src/sptensor/status.c:24-58,
 * src/sptensor/sort.c:371-380): the density, a printed summary, and the
 * reference's deterministic element shuffle (srand(z + 1) per position). */
double sptSparseTensorDensity(sptSparseTensor const *const tsr);
void   sptSparseTensorStatus(sptSparseTensor *tsr, FILE *fp);
void   sptGetRandomShuffleElements(sptSparseTensor *tsr);

void sptGetBestModeOrder(sptIndex *mode_order, sptIndex const mode, sptIndex const *ndims, sptIndex const nmodes);
void sptGetWorstModeOrder(sptIndex *mode_order, sptIndex const mode, sptIndex const *ndims, sptIndex const nmodes);

/* Device sorts, bit-exact with the reference's orders on unique coordinates
 * (src/sptensor/sort.c:410-585).  tk is accepted and ignored. */
void sptSparseTensorSortIndex(sptSparseTensor *tsr, int force, int tk);
void sptSparseTensorSortIndexAtMode(sptSparseTensor *tsr, sptIndex const mode, int force, int tk);
void sptSparseTensorSortIndexCustomOrder(sptSparseTensor *tsr, sptIndex const *mode_order, int force, int tk);
void sptSparseTensorSortIndexRowBlock(sptSparseTensor *tsr, int force, const sptNnzIndex begin,
                                      const sptNnzIndex end, const sptElementIndex sk_bits, int const tk);
void sptSparseTensorSortIndexMorton(sptSparseTensor *tsr, int force, const sptNnzIndex begin,
                                    const sptNnzIndex end, const sptElementIndex sb_bits, int tk);
int  sptSparseTensorMixedOrder(sptSparseTensor *tsr, const sptElementIndex sb_bits,
                               const sptElementIndex sk_bits, int const tk);

/* ------------------------------------------------------ HiCOO container -- */
int  sptNewSparseTensorHiCOO(sptSparseTensorHiCOO *hitsr, const sptIndex nmodes, const sptIndex ndims[],
                             const sptNnzIndex nnz, const sptElementIndex sb_bits,
                             const sptElementIndex sk_bits, const sptElementIndex sc_bits);
void sptFreeSparseTensorHiCOO(sptSparseTensorHiCOO *hitsr);
/* COO -> HiCOO on the GPU; sorts tsr in place exactly as the reference does
 * (src/sptensor/hicoo/convert.c:300-497). */
int  sptSparseTensorToHiCOO(sptSparseTensorHiCOO *hitsr, sptNnzIndex *max_nnzb, sptSparseTensor *tsr,
                            const sptElementIndex sb_bits, const sptElementIndex sk_bits, int const tk);
int  sptSetKernelPointers(sptNnzIndexVector *kptr, sptSparseTensor *tsr, const sptElementIndex sk_bits);
double sptSparseTensorFrobeniusNormSquaredHiCOO(sptSparseTensorHiCOO const *const hitsr);
/* The HiCOO summary the reference prints (hicoo/status.c:28-118): sizes,
 * storage, schedule per mode, block-size statistics and the suggested
 * parameters, in the same lines. */
void sptSparseTensorStatusHiCOO(sptSparseTensorHiCOO *hitsr, FILE *fp);

/* --------------------------------------------------------------- MTTKRP --
 * mats[0..nmodes-1] are the factor matrices, mats[nmodes] receives the
 * result rows [0, ndims[mode]); mats_order[1..nmodes-1] lists the factors
 * multiplied (src/sptensor/mttkrp.c:39-115).  All variants run on the GPU;
 * thread counts, reduction copies and impl_num are accepted and ignored. */
int sptMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[], sptIndex const mode);
int sptOmpMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[],
                 sptIndex const mode, const int tk);
int sptOmpMTTKRP_Reduce(sptSparseTensor const *const X, sptMatrix *mats[], sptMatrix *copy_mats[],
                        sptIndex const mats_order[], sptIndex const mode, const int tk);
/* mttkrp_omp.c:255-395; the lock pool is not used (the product runs on the GPU). */
int sptOmpMTTKRP_Lock(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex const mats_order[],
                      sptIndex const mode, const int tk, sptMutexPool *lock_pool);
int sptCudaMTTKRP(sptSparseTensor const *const X, sptMatrix *mats[], sptIndex *const mats_order,
                  sptIndex const mode, sptIndex const impl_num);
int sptCudaMTTKRPOneKernel(sptSparseTensor const *const X, sptMatrix **const mats, sptIndex *const mats_order,
                           sptIndex const mode, sptIndex const impl_num);
int sptMTTKRPHiCOO(sptSparseTensorHiCOO const *const hitsr, sptMatrix *mats[], sptIndex const mats_order[],
                   sptIndex const mode);
int sptOmpMTTKRPHiCOO(sptSparseTensorHiCOO const *const hitsr, sptMatrix *mats[], sptIndex const mats_order[],
                      sptIndex const mode, const int nt);
/* The rank-matrix forms (hicoo/mttkrp.c:158-245, hicoo/mttkrp_omp.c:158-212, :555-680, :1214-1351):
 * the same product with sptRankMatrix factors and output; thread counts, the
 * reduction copies and `balanced` are not used. */
int sptMTTKRPHiCOO_MatrixTiling(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                sptIndex const mats_order[], sptIndex const mode);
int sptOmpMTTKRPHiCOO_MatrixTiling(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                   sptIndex const mats_order[], sptIndex const mode, const int nt);
int sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                             sptIndex const mats_order[], sptIndex const mode, const int tk,
                                             int balanced);
int sptOmpMTTKRPHiCOO_MatrixTiling_Scheduled_Reduce(sptSparseTensorHiCOO const *const hitsr, sptRankMatrix *mats[],
                                                    sptRankMatrix *copy_mats[], sptIndex const mats_order[],
                                                    sptIndex const mode, const int tk, int balanced);

/* Semi-sparse tensors and sparse tensor times matrix (ssptensors.h:26-31,
 * sptensors.h:136-139): Y = X x_mode U, one dense fiber of U->ncols values per
 * distinct coordinate of the other modes.  X is sorted at `mode` (mode last)
 * in place, as the reference does; the products are accumulated on the GPU
 * in nonzero order with separately rounded multiplies and adds. */
int  sptNewSemiSparseTensor(sptSemiSparseTensor *tsr, sptIndex nmodes, sptIndex mode, const sptIndex ndims[]);
void sptFreeSemiSparseTensor(sptSemiSparseTensor *tsr);
int  sptSemiSparseTensorToSparseTensor(sptSparseTensor *dest, const sptSemiSparseTensor *src, sptValue epsilon);
int  sptSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U, sptIndex const mode);
int  sptOmpSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U, sptIndex const mode);
int  sptCudaSparseTensorMulMatrix(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U,
                                  sptIndex const mode);
int  sptCudaSparseTensorMulMatrixOneKernel(sptSemiSparseTensor *Y, sptSparseTensor *X, const sptMatrix *U,
                                           sptIndex const mode, sptIndex const impl_num,
                                           sptNnzIndex const smen_size);

/* Text tensor input (load.c:31-84): nmodes, sizes, then per nonzero the
 * indices (start_index based) and the value; parsed on the GPU, result equal
 * to the reference's (zero values removed as collect.c:29-49 does). */
int sptLoadSparseTensor(sptSparseTensor *tsr, sptIndex start_index, FILE *fp);
/* Text output in the reference's formats (sptensor/dump.c:29-52,
 * matrix/dump.c:34-50, ktensor/dump.c:24-51; NULL factor pointers skipped). */
int sptDumpSparseTensor(const sptSparseTensor *tsr, sptIndex start_index, FILE *fp);
int sptDumpMatrix(sptMatrix *mtx, FILE *fp);
/* vector/dump.c:32-176 ("<type> length: n", entries tab-separated) and
 * sptensor/hicoo/dump.c:28-72 (every HiCOO array in that layout). */
int sptDumpElementIndexVector(sptElementIndexVector *vec, FILE *fp);
int sptDumpIndexVector(sptIndexVector *vec, FILE *fp);
int sptDumpBlockIndexVector(sptBlockIndexVector *vec, FILE *fp);
int sptDumpNnzIndexVector(sptNnzIndexVector *vec, FILE *fp);
int sptDumpValueIndexVector(sptValueVector *vec, FILE *fp);
int sptDumpIndexArray(sptIndex *array, sptNnzIndex const n, FILE *fp);
int sptDumpNnzIndexArray(sptNnzIndex *array, sptNnzIndex const n, FILE *fp);
int sptDumpSparseTensorHiCOO(sptSparseTensorHiCOO *const hitsr, FILE *fp);

/* ------------------------------------------------------ Kruskal / CP-ALS -- */
int  sptNewKruskalTensor(sptKruskalTensor *ktsr, sptIndex nmodes, const sptIndex ndims[], sptIndex rank);
void sptFreeKruskalTensor(sptKruskalTensor *ktsr);
int  sptDumpKruskalTensor(sptKruskalTensor *ktsr, FILE *fp);

/* The dense ALS pieces on caller matrices (ranks up to 64), on the GPU:
 * Hadamard of the other Grams' upper triangles into mats[nmodes]
 * (matrix.c:341-386, FP32 in the same order); the normal equations X G = rhs
 * for every row of rhs, G that Hadamard (matrix_solver.c:32-83; FP64
 * Cholesky, LU when G is not positive definite); column 2-norm and max-norm
 * normalisation (matrix.c:390-554), GetFinalLambda (matrix.c:557-573); the
 * fit and its parts (ktensor.c:102-257, the same triangles and formulas). */
int    sptMatrixDotMulSeqTriangle(sptIndex const mode, sptIndex const nmodes, sptMatrix **mats);
int    sptMatrixSolveNormals(sptIndex const mode, sptIndex const nmodes, sptMatrix **aTa, sptMatrix *rhs);
int    sptMatrix2Norm(sptMatrix *const A, sptValue *const lambda);
int    sptMatrixMaxNorm(sptMatrix *const A, sptValue *const lambda);
void   GetFinalLambda(sptIndex const rank, sptIndex const nmodes, sptMatrix **mats, sptValue *const lambda);
double sptKruskalTensorFit(sptSparseTensor const *const spten, sptValue const *const lambda, sptMatrix **mats,
                           sptMatrix **ata);
double sptKruskalTensorFrobeniusNormSquared(sptIndex const nmodes, sptValue const *const lambda, sptMatrix **ata);
double sptSparseKruskalTensorInnerProduct(sptIndex const nmodes, sptValue const *const lambda, sptMatrix **mats);

/* One CP-ALS run from caller-initialised factors mats[0..nmodes-1] (and a
 * scratch mats[nmodes] with max_dim rows); returns the last fit
 * (src/sptensor/cpd.c:32-137). */
double CpdAlsStep(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters,
                  double const tol, sptMatrix **mats, sptValue *const lambda);
int sptCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters,
              double const tol, sptKruskalTensor *ktensor);
int sptOmpCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters,
                 double const tol, const int tk, const int use_reduce, sptKruskalTensor *ktensor);
int sptCudaCpdAls(sptSparseTensor const *const spten, sptIndex const rank, sptIndex const niters,
                  double const tol, sptKruskalTensor *ktensor);

/* Rank matrices and rank Kruskal tensors (matrices.h:69-74, ktensors.h:43-45). */
int  sptNewRankMatrix(sptRankMatrix *mtx, sptIndex const nrows, sptElementIndex const ncols);
int  sptRandomizeRankMatrix(sptRankMatrix *mtx, sptIndex const nrows, sptElementIndex const ncols);
int  sptConstantRankMatrix(sptRankMatrix *mtx, sptValue const val);
void sptFreeRankMatrix(sptRankMatrix *mtx);
int  sptNewRankKruskalTensor(sptRankKruskalTensor *ktsr, sptIndex nmodes, const sptIndex ndims[],
                             sptElementIndex rank);
void sptFreeRankKruskalTensor(sptRankKruskalTensor *ktsr);
int  sptDumpRankMatrix(sptRankMatrix *mtx, FILE *fp);
int  sptDumpRankKruskalTensor(sptRankKruskalTensor *ktsr, FILE *fp);

/* The dense ALS helpers on rank matrices (rankmatrix.c:137-378,
 * rankmatrix_solver.c:32-84, rankktensor.c:101-257): the same results as
 * the sptMatrix forms above; sptKruskalTensorFitHiCOO is sptKruskalTensorFit
 * with the HiCOO tensor's norm. */
int    sptRankMatrixDotMulSeqTriangle(sptIndex const mode, sptIndex const nmodes, sptRankMatrix **mats);
int    sptRankMatrixSolveNormals(sptIndex const mode, sptIndex const nmodes, sptRankMatrix **aTa,
                                 sptRankMatrix *rhs);
int    sptRankMatrix2Norm(sptRankMatrix *const A, sptValue *const lambda);
int    sptRankMatrixMaxNorm(sptRankMatrix *const A, sptValue *const lambda);
void   GetRankFinalLambda(sptElementIndex const rank, sptIndex const nmodes, sptRankMatrix **mats,
                          sptValue *const lambda);
double sptKruskalTensorFitHiCOO(sptSparseTensorHiCOO const *const hitsr, sptValue const *const lambda,
                                sptRankMatrix **mats, sptRankMatrix **ata);
double sptKruskalTensorFrobeniusNormSquaredRank(sptIndex const nmodes, sptValue const *const lambda,
                                                sptRankMatrix **ata);
double sptSparseKruskalTensorInnerProductRank(sptIndex const nmodes, sptValue const *const lambda,
                                              sptRankMatrix **mats);

/* CP-ALS over a HiCOO tensor (cpds.h:46-59, src/sptensor/hicoo/cpd.c:149-195):
 * the same loop with the HiCOO MTTKRP; factors are rank matrices.  The
 * OpenMP variant's tk and balanced arguments are accepted and ignored. */
int sptCpdAlsHiCOO(sptSparseTensorHiCOO const *const hitsr, sptIndex const rank, sptIndex const niters,
                   double const tol, sptRankKruskalTensor *ktensor);
int sptOmpCpdAlsHiCOO(sptSparseTensorHiCOO const *const hitsr, sptIndex const rank, sptIndex const niters,
                      double const tol, const int tk, int balanced, sptRankKruskalTensor *ktensor);

#ifdef __cplusplus
}
#endif

#endif /* PARTI_H */
