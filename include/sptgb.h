/*
 * sptgb.h -- GB300 extension API of the sparse MTTKRP / CP-ALS library.
 *
 * ParTI.h keeps the reference's host-buffer calling convention: every call
 * moves its inputs to the GPU and its result back.  The functions here let a
 * caller keep a tensor, its per-mode segmented copies and the factor
 * matrices resident in HBM and call the same kernels on device pointers and a
 * caller-chosen CUDA stream (passed as void* so that this header does not
 * need the CUDA headers; NULL is the CUDA default stream, as in the CUDA
 * runtime API).  Nothing here has a counterpart in the reference.
 */
#ifndef SPTGB_H
#define SPTGB_H

#include "ParTI.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ library -- */
const char *sptgbVersion(void);
/* Selects the device and creates the library stream; called lazily by every
 * entry point, so calling it is optional. */
int   sptgbInit(int device);
/* The stream the ParTI.h entry points run on (a cudaStream_t). */
void *sptgbStream(void);
/* Kernels launched by this library since it was loaded. */
uint64_t sptgbLaunchCount(void);
/* Seed for sptRandomizeMatrix and for the factor initialisation of
 * sptCpdAls (the reference seeds with time(NULL), matrix.c:69). */
void  sptgbSetSeed(uint64_t seed);

/* Page-locks (cudaHostRegister) the host arrays of a tensor or a matrix for
 * callers that pass the same host objects to many calls: the host-buffer
 * entry points (sptMTTKRP, sptCudaMTTKRP, sptCpdAls, ...) then copy them by
 * DMA without address translation of pageable pages.  The arrays must not be
 * reallocated or freed while pinned; unpin before freeing.  Pinning pinned
 * memory, or unpinning memory that is not pinned, returns
 * SPTERR_CUDA_ERROR + the CUDA error code. */
int sptgbPinSparseTensor(const sptSparseTensor *X);
int sptgbUnpinSparseTensor(const sptSparseTensor *X);
int sptgbPinMatrix(const sptMatrix *M);
int sptgbUnpinMatrix(const sptMatrix *M);

/* ------------------------------------------- device-resident COO tensor --
 * A COO tensor uploaded once.  sptgbCooPrepareMode builds, on the device,
 * the copy sorted by `mode` (mode first, then the remaining modes in
 * ascending order: sptSparseTensorSortIndexCustomOrder's order) together
 * with its segment data; sptgbCooMTTKRP then runs the segmented kernel on
 * it.  d_mats[m] (m < nmodes) are device factor matrices of ndims[m] rows
 * and `stride` floats per row; d_out receives ndims[mode] rows. */
typedef struct sptgbCoo sptgbCoo;
int  sptgbCooCreate(sptgbCoo **out, const sptSparseTensor *X, void *stream);
int  sptgbCooPrepareMode(sptgbCoo *t, sptIndex mode, void *stream);
int  sptgbCooMTTKRP(sptgbCoo *t, sptIndex mode, const sptIndex *mats_order,
                    const float *const *d_mats, sptIndex rank, sptIndex stride,
                    float *d_out, void *stream);
/* BF16 factor storage, FP32 accumulation: d_mats_bf16[m] hold bf16 rows of
 * `stride` elements (uint16_t bit patterns). */
int  sptgbCooMTTKRPBf16(sptgbCoo *t, sptIndex mode, const sptIndex *mats_order,
                        const uint16_t *const *d_mats_bf16, sptIndex rank, sptIndex stride,
                        float *d_out, void *stream);
/* Device arrays of the copy sorted by `mode` (prepared on demand): inds[m]
 * for m < nmodes and the values, nnz entries each, owned by t. */
int  sptgbCooModeArrays(sptgbCoo *t, sptIndex mode, const uint32_t **inds, const float **vals, void *stream);
sptNnzIndex sptgbCooNnz(const sptgbCoo *t);
size_t      sptgbCooDeviceBytes(const sptgbCoo *t);
/* Time of the last sptgbCooMTTKRP kernel sequence on its stream (ms),
 * measured with CUDA events when timing is enabled. */
void  sptgbCooSetTiming(sptgbCoo *t, int enable);
float sptgbCooLastKernelMs(const sptgbCoo *t);
void  sptgbCooFree(sptgbCoo *t);
/* sptLoadSparseTensor, then (on the device) a lexicographic sort with
 * duplicate coordinates summed in file order and zero sums dropped; the
 * result is marked sorted.  No counterpart in the reference (its loader keeps
 * duplicates). */
int sptgbLoadSparseTensorMerged(sptSparseTensor *tsr, sptIndex start_index, FILE *fp);

/* ------------------------------------------------ resident HiCOO tensor --
 * The HiCOO arrays uploaded once; per output mode, the output-window
 * schedule (blocks ordered by their block index in that mode) is built on
 * the device on first use.  Orders 3 and 4 run the window kernel, others
 * the block kernel.  Same argument meaning as sptgbCooMTTKRP. */
typedef struct sptgbHicoo sptgbHicoo;
int  sptgbHicooCreate(sptgbHicoo **out, const sptSparseTensorHiCOO *h, void *stream);
int  sptgbHicooPrepareMode(sptgbHicoo *t, sptIndex mode, void *stream);
int  sptgbHicooMTTKRP(sptgbHicoo *t, sptIndex mode, const sptIndex *mats_order, const float *const *d_mats,
                      sptIndex rank, sptIndex stride, float *d_out, void *stream);
size_t sptgbHicooDeviceBytes(const sptgbHicoo *t);
void sptgbHicooFree(sptgbHicoo *t);
/* CP-ALS over a HiCOO tensor from caller factors (rank matrices); results
 * as sptgbCpdAls. */
int sptgbCpdAlsHiCOO(sptSparseTensorHiCOO const *h, sptIndex rank, sptIndex niters, double tol,
                     sptRankMatrix **mats, sptValue *lambda, double *fits, sptIndex *iters_done);
/* Same for the HiCOO MTTKRP kernel of sptMTTKRPHiCOO (process-wide). */
void  sptgbHiCOOSetTiming(int enable);
float sptgbHiCOOLastKernelMs(void);

/* ----------------------------------------------------- synthetic tensors --
 * Seeded generator shared by the tests and the benchmark (SplitMix64
 * counter streams; inverse-CDF truncated Zipf; Box-Muller normals). */
enum { SPTGB_DIST_UNIFORM = 0, SPTGB_DIST_ZIPF = 1 };
enum { SPTGB_VAL_U01 = 0, SPTGB_VAL_UPM1 = 1, SPTGB_VAL_LOGNORMAL = 2, SPTGB_VAL_PLANTED = 3 };
typedef struct {
    uint64_t seed;
    sptIndex nmodes;
    sptIndex ndims[8];
    int      coord_dist[8];   /* SPTGB_DIST_* per mode */
    double   zipf_s[8];       /* Zipf exponent per mode */
    uint64_t count;           /* draws (merge=1) or exact unique nnz (merge=0) */
    int      merge_duplicates;/* 1: duplicate draws summed; 0: deduplicate and top up */
    int      value_dist;      /* SPTGB_VAL_* */
    sptIndex planted_rank;    /* SPTGB_VAL_PLANTED: rank of the planted model */
    uint64_t planted_seed;    /* seed of the planted factors, U[0,1) */
    double   noise_sigma;     /* Gaussian noise added to planted values */
} sptgbGenSpec;
/* Fills X (which must be uninitialised) with the generated tensor, sorted
 * lexicographically (mode 0 most significant). */
int sptgbGenerate(sptSparseTensor *X, const sptgbGenSpec *spec);
/* U[lo,hi) fill of rows x ncols (padding columns set to 0), seeded by
 * (seed, stream_id). */
int sptgbFillMatrix(sptMatrix *mtx, uint64_t seed, uint64_t stream_id, float lo, float hi);

/* --------------------------------------------------- CP-ALS with traces --
 * CpdAlsStep semantics from caller factors, returning the fit after every
 * iteration in fits[0..niters) (NaN past an early stop) and the iteration
 * count.  Fits are computed with the full symmetric Gram matrices. */
int sptgbCpdAls(sptSparseTensor const *spten, sptIndex rank, sptIndex niters, double tol,
                sptMatrix **mats, sptValue *lambda, double *fits, sptIndex *iters_done);

/* ------------------------------------------------- batched / served CP-ALS --
 * A server holds CP-ALS jobs of different sizes, orders (3 or 4) and ranks
 * (<= 64) as device-resident slots: mode-sorted tensor records, factors,
 * FP64 Grams.  One step runs one ALS iteration of every admitted job as a
 * single CUDA-graph launch (MTTKRP, solve, normalisation and fit for all
 * slots; the R x R factorisations in FP64, the row-wise contractions in
 * double-float), then completes the jobs that reached their iteration count
 * (GetFinalLambda, factors, lambda and per-iteration fits copied into the
 * job's buffers).  Jobs submitted while others run are admitted at the next
 * step as slots and HBM budget free up (continuous batching).  Each job
 * computes what sptgbCpdAls computes for it (tol = 0).  The MTTKRP unit length
 * per rank group is chosen by timing the candidates on the first step. */
typedef struct sptgbServer sptgbServer;
int  sptgbServerCreate(sptgbServer **out, size_t hbm_budget_bytes, uint32_t max_slots);
/* Queues a job.  X, init[m] (ndims[m] x rank), out[m] (same shape), lambda[rank]
 * and fits[niters] must stay valid until sptgbServerDone reports the job. */
int  sptgbServerSubmit(sptgbServer *s, const sptSparseTensor *X, sptIndex rank, sptIndex niters,
                       sptMatrix *const *init, sptMatrix *const *out, sptValue *lambda, double *fits,
                       uint64_t *ticket);
/* Admits what fits, runs one iteration of every admitted job, completes
 * finished jobs.  *active / *queued receive the counts after the step. */
int  sptgbServerStep(sptgbServer *s, uint32_t *active, uint32_t *queued);
/* 1 once the job's results are in its buffers, 0 before, -1 if it failed
 * (larger than the budget, or a coordinate out of range); *submit_s and
 * *done_s (CLOCK_MONOTONIC seconds) may be NULL. */
int  sptgbServerDone(sptgbServer *s, uint64_t ticket, double *submit_s, double *done_s);
/* Tickets of the jobs that finished (done or failed) since the previous call,
 * in completion order; at most `max` are returned, the rest on later calls. */
uint32_t sptgbServerCompleted(sptgbServer *s, uint64_t *tickets, uint32_t max);
/* Steps until every submitted job is done. */
int  sptgbServerDrain(sptgbServer *s);
size_t sptgbServerBytesInUse(const sptgbServer *s);
/* Unit length (nonzeros) the autotuner chose for rank group g (W = 2<<g). */
uint32_t sptgbServerUnitLength(const sptgbServer *s, int group);
/* 1 when each step runs as one persistent cooperative kernel (opt-in with
 * SPTGB_STEP=persistent when the device and the capture allow cooperative
 * launches), 0 when it runs as the kernel sequence (the default); meaningful
 * after the first step. */
int sptgbServerPersistent(const sptgbServer *s);
/* Kernels one ALS step launches (the nodes of the captured step graph: 1 for
 * the persistent step, one per phase and lane group for the sequence); 0
 * before the first step.  Admission and retirement kernels are not counted. */
uint32_t sptgbServerStepKernels(const sptgbServer *s);
/* The MTTKRP schedule the autotuner chose for rank group `group` (0..3: rank
 * <= 8, 16, 32, 64): unit length in nonzeros, deep (1) or shallow (0) record
 * batches, blocks per SM the kernel's registers are sized for (2 or 3; the
 * persistent step always runs 2), and *from_cache = 1 when the choice came
 * from an earlier server of this process, 0 when it was timed, -1 when the
 * group had no jobs at tuning time.  Meaningful after the first step. */
int sptgbServerSchedule(const sptgbServer *s, int group, uint32_t *unit_len, uint32_t *deep, uint32_t *blocks_per_sm,
                        int *from_cache);
/* Diagnostic of the persistent step's bounded grid barrier: a 4-block
 * cooperative kernel passes two barrier rounds and, with missing != 0, a third
 * that waits for a fifth block; every wait there gives up after 2^14 polls, so
 * the kernel returns with *err = 1 instead of hanging.  *rounds counts the
 * rounds completed, summed over blocks (8 in both cases). */
int sptgbGridBarrierSelfTest(int missing, int *err, unsigned int *rounds);
void sptgbServerFree(sptgbServer *s);

/* ------------------------------------------------ without device allocation --
 * No counterpart in the reference.  ||X||^2 of the tensor's values, as
 * SparseTensorFrobeniusNormSquared computes it (FP32 squares summed in FP64),
 * for callers that must not allocate device memory (their device memory is
 * owned by another allocator, or they cannot pay for cudaMalloc/cudaFree per
 * call): the values and the reduction partials are staged in a fixed 16 MiB
 * array inside the library instead.  At most 4,194,304 nonzeros
 * (SPTERR_VALUE_ERROR above that).  Runs on the calling thread's current
 * device; each call looks up the array's address in that device's context.
 * All calls share the array, so calls that overlap on the GPU race; serialise
 * them.  stream: cudaStream_t as void* (NULL = default stream); the call
 * synchronises the stream and returns once *normsq is written, so it cannot
 * be made while the stream is capturing a CUDA graph. */
int sptgbSparseTensorFrobeniusNormSquaredNoAlloc(sptSparseTensor const *spten, double *normsq, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPTGB_H */
