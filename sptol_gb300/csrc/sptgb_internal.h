/*
 * Internal interface between the C host layer (the .c files of csrc/host) and the CUDA
 * translation units (the .cu files of csrc/cuda).  Plain C types only; every launcher
 * is extern "C", takes device pointers and a stream, and returns a cudaError_t
 * value (0 on success) so that the host layer maps it to
 * SPTERR_CUDA_ERROR + code.
 */
#ifndef SPTGB_INTERNAL_H
#define SPTGB_INTERNAL_H

#include <stdint.h>
#include <stddef.h>
#include <cuda_runtime_api.h>
#include "../../include/ParTI.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SPTGB_MAX_MODES 8

/* ----------------------------------------------------------- context -- */
int          sptgb_ctx(void);            /* lazy init; returns SptError code */
cudaStream_t sptgb_stream(void);
int          sptgb_sm_count(void);        /* SMs of the library's device */
cudaStream_t sptgb_copy_stream(void);
void         sptgb_count_launch(unsigned n);
/* Kernels enqueued while a stream is captured run only when the graph is
 * launched: the capture takes its count back, each graph launch adds it. */
void         sptgb_uncount_launch(uint64_t n);

/* Records the error in the thread-local last-error slot and prints it like
 * the reference's spt_ComplainError (src/error/error.c:33-60). */
void spt_ComplainError(const char *module, int errcode, const char *file, unsigned line, const char *reason);
int  sptgb_cuda_fail(cudaError_t e, const char *module, const char *file, unsigned line);

#define SPTGB_CHECK(expr, module) do { int _e = (expr); if (_e) { \
        spt_ComplainError(module, _e, __FILE__, __LINE__, NULL); return _e; } } while (0)
#define SPTGB_CUDA(expr, module) do { cudaError_t _c = (expr); if (_c != cudaSuccess) \
        return sptgb_cuda_fail(_c, module, __FILE__, __LINE__); } while (0)

/* Grow-only device buffer. */
typedef struct { void *ptr; size_t cap; } sptgb_dbuf;
int  sptgb_dbuf_reserve(sptgb_dbuf *b, size_t bytes);
void sptgb_dbuf_release(sptgb_dbuf *b);

/* ----------------------------------------------------------- sorting --
 * Stable LSD radix sort of (key, val) u32 pairs over key bits [0, bits).
 * keys/vals are double buffers ([0] holds the input); on return *which
 * tells which buffer holds the result.  tmp must hold
 * sptgb_radix_tmp_bytes(n) bytes. */
size_t      sptgb_radix_tmp_bytes(uint64_t n);
cudaError_t sptgb_radix_sort_u32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int bits,
                                 void *tmp, int *which, cudaStream_t s);

/* Key slices computed from coordinates gathered through perm:
 *   kind 0: key = inds[mode][perm[i]] >> shift
 *   kind 1: 32-bit slice `slice` of the 3-D Morton key (sort.c:748-805)
 *   kind 2: 32-bit slice `slice` of the 4-D Morton key (sort.c:816-995) */
typedef struct {
    const uint32_t *inds[SPTGB_MAX_MODES];
    int nmodes;
    int kind;
    int mode;
    int shift;
    int slice;
} sptgb_keyspec;
cudaError_t sptgb_make_keys(const sptgb_keyspec *ks, const uint32_t *perm, uint32_t *keys,
                            uint64_t n, cudaStream_t s);
cudaError_t sptgb_iota_u32(uint32_t *p, uint64_t n, uint32_t start, cudaStream_t s);
/* out[i] = in[perm[i]] for 4-byte elements. */
cudaError_t sptgb_gather_u32(const uint32_t *in, const uint32_t *perm, uint32_t *out, uint64_t n, cudaStream_t s);
/* out[i] = in[perm[i]] for 1-byte elements. */
cudaError_t sptgb_gather_u8(const uint8_t *in, const uint32_t *perm, uint8_t *out, uint64_t n, cudaStream_t s);

/* ------------------------------------------------------- COO MTTKRP --
 * Segmented MTTKRP over a copy sorted by the output mode. */
typedef struct {
    const uint32_t *rows;                      /* [nnz] output-mode coordinates, non-decreasing */
    const uint32_t *idx[SPTGB_MAX_MODES - 1];  /* [nnz] coordinates of the product modes */
    const void     *fac[SPTGB_MAX_MODES - 1];  /* factor rows of the product modes (f32 or bf16) */
    const float    *vals;                      /* [nnz] */
    float          *out;                       /* [out_rows x stride] */
    uint64_t        nnz;
    uint32_t        out_rows;
    uint32_t        nprod;                     /* nmodes - 1 */
    uint32_t        rank;
    uint32_t        stride;
    int             bf16;                      /* factors stored as bf16 */
    const void     *rec;                       /* order 3: [nnz] 16-byte records {row, idx[0], idx[1], value}
                                                  (sptgb_pack_records), used instead of rows/idx/vals; order 4:
                                                  {row, idx[0], idx[1], idx[2]} (sptgb_pack_records4) with vals */
    /* Records only: run units [unit_begin, unit_end) of SPTGB_REC_UNIT
     * nonzeros (unit_end 0 = all) into an output that is already zero when
     * out_zeroed.  Ranges launched one after another on one stream give the
     * same result as one launch; rows below the first row of a later range
     * are final once the earlier ranges are done. */
    uint64_t        unit_begin, unit_end;
    int             out_zeroed;
} sptgb_mttkrp_args;
#define SPTGB_REC_UNIT 256u
/* Row-quantile split of sorted records into k ranges (1 < k <= 8): for
 * c = 1..k-1, out[2(c-1)] = the unit holding the first record whose row is
 * >= c*rows/k (rounded down to a unit boundary) and out[2(c-1)+1] = the row
 * of the record just before that unit (0 when the unit is 0). */
cudaError_t sptgb_rec_chunk_bounds(const void *rec, uint64_t n, uint32_t rows, int k, uint32_t *out, cudaStream_t s);
cudaError_t sptgb_mttkrp_coo(const sptgb_mttkrp_args *a, cudaStream_t s);
/* rec[i] = {rows[i], ia[i], ib[i], bits of vals[i]} for the order-3 kernel.
 * An ia / ib coordinate at or above lim_a / lim_b is replaced by 0 and, when
 * `bad` is given, sets *bad = 1 (so the product kernel only sees rows that
 * exist; the caller reports the error). */
cudaError_t sptgb_pack_records(const uint32_t *rows, const uint32_t *ia, const uint32_t *ib, const float *vals,
                               uint32_t lim_a, uint32_t lim_b, unsigned int *bad, void *rec, uint64_t n,
                               cudaStream_t s);
/* Order-4 records {rows[i], ia[i], ib[i], ic[i]} (the values stay in their own
 * array); out-of-range ia / ib / ic as in sptgb_pack_records. */
cudaError_t sptgb_pack_records4(const uint32_t *rows, const uint32_t *ia, const uint32_t *ib, const uint32_t *ic,
                                uint32_t lim_a, uint32_t lim_b, uint32_t lim_c, unsigned int *bad, void *rec,
                                uint64_t n, cudaStream_t s);
/* dst[i] = src[perm[i]] for 16-byte records. */
cudaError_t sptgb_gather_records(const void *src, const uint32_t *perm, void *dst, uint64_t n, cudaStream_t s);

/* ---------------------------------------------------- HiCOO pieces -- */
/* flags[i] = 1 when nonzero i starts a new group (coordinates >> bits differ
 * from nonzero i-1), for i in [0, n); flags[0] = 1. */
cudaError_t sptgb_mark_groups(const uint32_t *const *inds, int nmodes, int bits, uint64_t n,
                              uint32_t *flags, cudaStream_t s);
/* Exclusive prefix sum of u32 flags into u32 positions; *total receives the
 * sum (device pointer). */
size_t      sptgb_scan_tmp_bytes(uint64_t n);
cudaError_t sptgb_exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total,
                                     void *tmp, cudaStream_t s);
/* For each i with flags[i]: starts[pos[i]] = i. */
cudaError_t sptgb_compact_starts(const uint32_t *flags, const uint32_t *pos, uint64_t n, uint64_t *starts,
                                 cudaStream_t s);
/* For each i with flags[i]: out[pos[i]] = vals[i]. */
cudaError_t sptgb_compact_u32(const uint32_t *flags, const uint32_t *pos, const uint32_t *vals, uint64_t n,
                              uint32_t *out, cudaStream_t s);
/* *unsorted (device) = 1 when v is not non-decreasing. */
cudaError_t sptgb_check_sorted(const uint32_t *v, uint64_t n, unsigned int *unsorted, cudaStream_t s);
/* *bad (device) = 1 when some inds[m][i] >= lims[m] (null inds[m] skipped). */
cudaError_t sptgb_check_bounds(const uint32_t *const *inds, const uint32_t *lims, int nmodes, uint64_t n,
                               unsigned int *bad, cudaStream_t s);
/* HiCOO element split: einds[m][i] = inds[m][i] & ((1<<sb)-1) and, at block
 * starts, binds[m][b] = inds[m][i] >> sb. */
cudaError_t sptgb_hicoo_split(const uint32_t *const *inds, int nmodes, int sb_bits, uint64_t n,
                              const uint32_t *bflags, const uint32_t *bpos,
                              uint8_t *const *einds, uint32_t *const *binds, cudaStream_t s);

typedef struct {
    const uint64_t *bptr;                      /* [nb+1] */
    const uint32_t *binds[SPTGB_MAX_MODES];
    const uint8_t  *einds[SPTGB_MAX_MODES];
    const float    *vals;
    const float    *fac[SPTGB_MAX_MODES];      /* all factor matrices, by mode */
    float          *out;
    uint64_t        nb;
    uint32_t        out_rows;
    uint32_t        nmodes;
    uint32_t        mode;
    uint32_t        order[SPTGB_MAX_MODES];    /* mats_order */
    uint32_t        rank;
    uint32_t        stride;
    uint32_t        sb_bits;
    uint32_t        ndims[SPTGB_MAX_MODES];    /* elements outside are skipped and flagged */
    unsigned int   *err;                       /* device flag, set to 1 on an out-of-range element */
    /* output-window schedule of `mode` (sptgb_hicoo_schedule); perm == NULL
     * runs the block-parallel kernel with per-row atomics instead */
    const uint32_t *perm;                      /* [nb] blocks ordered by binds[mode] (stable) */
    const uint32_t *pnnz;                      /* [nb+1] exclusive prefix of block sizes in that order */
    const uint64_t *wst;                       /* [nwin+1] first position of each output window; wst[nwin] = nb */
    uint32_t        nwin;
    const uint64_t *heavy;                     /* [nheavy] ascending ids of the windows holding at least
                                                  heavy_nnz nonzeros (order 3) */
    uint32_t        nheavy;
    uint32_t        heavy_nnz;                 /* sptgb_hicoo_heavy_nnz(nnz) */
    uint64_t        nnz;                       /* = bptr[nb]; below 2^32 for the window kernel */
} sptgb_hicoo_args;
cudaError_t sptgb_mttkrp_hicoo(const sptgb_hicoo_args *a, cudaStream_t s);
/* *a->err = 1 when an element lies outside its mode or its element offset is
 * not below 2^sb_bits (a->bptr, binds, einds, ndims, nmodes, nb used). */
cudaError_t sptgb_hicoo_check(const sptgb_hicoo_args *a, cudaStream_t s);
/* *bad = 1 unless bptr[0] == 0, bptr[nb] == nnz and bptr is non-decreasing
 * (nb = 0: *bad = 0). */
cudaError_t sptgb_hicoo_check_bptr(const uint64_t *bptr, uint64_t nb, uint64_t nnz, unsigned int *bad,
                                   cudaStream_t s);
/* Output-window schedule of one mode: blocks stably sorted by their block
 * index in `mode` (keys = binds_mode, window_bits significant bits), the
 * prefix of their sizes, the start of each run of equal keys (a window) and
 * the ascending list of windows with at least heavy_nnz nonzeros (heavy, [nb]
 * capacity).  Scratch: keys/vals double buffers [nb] each, radix tmp,
 * flags/pos [nb], scan tmp.  *nwin_out and *nheavy_out are read back (the
 * stream is synchronised).  nnz < 2^32. */
#define SPTGB_HICOO_HEAVY_MIN 8192u
#define SPTGB_HICOO_HEAVY_DIV 32u
/* Order-3 window kernel: a window of 2^sb output rows holding at least this
 * many nonzeros is summed in the shared-memory tile and written once; the
 * rows of lighter windows go to the output with global vector atomics.  Only
 * a window that holds a large share of the whole tensor (a power-law mode's
 * head) puts enough atomics on a few rows to need the tile: on a 100M-nonzero
 * tensor with two Zipf(1.2) modes the global atomics were faster for every
 * window below a few million nonzeros. */
static inline uint32_t sptgb_hicoo_heavy_nnz(uint64_t nnz) {
    const uint64_t h = nnz / SPTGB_HICOO_HEAVY_DIV;
    return h < SPTGB_HICOO_HEAVY_MIN ? SPTGB_HICOO_HEAVY_MIN : h > 0xffffffffull ? 0xffffffffu : (uint32_t)h;
}
typedef struct {
    uint32_t *keys[2], *vals[2], *flags, *pos;
    void *rtmp, *stmp;
} sptgb_hicoo_sched_scratch;
cudaError_t sptgb_hicoo_schedule(const uint32_t *binds_mode, const uint64_t *bptr, uint64_t nb, int window_bits,
                                 uint32_t heavy_nnz, const sptgb_hicoo_sched_scratch *w, uint32_t *perm, uint32_t *pnnz, uint64_t *wst,
                                 uint32_t *nwin_out, uint64_t *heavy, uint32_t *nheavy_out, cudaStream_t s);

/* ---------------------------------------------------- dense CP-ALS --
 * FP64 pieces; matrices are row-major with `stride` floats per row. */
typedef struct {
    int      rank;
    int      stride;
    double  *ws;        /* device workspace, sptgb_dense_ws_bytes() */
} sptgb_dense_ctx;
/* Blocks of the dense reductions (Grams, norms, fit terms, ||X||^2): a fixed
 * count, two per SM of a GB300, so the partial sums and the order in which
 * they are combined do not depend on the device; workspaces hold this many
 * partials. */
#define SPTGB_NPART 304
size_t      sptgb_dense_ws_bytes(int rank, int max_blocks);
/* G = A^T A in FP64 (full symmetric) over rows [0, nrows). */
cudaError_t sptgb_gram(const float *A, uint32_t nrows, int rank, int stride, double *G, double *ws,
                       cudaStream_t s);
/* Builds H = Hadamard of grams[m] for m != mode (grams: host array of
 * device pointers), factorises it (Cholesky, or LU with partial pivoting
 * when H is not SPD) and writes S = (H^{-1})^T to Hinv.
 * status (device int): bits 0-7 = 0 Cholesky, 1 LU fallback, 2 singular;
 * bits 8 and up = e, the inverse stored divided by 2^e (e > 0 only when its
 * largest entry exceeds 2^32). */
cudaError_t sptgb_solve_prepare(const double *const *grams, int nmodes, int mode, int rank,
                                double *Hinv, int *status, cudaStream_t s);
/* X[i,:] solves H x = M[i,:] for i < nrows (FP64 arithmetic, FP32
 * storage) given S = (H^{-1})^T and the status word sptgb_solve_prepare
 * wrote with it (its scale exponent); leaves per-block partials of X^T X and
 * of the column maxima in ws for sptgb_normalize.  X must not alias M. */
cudaError_t sptgb_solve_rows(const float *M, float *X, uint32_t nrows, int rank, int stride,
                             const double *S, const int *status, double *ws, cudaStream_t s);
/* lambda from those partials (2-norm when use_2norm, else the column maximum
 * clamped to >= 1, matrix.c:390-554), X's columns divided by lambda, and
 * gram = the Gram matrix of the normalised X. */
cudaError_t sptgb_normalize(float *X, uint32_t nrows, int rank, int stride, double *gram,
                            int use_2norm, float *lambda_f32, const double *ws, cudaStream_t s);
/* <X, K> = sum_r lambda_r sum_i A[i,r] M[i,r] and ||K||^2 from the Grams
 * (grams: host array of device pointers); writes the fit into *fit_out
 * given normX2 (device double). */
cudaError_t sptgb_fit(const float *A, const float *M, uint32_t nrows, int rank, int stride,
                      const float *lambda, const double *const *grams, int nmodes,
                      const double *normX2, double *fit_out, double *ws, cudaStream_t s);
/* sum of squares of values in FP64. */
cudaError_t sptgb_sumsq(const float *v, uint64_t n, double *out, double *ws, cudaStream_t s);
/* Column 2-norms of A (FP64 accumulate) into lambda (float) and A /= lambda
 * (GetFinalLambda multiplies these into the running lambda). */
cudaError_t sptgb_colnorm_scale(float *A, uint32_t nrows, int rank, int stride, float *lambda_mul,
                                double *ws, cudaStream_t s);

/* ------------------------------------------------------ text ingest --
 * Token-parallel parse of a whitespace-separated tensor body (ingest.cu). */
typedef struct {
    uint32_t nmodes, start_index;
    uint64_t max_records;
    uint32_t *inds[SPTGB_MAX_MODES];   /* [max_records] each, index - start_index */
    float *vals;                       /* [max_records] */
    uint64_t *first_bad;               /* device: smallest invalid token (init ~0) */
    uint64_t *first_below;             /* device: smallest index token below start_index (init ~0) */
    uint64_t *nslow;                   /* device: values left to the host parser */
    uint64_t slow_cap;
    uint64_t *slow_rec, *slow_off;     /* [slow_cap]: record and byte offset (from base_off) */
    uint64_t base_off;                 /* byte offset of this chunk in the body */
} sptgb_ingest_out;
/* Token starts of buf[0, n): starts[0, *ntok) (device count). */
cudaError_t sptgb_ingest_token_starts(const void *buf, uint64_t n, uint32_t *flags, uint32_t *pos, uint32_t *ntok,
                                      void *scan_tmp, uint64_t *starts, cudaStream_t s);
cudaError_t sptgb_ingest_parse(const void *buf, uint64_t n, const uint64_t *starts, uint64_t ntok, uint64_t base_tok,
                               const sptgb_ingest_out *o, cudaStream_t s);
/* Sum of vals[starts[g] .. starts[g+1]) in order for each group g < ng
 * (starts[ng] = n), into out[g]. */
cudaError_t sptgb_segment_sums(const uint64_t *starts, uint64_t ng, uint64_t n, const float *vals, float *out,
                               cudaStream_t s);

/* ------------------------------------------------- batched CP-ALS --
 * Device descriptor of one tensor ("slot") of a batch, written once at
 * admission.  Records for mode m are 16-byte {row, a, b, value} (order 3) or
 * {row, a, b, c} with the value in val4[m] (order 4), a < b < c the other
 * modes, grouped by row (stable in the submitted order within a row).
 * status[0..3]: solve status per mode; status[4]: iterations completed. */
typedef struct {
    uint32_t nmodes, rank, stride, pad_;
    uint32_t ndims[4];
    uint64_t nnz;
    const void *rec[4];
    const float *val4[4];
    float *fac[4];
    float *M;
    double *gram[4];
    double *S;
    float *lambda;
    double *ws;
    double *fits;
    double *normX2;
    int *status;
} sptgb_slot;

/* A work list: count active entries (device u32), their slot ids and the
 * exclusive prefix of work items per entry (pre[count] = total items). */
typedef struct {
    const uint32_t *count;
    const uint32_t *ids;
    const uint64_t *pre;
} sptgb_wlist;

/* One ALS iteration of every listed slot, as a fixed kernel sequence (graph
 * capturable: all sizes are read from device memory).  mt[m][g]: MTTKRP unit
 * lists of mode m for lane group g (W = 2, 4, 8, 16); dn[m]: slots with more
 * than m modes, items = solve row blocks (any count in [1, NBLK]: each block
 * leaves one Gram partial); one[m]: the same slots in the same order, one item
 * each; zr[m]: row chunks to zero; fit: slots, items = fit blocks; fit_one:
 * the fit's slots in the same order, one item each. */
typedef struct {
    sptgb_wlist mt[4][4];
    uint32_t ul[4];     /* MTTKRP unit length per lane group */
    uint32_t sched[4];  /* MTTKRP schedule per lane group: bit 0 deep record batches, bit 1 the
                           3-blocks-per-SM build (the persistent step honours bit 0 only) */
    sptgb_wlist zr[4], one[4], dn[4], fit, fit_one;
} sptgb_step_lists;
cudaError_t sptgb_batch_step(const sptgb_slot *slots, const sptgb_step_lists *L, cudaStream_t s);
/* The same ALS iteration as ONE cooperative launch of a persistent kernel,
 * its phases separated by a grid barrier on *bar (zeroed once, device
 * memory; err set when a bounded barrier wait ran out).  cudaErrorNotSupported
 * when the device cannot launch cooperatively. */
typedef struct { unsigned int count, gen; int err, pad; } sptgb_grid_bar;
cudaError_t sptgb_batch_step_persistent(const sptgb_slot *slots, const sptgb_step_lists *L, sptgb_grid_bar *bar,
                                        cudaStream_t s);
/* The grid barrier of the persistent step on a 4-block grid: every round
 * completes (missing = 0) or the last round waits for one block too many and
 * every wait gives up (missing = 1); *err = the barrier's error word after the
 * launch, *rounds = rounds completed summed over blocks. */
cudaError_t sptgb_grid_barrier_selftest(int missing, int *err, unsigned int *rounds);
/* The MTTKRP launch of mode m, lane group g alone (for timing). */
cudaError_t sptgb_batch_mttkrp(const sptgb_slot *slots, const sptgb_wlist *w, int mode, int group, uint32_t ul,
                               uint32_t sched, cudaStream_t s);
/* Grid sizes the step uses, so that hosts size their prefix lists. */
uint32_t sptgb_batch_solve_tile_rows(uint32_t rank);   /* rows per row-solve tile at this rank */
uint32_t sptgb_batch_fit_rows_per_block(void);
uint32_t sptgb_batch_zero_rows(void);
uint32_t sptgb_batch_max_blocks(void);
/* Admission of a group of jobs.  Their nonzeros are staged back to back
 * (job j at [offs[j], offs[j+1])) in ind[m] / val, in the caller's order. */
typedef struct {
    uint64_t off, n;
    uint32_t slot, nmodes;
    uint32_t ndims[4];
} sptgb_adm_job;
typedef struct {
    const uint32_t *ind[4];
    const float *val;
    const uint64_t *offs;        /* [njobs + 1] */
    const sptgb_adm_job *jobs;   /* [njobs] */
    uint32_t njobs;
    uint64_t total;
    unsigned int *err;           /* [njobs]: set to 1 when a coordinate is out of range */
} sptgb_adm_group;
/* err[j] for every job with a coordinate >= its mode size. */
cudaError_t sptgb_adm_check(const sptgb_adm_group *g, cudaStream_t s);
/* keys[p] for q = perm ? perm[p] : p, j = job of q, row = ind[mode][q]
 * (0 for jobs of order <= mode):  kind 0: (j << rowbits) | row,
 * kind 1: row,  kind 2: j. */
cudaError_t sptgb_adm_keys(const sptgb_adm_group *g, int mode, int rowbits, int kind, const uint32_t *perm,
                           uint32_t *keys, cudaStream_t s);
/* Writes the mode-`mode` records (and order-4 values) of every job of order
 * > mode into its slot, from the (job, row)-sorted permutation perm. */
cudaError_t sptgb_adm_pack(const sptgb_adm_group *g, const sptgb_slot *slots, int mode, const uint32_t *perm,
                           cudaStream_t s);
/* ||X||^2 per job (sq: job ids, items = sum-of-squares blocks; one: same
 * jobs, one item each), also clears status and sets lambda to 1. */
cudaError_t sptgb_adm_normsq(const sptgb_slot *slots, const sptgb_adm_group *g, const sptgb_wlist *sq,
                             const sptgb_wlist *one, cudaStream_t s);
/* Gram of factor `mode` per listed slot (dn: slot ids, items = row blocks;
 * one: same slots, one item each). */
cudaError_t sptgb_batch_gram(const sptgb_slot *slots, const sptgb_wlist *dn, const sptgb_wlist *one, int mode,
                             cudaStream_t s);
/* GetFinalLambda of factor `mode` per listed slot (dn: items = column-norm
 * blocks; one: one item each). */
cudaError_t sptgb_batch_final_lambda(const sptgb_slot *slots, const sptgb_wlist *dn, const sptgb_wlist *one,
                                     int mode, cudaStream_t s);
/* Block counts the single-tensor kernels use, for identical partial sums. */
uint32_t sptgb_sumsq_blocks(uint64_t n);
uint32_t sptgb_colnorm_blocks(uint32_t nrows);
uint32_t sptgb_gram_blocks(uint32_t nrows);


/* ------------------------------------------------- BF16 conversion -- */
cudaError_t sptgb_f32_to_bf16(const float *in, uint16_t *out, uint64_t n, cudaStream_t s);

#ifdef __cplusplus
}
#endif

#endif
