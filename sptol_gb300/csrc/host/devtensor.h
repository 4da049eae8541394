/* Host-side helpers shared by the drop-in entry points (the .c files of csrc/host). */
#ifndef SPTGB_DEVTENSOR_H
#define SPTGB_DEVTENSOR_H

#include <pthread.h>
#include "../sptgb_internal.h"
#include "../../../include/sptgb.h"

/* Grow-only device buffers reused by every host-buffer call; one lock
 * serialises those calls (the reference's CUDA path is not re-entrant
 * either, src/sptensor/mttkrp_cuda_onekernel.cu). */
typedef struct {
    pthread_mutex_t lock;
    sptgb_dbuf inds[SPTGB_MAX_MODES], vals;
    sptgb_dbuf sinds[SPTGB_MAX_MODES], svals;
    sptgb_dbuf keys[2], perm[2], rtmp;
    sptgb_dbuf fac[SPTGB_MAX_MODES], out;
    sptgb_dbuf flag, misc[8];
    unsigned int *hflag;            /* pinned, 16 words: flags and row numbers read back without
                                       blocking the host */
    cudaEvent_t ev[4];              /* ordering between the compute and the copy stream */
    cudaEvent_t cev[8];             /* one per output chunk of a host-buffer MTTKRP */
} sptgb_workspace;
extern sptgb_workspace g_ws;

/* SPTGB_TRACE=1 prints the wall time of each phase of a host-buffer call to
 * stderr (the reference prints its H2D / kernel / D2H times the same way,
 * src/sptensor/mttkrp_cuda_onekernel.cu:151-155, :381-404); a trace point
 * synchronises the stream first. */
int    sptgb_trace_on(void);
double sptgb_wall(void);
#define SPTGB_TRACE_POINT(name, stream, t_prev)                                          \
    do {                                                                                 \
        if (sptgb_trace_on()) {                                                          \
            cudaStreamSynchronize(stream);                                               \
            const double _t = sptgb_wall();                                              \
            fprintf(stderr, "[sptgb trace] %-10s %8.3f ms\n", name, (_t - (t_prev)) * 1e3); \
            (t_prev) = _t;                                                               \
        }                                                                                \
    } while (0)

void sptgb_lock(void);
/* Pinned flag words and the two events above, created on first use (lock held). */
int  sptgb_ws_sync_objects(void);
void sptgb_unlock(void);
int  sptgb_quiet(void);
int  sptgb_bitwidth(uint64_t x);

/* One stable radix pass group: kind/mode/shift/slice as sptgb_keyspec,
 * `bits` significant key bits (0 = skip). */
typedef struct { int kind, mode, shift, slice, bits; } sptgb_sortpass;

int sptgb_lex_passes(const sptIndex *ndims, const sptIndex *order, int nmodes, sptgb_sortpass *passes);
int sptgb_hicoo_passes(const sptIndex *ndims, int nmodes, int sk_bits, int with_kernels, sptgb_sortpass *passes);
int sptgb_sort_perm(uint32_t *const *d_inds, int nmodes, uint64_t n, const sptgb_sortpass *passes, int npasses,
                    uint32_t **perm_out, cudaStream_t s);
int sptgb_gather_tensor(uint32_t *const *src_inds, const float *src_vals, uint32_t *const *dst_inds, float *dst_vals,
                        int nmodes, const uint32_t *perm, uint64_t n, cudaStream_t s);
int sptgb_upload_tensor(const sptSparseTensor *X, sptgb_dbuf *inds, sptgb_dbuf *vals, const int *need,
                        cudaStream_t s);
/* Checks every coordinate against its mode size and, when sorted_check is
 * given, whether that array is non-decreasing (*unsorted_out).  Syncs. */
int sptgb_validate(uint32_t *const *d_inds, const sptIndex *ndims, int nmodes, uint64_t n,
                   const uint32_t *sorted_check, int *unsorted_out, cudaStream_t s);

struct sptgbCoo {
    sptIndex nmodes;
    sptIndex ndims[SPTGB_MAX_MODES];
    uint64_t nnz;
    uint32_t *inds[SPTGB_MAX_MODES];
    float *vals;
    int ready[SPTGB_MAX_MODES];
    uint32_t *minds[SPTGB_MAX_MODES][SPTGB_MAX_MODES];
    float *mvals[SPTGB_MAX_MODES];
    void *mrec[SPTGB_MAX_MODES];   /* orders 3 and 4: 16-byte records of the mode copy */
    size_t bytes;
    int timing;
    cudaEvent_t ev0, ev1;
    float last_ms;
};

struct sptgbHicoo {
    sptIndex nmodes;
    sptIndex ndims[SPTGB_MAX_MODES];
    uint64_t nnz, nb;
    int sb_bits;
    uint64_t *bptr;
    uint32_t *binds[SPTGB_MAX_MODES];
    uint8_t *einds[SPTGB_MAX_MODES];
    float *vals;
    /* output-window schedule per mode (orders 3 and 4) */
    uint32_t *perm[SPTGB_MAX_MODES], *pnnz[SPTGB_MAX_MODES];
    uint64_t *wst[SPTGB_MAX_MODES];    /* [nb+1] window starts, then [nb] heavy window ids */
    uint32_t nwin[SPTGB_MAX_MODES], nheavy[SPTGB_MAX_MODES];
    int ready[SPTGB_MAX_MODES];
    unsigned int *err;
    size_t bytes;
};

#endif
