// Batched CP-ALS: one ALS iteration for every tensor ("slot") of a batch as a
// fixed sequence of kernels, one per phase of batch_phases.cuh, plus the
// admission kernels that pack a group of jobs into slots.  (batch_step.cu runs
// the same phases as one persistent launch.)
//
// Each kernel walks a work list in device memory with a fixed grid.  Sizes are
// read on the device, so the host can change which slots are listed between
// launches without touching the launch parameters, and the whole step can be
// captured once in a CUDA graph and replayed.
//
// Per mode m (slots with fewer modes are simply not listed):
//   zero      rows of the slot's MTTKRP output
//   mttkrp    one launch per lane group W in {2,4,8,16} (rank <= 8, 16, 32,
//             64), work items = 'ul'-nonzero units, same unit body as the
//             single-tensor kernel (mttkrp_unit.cuh)
//   prepare   one block per slot: Hadamard of the other Grams, FP64
//             Cholesky / LU, inverse (dense_common.cuh)
//   solve     row blocks: rows solved in FP64, Gram and column-max partials
//   lambda    one block per slot: 2-norm at the slot's first iteration, else
//             max-norm, normalised Gram
//   scale     row blocks: columns divided by lambda
// then the fit (inner-product partials, final) and the slot's iteration
// counter.  The per-slot decomposition into blocks is the single-tensor one,
// so a slot computes the same arithmetic alone, in a batch, or through
// sptgbCpdAls.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "batch_phases.cuh"

namespace {

using namespace sptgb_dense;
using namespace sptgb_batch;

// The step's kernels: each phase as its own launch ...
__global__ void k_b_zero(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) { ph_zero(slots, w, mode); }
// MINB: resident blocks per SM the registers are sized for (2: 128
// registers a thread, 3: 80).
template <int W, bool DEEP, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_b_mttkrp(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode,
                                                      uint32_t ul) {
    ph_mttkrp<W, false, DEEP>(slots, w, mode, ul);
}
__global__ void __launch_bounds__(DT) k_b_prepare(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    ph_prepare(slots, w, mode);
}
__global__ void __launch_bounds__(DT, 2) k_b_solve(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    ph_solve(slots, w, mode);
}
__global__ void k_b_lambda(const sptgb_slot *__restrict__ slots, sptgb_wlist w, sptgb_wlist parts, int mode) {
    ph_lambda(slots, w, parts, mode);
}
__global__ void k_b_scale(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) { ph_scale(slots, w, mode); }
__global__ void __launch_bounds__(DT) k_b_fit_partial(const sptgb_slot *__restrict__ slots, sptgb_wlist w) {
    ph_fit_partial(slots, w);
}
__global__ void k_b_fit_final(const sptgb_slot *__restrict__ slots, sptgb_wlist w, sptgb_wlist parts) {
    ph_fit_final(slots, w, parts);
}

// ------------------------------------------------------------ admission --
// Last job j with offs[j] <= i.
__device__ __forceinline__ uint32_t job_of(const uint64_t *offs, uint32_t njobs, uint64_t i) {
    uint32_t lo = 0, hi = njobs;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offs[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_adm_check(sptgb_adm_group g) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < g.total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = job_of(g.offs, g.njobs, i);
        const sptgb_adm_job &jb = g.jobs[j];
        bool bad = false;
        for (uint32_t m = 0; m < jb.nmodes && m < 4; ++m) bad |= g.ind[m][i] >= jb.ndims[m];
        if (bad) g.err[j] = 1u;
    }
}

__global__ void k_adm_keys(sptgb_adm_group g, int mode, int rowbits, int kind, const uint32_t *__restrict__ perm,
                           uint32_t *__restrict__ keys) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < g.total;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t q = perm ? perm[p] : p;
        const uint32_t j = job_of(g.offs, g.njobs, q);
        const uint32_t row = g.jobs[j].nmodes > (uint32_t)mode ? g.ind[mode][q] : 0u;
        keys[p] = kind == 0 ? ((j << rowbits) | row) : kind == 1 ? row : j;
    }
}

__global__ void k_adm_pack(sptgb_adm_group g, const sptgb_slot *__restrict__ slots, int mode,
                           const uint32_t *__restrict__ perm) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < g.total;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t j = job_of(g.offs, g.njobs, p);   // sorted by job: same job as perm[p]
        const sptgb_adm_job &jb = g.jobs[j];
        if (jb.nmodes <= (uint32_t)mode) continue;
        const sptgb_slot &s = slots[jb.slot];
        const uint64_t q = perm[p];
        const uint64_t k = p - g.offs[j];
        const uint32_t o0 = 0 + (0 >= mode), o1 = 1 + (1 >= mode), o2 = 2 + (2 >= mode);
        uint4 r;
        r.x = g.ind[mode][q];
        r.y = g.ind[o0][q];
        r.z = g.ind[o1][q];
        const float v = g.val[q];
        if (jb.nmodes == 3) {
            r.w = __float_as_uint(v);
        } else {
            r.w = g.ind[o2][q];
            const_cast<float *>(s.val4[mode])[k] = v;
        }
        static_cast<uint4 *>(const_cast<void *>(s.rec[mode]))[k] = r;
    }
}

__global__ void __launch_bounds__(DT) k_adm_sumsq_partial(const sptgb_slot *__restrict__ slots, sptgb_adm_group g,
                                                          sptgb_wlist w) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, it);
        const sptgb_adm_job &jb = g.jobs[w.ids[e]];
        const sptgb_slot &s = slots[jb.slot];
        sumsq_partial_body(g.val + jb.off, jb.n, s.ws, (unsigned)(it - w.pre[e]), (unsigned)(w.pre[e + 1] - w.pre[e]));
        __syncthreads();
    }
}

__global__ void k_adm_sum_final(const sptgb_slot *__restrict__ slots, sptgb_adm_group g, sptgb_wlist w,
                                sptgb_wlist parts) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[g.jobs[w.ids[e]].slot];
        sum_final_body(s.ws, (int)(parts.pre[e + 1] - parts.pre[e]), s.normX2);
        for (uint32_t r = threadIdx.x; r < s.rank; r += blockDim.x) s.lambda[r] = 1.0f;
        if (threadIdx.x < 5) s.status[threadIdx.x] = 0;
    }
}

__global__ void __launch_bounds__(DT) k_b_gram_partial(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, it);
        const sptgb_slot &s = slots[w.ids[e]];
        gram_partial_body(s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride, s.ws, (unsigned)(it - w.pre[e]),
                          (unsigned)(w.pre[e + 1] - w.pre[e]));
        __syncthreads();
    }
}

__global__ void __launch_bounds__(DT) k_b_gram_reduce(const sptgb_slot *__restrict__ slots, sptgb_wlist w,
                                                      sptgb_wlist parts, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        gram_reduce_body(s.ws, (int)(parts.pre[e + 1] - parts.pre[e]), (int)s.rank, s.gram[mode]);
        __syncthreads();
    }
}

// ----------------------------------------------------------- retirement --
__global__ void __launch_bounds__(DT) k_b_colsq_partial(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, it);
        const sptgb_slot &s = slots[w.ids[e]];
        colsq_partial_body(s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride, s.ws, (unsigned)(it - w.pre[e]),
                           (unsigned)(w.pre[e + 1] - w.pre[e]));
        __syncthreads();
    }
}

__global__ void k_b_colnorm_final(const sptgb_slot *__restrict__ slots, sptgb_wlist w, sptgb_wlist parts, int mode) {
    const uint32_t cnt = *w.count;
    for (uint32_t e = blockIdx.x; e < cnt; e += gridDim.x) {
        const sptgb_slot &s = slots[w.ids[e]];
        colnorm_final_body(s.ws, (int)(parts.pre[e + 1] - parts.pre[e]), (int)s.rank, s.lambda,
                           reinterpret_cast<float *>(s.ws + (size_t)NBLK * s.rank));
    }
}

__global__ void k_b_scale_norms(const sptgb_slot *__restrict__ slots, sptgb_wlist w, int mode) {
    const uint32_t cnt = *w.count;
    if (cnt == 0) return;
    const uint64_t total = w.pre[cnt];
    for (uint64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const uint32_t e = find_entry(w.pre, cnt, it);
        const sptgb_slot &s = slots[w.ids[e]];
        scale_cols_body(s.fac[mode], s.ndims[mode], (int)s.rank, (int)s.stride,
                        reinterpret_cast<const float *>(s.ws + (size_t)NBLK * s.rank), (unsigned)(it - w.pre[e]),
                        (unsigned)(w.pre[e + 1] - w.pre[e]));
    }
}

unsigned grid_for(uint64_t n, unsigned cap) {
    uint64_t b = (n + 255) / 256;
    if (b > cap) b = cap;
    return b ? (unsigned)b : 1u;
}

int g_mt_blocks[4][2][2];   // [group][deep][occupancy 2 / 3]: grid of each MTTKRP kernel

template <int W, bool DEEP, int MINB>
void size_mttkrp(int g, int n) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_mttkrp<W, DEEP, MINB>, BT, 0);
    g_mt_blocks[g][DEEP][MINB - 2] = (per < 1 ? 1 : per) * n;
}
template <int W>
void size_group(int g, int n) {
    size_mttkrp<W, false, 2>(g, n);
    size_mttkrp<W, true, 2>(g, n);
    size_mttkrp<W, false, 3>(g, n);
    size_mttkrp<W, true, 3>(g, n);
}

// SM count; the first call also sets the kernels' shared-memory limits and
// sizes the MTTKRP grids.  A function-local static is initialised by one
// thread while the others wait, so no caller sees the grids half sized.
int nsm() {
    static const int n = [] {
        const int c = sptgb_sm_count();
        cudaFuncSetAttribute(k_b_prepare, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PREP_SMEM);
        cudaFuncSetAttribute(k_b_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOLVE_SMEM);
        size_group<2>(0, c);
        size_group<4>(1, c);
        size_group<8>(2, c);
        size_group<16>(3, c);
        return c;
    }();
    return n;
}

template <int W>
void launch_group(const sptgb_slot *slots, const sptgb_wlist &w, int mode, int g, uint32_t ul, uint32_t sched,
                  cudaStream_t s) {
    const bool deep = sched & 1u, occ3 = sched & 2u;
    const int blocks = g_mt_blocks[g][deep][occ3];
    if (deep && occ3) k_b_mttkrp<W, true, 3><<<blocks, BT, 0, s>>>(slots, w, mode, ul);
    else if (deep) k_b_mttkrp<W, true, 2><<<blocks, BT, 0, s>>>(slots, w, mode, ul);
    else if (occ3) k_b_mttkrp<W, false, 3><<<blocks, BT, 0, s>>>(slots, w, mode, ul);
    else k_b_mttkrp<W, false, 2><<<blocks, BT, 0, s>>>(slots, w, mode, ul);
}

// sched bit 0: deep record batches, bit 1: the 3-blocks-per-SM build
cudaError_t mttkrp_group(const sptgb_slot *slots, const sptgb_wlist &w, int mode, int group, uint32_t ul,
                         uint32_t sched, cudaStream_t s) {
    switch (group) {
        case 0: launch_group<2>(slots, w, mode, 0, ul, sched, s); break;
        case 1: launch_group<4>(slots, w, mode, 1, ul, sched, s); break;
        case 2: launch_group<8>(slots, w, mode, 2, ul, sched, s); break;
        default: launch_group<16>(slots, w, mode, 3, ul, sched, s); break;
    }
    sptgb_count_launch(1);
    return cudaGetLastError();
}

}  // namespace

extern "C" uint32_t sptgb_batch_solve_tile_rows(uint32_t rank) { return (uint32_t)solve_tile_rows((int)rank); }
extern "C" uint32_t sptgb_batch_fit_rows_per_block(void) { return FIT_ROWS; }
extern "C" uint32_t sptgb_batch_zero_rows(void) { return ZERO_ROWS; }
extern "C" uint32_t sptgb_batch_max_blocks(void) { return NBLK; }

extern "C" cudaError_t sptgb_batch_mttkrp(const sptgb_slot *slots, const sptgb_wlist *w, int mode, int group,
                                          uint32_t ul, uint32_t sched, cudaStream_t s) {
    nsm();
    return mttkrp_group(slots, *w, mode, group, ul, sched, s);
}

extern "C" cudaError_t sptgb_batch_step(const sptgb_slot *slots, const sptgb_step_lists *L, cudaStream_t s) {
    const int n = nsm();
    for (int m = 0; m < 4; ++m) {
        k_b_zero<<<n * 8, BT, 0, s>>>(slots, L->zr[m], m);
        sptgb_count_launch(1);
        for (int g = 0; g < 4; ++g) {
            cudaError_t e = mttkrp_group(slots, L->mt[m][g], m, g, L->ul[g], L->sched[g], s);
            if (e != cudaSuccess) return e;
        }
        k_b_prepare<<<n * 2, DT, PREP_SMEM, s>>>(slots, L->one[m], m);
        k_b_solve<<<n * 2, DT, SOLVE_SMEM, s>>>(slots, L->dn[m], m);
        k_b_lambda<<<n * 2, DT, 0, s>>>(slots, L->one[m], L->dn[m], m);
        k_b_scale<<<n * 8, 256, 0, s>>>(slots, L->dn[m], m);
        sptgb_count_launch(4);
    }
    k_b_fit_partial<<<n * 4, DT, 0, s>>>(slots, L->fit);
    k_b_fit_final<<<n * 2, DT, 0, s>>>(slots, L->fit_one, L->fit);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" uint32_t sptgb_sumsq_blocks(uint64_t n) {
    uint64_t b = (n + DT - 1) / DT;
    if (b > (uint64_t)NBLK) b = NBLK;
    return b ? (uint32_t)b : 1u;
}
extern "C" uint32_t sptgb_colnorm_blocks(uint32_t nrows) {
    uint32_t b = (nrows + 7) / 8;
    if (b > (uint32_t)NBLK) b = NBLK;
    return b ? b : 1u;
}
extern "C" uint32_t sptgb_gram_blocks(uint32_t nrows) { return (uint32_t)nblocks_for_rows(nrows); }

extern "C" cudaError_t sptgb_adm_check(const sptgb_adm_group *g, cudaStream_t s) {
    if (g->total == 0) return cudaSuccess;
    k_adm_check<<<grid_for(g->total, (unsigned)sptgb_sm_count() * 16), 256, 0, s>>>(*g);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_adm_keys(const sptgb_adm_group *g, int mode, int rowbits, int kind,
                                      const uint32_t *perm, uint32_t *keys, cudaStream_t s) {
    if (g->total == 0) return cudaSuccess;
    k_adm_keys<<<grid_for(g->total, (unsigned)sptgb_sm_count() * 16), 256, 0, s>>>(*g, mode, rowbits, kind, perm, keys);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_adm_pack(const sptgb_adm_group *g, const sptgb_slot *slots, int mode,
                                      const uint32_t *perm, cudaStream_t s) {
    if (g->total == 0) return cudaSuccess;
    k_adm_pack<<<grid_for(g->total, (unsigned)sptgb_sm_count() * 16), 256, 0, s>>>(*g, slots, mode, perm);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_adm_normsq(const sptgb_slot *slots, const sptgb_adm_group *g, const sptgb_wlist *sq,
                                        const sptgb_wlist *one, cudaStream_t s) {
    const int n = nsm();
    k_adm_sumsq_partial<<<n * 4, DT, 0, s>>>(slots, *g, *sq);
    k_adm_sum_final<<<n * 2, 64, 0, s>>>(slots, *g, *one, *sq);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_batch_gram(const sptgb_slot *slots, const sptgb_wlist *dn, const sptgb_wlist *one,
                                        int mode, cudaStream_t s) {
    const int n = nsm();
    k_b_gram_partial<<<n * 3, DT, 0, s>>>(slots, *dn, mode);
    k_b_gram_reduce<<<n * 2, DT, 0, s>>>(slots, *one, *dn, mode);
    sptgb_count_launch(2);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_batch_final_lambda(const sptgb_slot *slots, const sptgb_wlist *dn,
                                                const sptgb_wlist *one, int mode, cudaStream_t s) {
    const int n = nsm();
    k_b_colsq_partial<<<n * 4, DT, 0, s>>>(slots, *dn, mode);
    k_b_colnorm_final<<<n * 2, 64, 0, s>>>(slots, *one, *dn, mode);
    k_b_scale_norms<<<n * 8, 256, 0, s>>>(slots, *dn, mode);
    sptgb_count_launch(3);
    return cudaGetLastError();
}
