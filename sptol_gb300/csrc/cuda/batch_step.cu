// The batched CP-ALS step as ONE persistent cooperative launch: every phase of
// batch_phases.cuh (per mode: zero, MTTKRP of the four lane groups, prepare,
// solve, lambda, scale; then the fit) runs in turn over the same resident
// grid, the phases separated by a grid barrier, instead of the ~38 launches of
// the kernel sequence (batch.cu).  Same work lists, same per-slot items, so
// the arithmetic is the sequence's; only the launch count changes.  Opt-in
// (SPTGB_STEP=persistent): every phase runs with the solve's shared-memory
// allocation, which leaves the gather-bound MTTKRP phase a small L1, and the
// grid fills every SM, so admission kernels cannot overlap it; on GB300 the
// sequence is faster for served streams.
//
// Every phase reads what an earlier phase of this launch wrote (the MTTKRP
// output, the inverse, the new factor rows, lambda, the Gram and fit
// partials), so no load of this unit may take the read-only (non-coherent)
// path: the bodies are compiled without __restrict__ on their operands and
// the factor rows are gathered with coherent loads.  Only the sorted records
// and values, which no phase writes, keep the read-only path.
#define SPTGB_RESTRICT
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "batch_phases.cuh"

namespace {

using namespace sptgb_dense;
using namespace sptgb_batch;

// Grid barrier: block leaders count arrivals on bar->count; the last one
// resets the count and advances bar->gen, the others wait for gen to move.
// The wait is bounded: a block that gives up (after BAR_SPINS polls, about a
// second or more) or that sees bar->err set marks bar->err and returns false,
// and every other block gives up at its own next wait, so a broken launch ends
// with the error reported to the host instead of hanging the device.  Every
// thread fences after the barrier so that the writes of the phase before it
// are visible to the loads of the phase after it.
constexpr uint32_t BAR_SPINS = 1u << 23;

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// `arrivals`: blocks that must arrive (the grid; the self-test asks for one
// more than it launches so that the wait runs out).
__device__ __forceinline__ bool grid_sync(sptgb_grid_bar *bar, uint32_t arrivals = 0, uint32_t max_spins = BAR_SPINS) {
    __shared__ int s_ok;
    if (arrivals == 0) arrivals = gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int gen = ld_acquire(&bar->gen);
        __threadfence();
        int ok = 1;
        if (atomicAdd(&bar->count, 1u) + 1u == arrivals) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            uint32_t spins = 0;
            while (ld_acquire(&bar->gen) == gen) {
                if (++spins > max_spins || ld_relaxed(&bar->err) != 0) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        if (!ok) atomicOr(&bar->err, 1);
        s_ok = ok;
    }
    __syncthreads();
    __threadfence();
    return s_ok != 0;
}

// The phases as separate functions: each gets its own register allocation
// instead of the union of all of them.
__device__ __noinline__ void pz(const sptgb_slot *sl, const sptgb_wlist w, int m) { ph_zero(sl, w, m); }
template <int W, bool DEEP>
__device__ __noinline__ void pm(const sptgb_slot *sl, const sptgb_wlist w, int m, uint32_t ul) {
    ph_mttkrp<W, true, DEEP>(sl, w, m, ul);
}
template <int W>
__device__ __forceinline__ void pm_sched(const sptgb_slot *sl, const sptgb_wlist &w, int m, uint32_t ul,
                                         uint32_t sched) {
    if (sched & 1u) pm<W, true>(sl, w, m, ul);
    else pm<W, false>(sl, w, m, ul);
}
__device__ __noinline__ void pp(const sptgb_slot *sl, const sptgb_wlist w, int m) { ph_prepare(sl, w, m); }
__device__ __noinline__ void ps(const sptgb_slot *sl, const sptgb_wlist w, int m) { ph_solve(sl, w, m); }
__device__ __noinline__ void pl(const sptgb_slot *sl, const sptgb_wlist w, const sptgb_wlist p, int m) {
    ph_lambda(sl, w, p, m);
}
__device__ __noinline__ void pc(const sptgb_slot *sl, const sptgb_wlist w, int m) { ph_scale(sl, w, m); }
__device__ __noinline__ void pf(const sptgb_slot *sl, const sptgb_wlist w) { ph_fit_partial(sl, w); }
__device__ __noinline__ void pg(const sptgb_slot *sl, const sptgb_wlist w, const sptgb_wlist p) {
    ph_fit_final(sl, w, p);
}

__global__ void __launch_bounds__(BT, 2) k_b_step(const sptgb_slot *__restrict__ slots, sptgb_step_lists L,
                                                 sptgb_grid_bar *bar) {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        pz(slots, L.zr[m], m);
        if (!grid_sync(bar)) return;
        pm_sched<2>(slots, L.mt[m][0], m, L.ul[0], L.sched[0]);
        pm_sched<4>(slots, L.mt[m][1], m, L.ul[1], L.sched[1]);
        pm_sched<8>(slots, L.mt[m][2], m, L.ul[2], L.sched[2]);
        pm_sched<16>(slots, L.mt[m][3], m, L.ul[3], L.sched[3]);
        if (!grid_sync(bar)) return;
        pp(slots, L.one[m], m);
        if (!grid_sync(bar)) return;
        ps(slots, L.dn[m], m);
        if (!grid_sync(bar)) return;
        pl(slots, L.one[m], L.dn[m], m);
        if (!grid_sync(bar)) return;
        pc(slots, L.dn[m], m);
        if (!grid_sync(bar)) return;
    }
    pf(slots, L.fit);
    if (!grid_sync(bar)) return;
    pg(slots, L.fit_one, L.fit);
}

// The barrier on a small grid: two rounds that every block reaches, then
// (when `missing` is set) a round that waits for one block more than the grid
// has, so that every wait runs out after `max_spins` polls and the kernel
// returns with bar->err set instead of hanging.
__global__ void k_bar_selftest(sptgb_grid_bar *bar, int missing, uint32_t max_spins, unsigned int *rounds) {
    for (int r = 0; r < 2; ++r) {
        if (!grid_sync(bar, 0, max_spins)) return;
        if (threadIdx.x == 0) atomicAdd(rounds, 1u);
    }
    if (missing) {
        if (!grid_sync(bar, gridDim.x + 1, max_spins)) return;
        if (threadIdx.x == 0) atomicAdd(rounds, 1u);
    }
}

// Resident blocks of k_b_step (< 0: cooperative launch unsupported), sized on
// first use; a function-local static is initialised by one thread while the
// others wait.
int step_blocks() {
    static const int blocks = [] {
        int dev = 0, coop = 0, per = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop &&
            cudaFuncSetAttribute(k_b_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOLVE_SMEM) ==
                cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_b_step, BT, SOLVE_SMEM) == cudaSuccess && per >= 1)
            return (per < 2 ? per : 2) * sptgb_sm_count();
        cudaGetLastError();
        return -1;
    }();
    return blocks;
}

}  // namespace

// Sized once: every block of a cooperative launch must be resident at once,
// so the grid is (blocks per SM, at most 2) x SMs; the runtime refuses a
// cooperative launch that does not fit rather than running it.
extern "C" cudaError_t sptgb_batch_step_persistent(const sptgb_slot *slots, const sptgb_step_lists *L,
                                                   sptgb_grid_bar *bar, cudaStream_t s) {
    const int blocks = step_blocks();
    if (blocks < 0) return cudaErrorNotSupported;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(BT);
    cfg.dynamicSmemBytes = SOLVE_SMEM;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_b_step, slots, *L, bar);
    sptgb_count_launch(1);
    return e;
}

// Runs k_bar_selftest on 4 blocks of 64 threads (a cooperative launch, so all
// blocks are resident) with a bound of 2^14 polls per wait; *err = bar->err
// after the launch, *rounds = barrier rounds completed, summed over blocks.
extern "C" cudaError_t sptgb_grid_barrier_selftest(int missing, int *err, unsigned int *rounds) {
    struct scratch {
        sptgb_grid_bar bar;
        unsigned int rounds;
    } *d = nullptr, h;
    cudaError_t e = cudaMalloc((void **)&d, sizeof *d);
    if (e != cudaSuccess) return e;
    e = cudaMemset(d, 0, sizeof *d);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(4);
    cfg.blockDim = dim3(64);
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, k_bar_selftest, &d->bar, missing, 1u << 14, &d->rounds);
    if (e == cudaSuccess) sptgb_count_launch(1);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return e;
    *err = h.bar.err;
    *rounds = h.rounds;
    return cudaSuccess;
}
