// Device sorting and segmentation primitives for the sparse-tensor orders.
//
// Every order the reference sorts by (lexicographic sptSparseTensorSortIndex,
// sptSparseTensorSortIndexCustomOrder, the row-block + Morton order of the
// HiCOO conversion; src/sptensor/sort.c:410-585, :629-995) is a total order on
// unique coordinates, so a STABLE least-significant-digit radix sort over the
// same key reproduces the reference's permutation exactly even though the
// reference's quicksort (sort.c:1166-1195) is unstable.  Keys longer than 32
// bits are sorted as a sequence of stable 32-bit key passes, least significant
// slice first, each slice recomputed from the coordinates through the current
// permutation.
//
// Radix pass structure (8-bit digits, 4096-element tiles):
//   upsweep   per-tile digit histogram       counts[digit][tile]
//   rowscan   one CTA per digit, exclusive    scan along tiles, digit totals
//   downsweep stable rank within the tile (warp __match_any_sync ranking,
//             warps own contiguous sub-ranges) and scatter.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr unsigned FULL = 0xffffffffu;

__global__ void __launch_bounds__(RS_THREADS)
rs_upsweep(const uint32_t *__restrict__ keys, uint64_t n, int shift, uint32_t *__restrict__ counts,
           uint32_t ntiles) {
    __shared__ uint32_t h[RS_WARPS][256];
    const int warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int i = 0; i < RS_ITEMS; ++i) {
        const uint64_t k = base + (uint64_t)i * RS_THREADS + threadIdx.x;
        if (k < n) atomicAdd(&h[warp][(keys[k] >> shift) & 255u], 1u);
    }
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) c += h[w][threadIdx.x];
    counts[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = c;
}

// Exclusive scan of one digit's row of per-tile counts; totals[digit] = sum.
__global__ void __launch_bounds__(1024)
rs_rowscan(uint32_t *__restrict__ counts, uint32_t ntiles, uint32_t *__restrict__ totals) {
    __shared__ uint32_t wsum[32];
    uint32_t *row = counts + (uint64_t)blockIdx.x * ntiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < ntiles; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < ntiles ? row[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, w, o);
                if (lane >= o) w += y;
            }
            wsum[lane] = w;
        }
        __syncthreads();
        const uint32_t incl = x + (warp ? wsum[warp - 1] : 0u);
        if (i < ntiles) row[i] = carry + incl - v;
        carry += wsum[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(RS_THREADS)
rs_downsweep(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout,
             uint32_t *__restrict__ vout, uint64_t n, int shift, const uint32_t *__restrict__ counts,
             const uint32_t *__restrict__ totals, uint32_t ntiles) {
    __shared__ uint32_t s_cnt[RS_WARPS][256];
    __shared__ uint32_t s_goff[256];     // global position of the tile's first element of each digit
    __shared__ uint32_t s_tstart[256];   // tile-local position of the first element of each digit
    __shared__ uint32_t s_wtot[RS_WARPS];
    __shared__ uint32_t s_key[RS_TILE], s_val[RS_TILE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // Global offset of each digit for this tile: exclusive scan of the digit
    // totals plus this tile's position in the digit's row.
    {
        const uint32_t t = totals[threadIdx.x];
        uint32_t x = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wtot[warp] = x;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += s_wtot[w];
        s_goff[threadIdx.x] = before + x - t + counts[(uint64_t)threadIdx.x * ntiles + blockIdx.x];
    }
    for (int i = lane; i < 256; i += 32) s_cnt[warp][i] = 0;
    __syncwarp();

    // Stable rank of every element among equal digits: warp-local ranks from
    // __match_any_sync, in warp order within the tile.
    const uint64_t tbase = (uint64_t)blockIdx.x * RS_TILE;
    const uint64_t wbase = tbase + (uint64_t)warp * (RS_ITEMS * 32);
    const unsigned lt_mask = (1u << lane) - 1u;
    uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const uint64_t k = wbase + (uint64_t)r * 32 + lane;
        const bool valid = k < n;
        key[r] = valid ? kin[k] : 0u;
        val[r] = valid ? vin[k] : 0u;
        rank[r] = 0;
        const unsigned vmask = __ballot_sync(FULL, valid);
        if (valid) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const unsigned peers = __match_any_sync(vmask, d);
            const uint32_t lt = __popc(peers & lt_mask);
            const uint32_t b = s_cnt[warp][d];
            rank[r] = b + lt;
            __syncwarp(vmask);
            if (lt == 0) s_cnt[warp][d] = b + __popc(peers);
            __syncwarp(vmask);
        }
    }
    __syncthreads();
    // per digit: offsets of the warps within the tile's run of that digit,
    // then the tile-local start of every digit (exclusive scan over digits)
    {
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = s_cnt[w][d];
            s_cnt[w][d] = run;
            run += c;
        }
        uint32_t x = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        __syncthreads();   // s_wtot is reused
        if (lane == 31) s_wtot[warp] = x;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += s_wtot[w];
        s_tstart[d] = before + x - run;
    }
    __syncthreads();
    // the tile in digit order in shared memory
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const uint64_t k = wbase + (uint64_t)r * 32 + lane;
        if (k < n) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t lp = s_tstart[d] + s_cnt[warp][d] + rank[r];
            if (lp < (uint32_t)RS_TILE) {   // always true for consistent counts
                s_key[lp] = key[r];
                s_val[lp] = val[r];
            }
        }
    }
    __syncthreads();
    // runs of equal digits go to consecutive global positions: coalesced writes
    const uint32_t tn = (uint32_t)min((uint64_t)RS_TILE, n - tbase);
    for (uint32_t i = threadIdx.x; i < tn; i += RS_THREADS) {
        const uint32_t kk = s_key[i];
        const uint32_t d = (kk >> shift) & 255u;
        const uint64_t pos = (uint64_t)s_goff[d] + (i - s_tstart[d]);
        if (pos < n) {   // always true for consistent counts; keeps a bad count in bounds
            kout[pos] = kk;
            vout[pos] = s_val[i];
        }
    }
}

// 3-D Morton key of sort.c:748-805 restated: the reference builds a 128-bit
// value from byte-wise interleaving tables whose top byte is shifted out, so
// the ordering equals that of the 72-bit interleave of the low 24 bits of
// (x, y, z), x the most significant bit of each triple.  Returns bits
// [32*slice, 32*slice+32) of that 72-bit value.
__device__ __forceinline__ uint32_t morton3_slice(uint32_t x, uint32_t y, uint32_t z, int slice) {
    uint32_t out = 0;
    const int lo = slice * 32;
#pragma unroll 1
    for (int b = 0; b < 32; ++b) {
        const int j = lo + b;          // bit position in the 72-bit key
        if (j >= 72) break;
        const int cb = j / 3;          // coordinate bit
        const int which = j % 3;       // 0 -> z, 1 -> y, 2 -> x
        const uint32_t c = which == 0 ? z : (which == 1 ? y : x);
        out |= ((c >> cb) & 1u) << b;
    }
    return out;
}

// 4-D Morton key of sort.c:816-995: every coordinate bit i is spread to bit
// 4*i, key = w | z<<1 | y<<2 | x<<3 (128 bits).  Slice s holds coordinate
// bits [8s, 8s+8) of all four coordinates.
__device__ __forceinline__ uint32_t morton4_slice(uint32_t x, uint32_t y, uint32_t z, uint32_t w, int slice) {
    uint32_t out = 0;
    const int cb0 = slice * 8;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int cb = cb0 + b;
        out |= ((w >> cb) & 1u) << (4 * b);
        out |= ((z >> cb) & 1u) << (4 * b + 1);
        out |= ((y >> cb) & 1u) << (4 * b + 2);
        out |= ((x >> cb) & 1u) << (4 * b + 3);
    }
    return out;
}

__global__ void k_make_keys(sptgb_keyspec ks, const uint32_t *__restrict__ perm, uint32_t *__restrict__ keys,
                            uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = perm ? perm[i] : (uint32_t)i;
        uint32_t k;
        if (ks.kind == 0) {
            k = ks.inds[ks.mode][p] >> ks.shift;
        } else if (ks.kind == 1) {
            k = morton3_slice(ks.inds[0][p], ks.inds[1][p], ks.inds[2][p], ks.slice);
        } else {
            k = morton4_slice(ks.inds[0][p], ks.inds[1][p], ks.inds[2][p], ks.inds[3][p], ks.slice);
        }
        keys[i] = k;
    }
}

__global__ void k_iota(uint32_t *p, uint64_t n, uint32_t start) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = start + (uint32_t)i;
}

template <typename T>
__global__ void k_gather(const T *__restrict__ in, const uint32_t *__restrict__ perm, T *__restrict__ out,
                         uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[perm[i]];
}

struct IndsArg { const uint32_t *p[SPTGB_MAX_MODES]; };

__global__ void k_mark_groups(IndsArg ia, int nmodes, int bits, uint64_t n, uint32_t *__restrict__ flags) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t f = (i == 0);
        if (i > 0) {
            for (int m = 0; m < nmodes; ++m)
                f |= (ia.p[m][i] >> bits) != (ia.p[m][i - 1] >> bits);
        }
        flags[i] = f;
    }
}

// Three-phase exclusive scan: per-block sums, scan of block sums (one CTA),
// block-local scan plus offset.
constexpr int SC_THREADS = 1024;
constexpr int SC_ITEMS = 8;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__device__ __forceinline__ uint32_t block_incl_scan(uint32_t x, uint32_t *wsum, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    const uint32_t r = x + (warp ? wsum[warp - 1] : 0u);
    *total = wsum[31];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SC_THREADS)
k_scan_reduce(const uint32_t *__restrict__ in, uint64_t n, uint32_t *__restrict__ bsum) {
    __shared__ uint32_t wsum[32];
    const uint64_t base = (uint64_t)blockIdx.x * SC_TILE;
    uint32_t s = 0;
    for (int i = 0; i < SC_ITEMS; ++i) {
        const uint64_t k = base + (uint64_t)i * SC_THREADS + threadIdx.x;
        if (k < n) s += in[k];
    }
    uint32_t tot;
    block_incl_scan(s, wsum, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SC_THREADS)
k_scan_blocks(uint32_t *bsum, uint32_t nb, uint32_t *total) {
    __shared__ uint32_t wsum[32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SC_THREADS) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? bsum[i] : 0u;
        uint32_t tot;
        const uint32_t incl = block_incl_scan(v, wsum, &tot);
        if (i < nb) bsum[i] = carry + incl - v;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(SC_THREADS)
k_scan_down(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t n,
            const uint32_t *__restrict__ bsum) {
    __shared__ uint32_t wsum[32];
    const uint64_t base = (uint64_t)blockIdx.x * SC_TILE + (uint64_t)threadIdx.x * SC_ITEMS;
    uint32_t v[SC_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) {
        const uint64_t k = base + i;
        v[i] = k < n ? in[k] : 0u;
        s += v[i];
    }
    uint32_t tot;
    const uint32_t incl = block_incl_scan(s, wsum, &tot);
    uint32_t run = bsum[blockIdx.x] + incl - s;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) {
        const uint64_t k = base + i;
        if (k < n) out[k] = run;
        run += v[i];
    }
}

__global__ void k_compact_starts(const uint32_t *__restrict__ flags, const uint32_t *__restrict__ pos, uint64_t n,
                                 uint64_t *__restrict__ starts) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (flags[i]) starts[pos[i]] = i;
}

__global__ void k_compact_u32(const uint32_t *__restrict__ flags, const uint32_t *__restrict__ pos,
                              const uint32_t *__restrict__ vals, uint64_t n, uint32_t *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        if (flags[i]) out[pos[i]] = vals[i];
}

__global__ void k_check_sorted(const uint32_t *__restrict__ v, uint64_t n, unsigned int *__restrict__ unsorted) {
    unsigned int bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x + 1; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        bad |= v[i] < v[i - 1];
    bad = __any_sync(FULL, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(unsorted, 1u);
}

struct BoundsArg { const uint32_t *p[SPTGB_MAX_MODES]; uint32_t lim[SPTGB_MAX_MODES]; };

__global__ void k_check_bounds(BoundsArg b, int nmodes, uint64_t n, unsigned int *__restrict__ bad_out) {
    unsigned int bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        for (int m = 0; m < nmodes; ++m)
            if (b.p[m]) bad |= b.p[m][i] >= b.lim[m];
    bad = __any_sync(FULL, bad);
    if (bad && (threadIdx.x & 31) == 0) atomicOr(bad_out, 1u);
}

struct SplitArg {
    const uint32_t *inds[SPTGB_MAX_MODES];
    uint8_t *einds[SPTGB_MAX_MODES];
    uint32_t *binds[SPTGB_MAX_MODES];
};

__global__ void k_hicoo_split(SplitArg a, int nmodes, int sb, uint64_t n, const uint32_t *__restrict__ bflags,
                              const uint32_t *__restrict__ bpos) {
    const uint32_t emask = (1u << sb) - 1u;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const bool head = bflags[i] != 0;
        const uint32_t b = bpos[i];
        for (int m = 0; m < nmodes; ++m) {
            const uint32_t c = a.inds[m][i];
            a.einds[m][i] = (uint8_t)(c & emask);
            if (head) a.binds[m][b] = c >> sb;
        }
    }
}

inline unsigned grid_for(uint64_t n, unsigned threads) {
    uint64_t g = (n + threads - 1) / threads;
    if (g > (uint64_t)sptgb_sm_count() * 32) g = (uint64_t)sptgb_sm_count() * 32;
    if (g == 0) g = 1;
    return (unsigned)g;
}

}  // namespace

extern "C" size_t sptgb_radix_tmp_bytes(uint64_t n) {
    const uint64_t ntiles = (n + RS_TILE - 1) / RS_TILE + 1;
    return (size_t)(256 * ntiles + 256) * sizeof(uint32_t) + 256;
}

extern "C" cudaError_t sptgb_radix_sort_u32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int bits,
                                            void *tmp, int *which, cudaStream_t s) {
    *which = 0;
    if (n <= 1 || bits <= 0) return cudaSuccess;
    const uint32_t ntiles = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
    uint32_t *counts = (uint32_t *)tmp;
    uint32_t *totals = counts + (uint64_t)256 * ntiles;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        rs_upsweep<<<ntiles, RS_THREADS, 0, s>>>(keys[cur], n, shift, counts, ntiles);
        rs_rowscan<<<256, 1024, 0, s>>>(counts, ntiles, totals);
        rs_downsweep<<<ntiles, RS_THREADS, 0, s>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, shift,
                                                   counts, totals, ntiles);
        sptgb_count_launch(3);
        cur ^= 1;
    }
    *which = cur;
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_make_keys(const sptgb_keyspec *ks, const uint32_t *perm, uint32_t *keys, uint64_t n,
                                       cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_make_keys<<<grid_for(n, 256), 256, 0, s>>>(*ks, perm, keys, n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_iota_u32(uint32_t *p, uint64_t n, uint32_t start, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(p, n, start);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_gather_records(const void *src, const uint32_t *perm, void *dst, uint64_t n,
                                            cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_gather<uint4><<<grid_for(n, 256), 256, 0, s>>>(static_cast<const uint4 *>(src), perm, static_cast<uint4 *>(dst), n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_gather_u32(const uint32_t *in, const uint32_t *perm, uint32_t *out, uint64_t n,
                                        cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_gather<uint32_t><<<grid_for(n, 256), 256, 0, s>>>(in, perm, out, n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_gather_u8(const uint8_t *in, const uint32_t *perm, uint8_t *out, uint64_t n,
                                       cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_gather<uint8_t><<<grid_for(n, 256), 256, 0, s>>>(in, perm, out, n);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_mark_groups(const uint32_t *const *inds, int nmodes, int bits, uint64_t n,
                                         uint32_t *flags, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    IndsArg ia;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) ia.p[m] = m < nmodes ? inds[m] : nullptr;
    k_mark_groups<<<grid_for(n, 256), 256, 0, s>>>(ia, nmodes, bits, n, flags);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" size_t sptgb_scan_tmp_bytes(uint64_t n) {
    return ((n + SC_TILE - 1) / SC_TILE + 1) * sizeof(uint32_t) + 256;
}

extern "C" cudaError_t sptgb_exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total,
                                                void *tmp, cudaStream_t s) {
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return cudaSuccess;
    }
    const uint32_t nb = (uint32_t)((n + SC_TILE - 1) / SC_TILE);
    uint32_t *bsum = (uint32_t *)tmp;
    k_scan_reduce<<<nb, SC_THREADS, 0, s>>>(in, n, bsum);
    k_scan_blocks<<<1, SC_THREADS, 0, s>>>(bsum, nb, total);
    k_scan_down<<<nb, SC_THREADS, 0, s>>>(in, out, n, bsum);
    sptgb_count_launch(3);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_compact_starts(const uint32_t *flags, const uint32_t *pos, uint64_t n,
                                            uint64_t *starts, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_compact_starts<<<grid_for(n, 256), 256, 0, s>>>(flags, pos, n, starts);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_compact_u32(const uint32_t *flags, const uint32_t *pos, const uint32_t *vals,
                                         uint64_t n, uint32_t *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_compact_u32<<<grid_for(n, 256), 256, 0, s>>>(flags, pos, vals, n, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_check_sorted(const uint32_t *v, uint64_t n, unsigned int *unsorted, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(unsorted, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess || n < 2) return e;
    k_check_sorted<<<grid_for(n, 256), 256, 0, s>>>(v, n, unsorted);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_check_bounds(const uint32_t *const *inds, const uint32_t *lims, int nmodes, uint64_t n,
                                          unsigned int *bad, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess || n == 0) return e;
    BoundsArg b;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) {
        b.p[m] = m < nmodes ? inds[m] : nullptr;
        b.lim[m] = m < nmodes ? lims[m] : 0u;
    }
    k_check_bounds<<<grid_for(n, 256), 256, 0, s>>>(b, nmodes, n, bad);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_hicoo_split(const uint32_t *const *inds, int nmodes, int sb_bits, uint64_t n,
                                         const uint32_t *bflags, const uint32_t *bpos, uint8_t *const *einds,
                                         uint32_t *const *binds, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    SplitArg a;
    for (int m = 0; m < SPTGB_MAX_MODES; ++m) {
        a.inds[m] = m < nmodes ? inds[m] : nullptr;
        a.einds[m] = m < nmodes ? einds[m] : nullptr;
        a.binds[m] = m < nmodes ? binds[m] : nullptr;
    }
    k_hicoo_split<<<grid_for(n, 256), 256, 0, s>>>(a, nmodes, sb_bits, n, bflags, bpos);
    sptgb_count_launch(1);
    return cudaGetLastError();
}
