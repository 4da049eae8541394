// HiCOO MTTKRP for sm_103a (sptMTTKRPHiCOO, src/sptensor/hicoo/mttkrp.c:53-144).
//
// Window kernel (k_hicoo_win2, orders 3 and 4): the blocks are visited in
// the order of their block index in the output mode (a stable device sort of
// binds[mode], sptgb_hicoo_schedule), so all blocks writing one output window
// of 2^sb rows are consecutive.  The nonzeros, in that order, are split
// evenly over persistent CTAs.  A window holding a large share of the tensor
// (a heavy window: the head of a power-law mode) is summed in a shared-memory
// tile (2^sb rows x stride, shared atomics) that is written once: plain
// stores when the CTA covers the whole window, vector atomics when the window
// continues in a neighbouring CTA, so skewed rows cost shared-memory atomics,
// not contended global ones.  Light windows go straight to the output.
//
// Light kernel (k_hicoo_light, orders 3 and 4): a schedule with no heavy
// window runs the window kernel's light path over all its positions, without
// the tile's shared memory and, for order 3, at a higher CTA count per SM.
//
// Block kernel (k_mttkrp_hicoo, any order; used without a schedule): a
// worker (W lanes, one float4 column group per lane) owns one HiCOO block
// at a time.  Element coordinates are rebuilt as (binds << sb_bits) + einds
// (hicoo/mttkrp.c:109); the product runs over mats_order[1..N-1] in order.
// Consecutive elements of a block that hit the same output row are summed in
// registers; each finished row partial is added to the (pre-zeroed) output
// with one vector atomic, because several blocks (in different kernels) share
// output rows.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"

namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr int BLOCK = 256;

template <int W>
__global__ void __launch_bounds__(BLOCK) k_mttkrp_hicoo(sptgb_hicoo_args a) {
    const int lane = threadIdx.x & 31;
    const int sl = lane % W;
    const uint64_t worker = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BLOCK) / W;
    const bool col_ok = (uint32_t)(sl * 4) < a.stride;
    const int c0 = sl * 4;
    const bool m0 = c0 + 0 < (int)a.rank, m1 = c0 + 1 < (int)a.rank;
    const bool m2 = c0 + 2 < (int)a.rank, m3 = c0 + 3 < (int)a.rank;
    const int N = (int)a.nmodes;
    const uint32_t mode = a.mode;

    for (uint64_t b = worker; b < a.nb; b += nworkers) {
        uint32_t base[SPTGB_MAX_MODES];
#pragma unroll
        for (int m = 0; m < SPTGB_MAX_MODES; ++m) base[m] = m < N ? (a.binds[m][b] << a.sb_bits) : 0u;
        const uint64_t z0 = a.bptr[b], z1 = a.bptr[b + 1];
        uint32_t cur = NONE;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (uint64_t z = z0; z < z1; ++z) {
            const uint32_t row = base[mode] + a.einds[mode][z];
            bool inside = row < a.out_rows;
            for (int i = 1; i < N; ++i) {
                const uint32_t fm = a.order[i];
                inside &= base[fm] + a.einds[fm][z] < a.ndims[fm];
            }
            if (!inside) {
                if (sl == 0) atomicOr(a.err, 1u);
                continue;
            }
            const float v = a.vals[z];
            float4 p = make_float4(v, v, v, v);
            if (col_ok) {
                for (int i = 1; i < N; ++i) {
                    const uint32_t fm = a.order[i];
                    const uint32_t ri = base[fm] + a.einds[fm][z];
                    const float4 f = __ldg(reinterpret_cast<const float4 *>(a.fac[fm] + (size_t)ri * a.stride) + sl);
                    p.x *= f.x;
                    p.y *= f.y;
                    p.z *= f.z;
                    p.w *= f.w;
                }
            }
            if (row != cur) {
                if (cur != NONE && col_ok)
                    atomicAdd(reinterpret_cast<float4 *>(a.out + (size_t)cur * a.stride) + sl, acc);
                cur = row;
                acc = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (m0) acc.x += p.x;
            if (m1) acc.y += p.y;
            if (m2) acc.z += p.z;
            if (m3) acc.w += p.w;
        }
        if (cur != NONE && col_ok) atomicAdd(reinterpret_cast<float4 *>(a.out + (size_t)cur * a.stride) + sl, acc);
    }
}

// Block k (position in the schedule) holding schedule position p.
__device__ __forceinline__ uint64_t block_at(const uint32_t *pnnz, uint64_t lo, uint64_t hi, uint32_t p) {
    while (hi - lo > 1) {   // last k in [lo, hi) with pnnz[k] <= p
        const uint64_t mid = (lo + hi) >> 1;
        if (pnnz[mid] <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The window kernels' work, per worker:
//  * Decoding: each worker owns a contiguous share of its positions, and its
//    W lanes decode W consecutive schedule positions together: they load the
//    next W block boundaries (pnnz) at once and each lane finds its block
//    with a log2(W)-step search over them through shuffles (exact with empty
//    blocks), so the block and element loads of the 32 positions of a warp
//    are in flight together instead of one dependent chain per element.  The
//    decoded records (output row, the product modes' rows, value) go through
//    shared memory to the worker, which issues the factor-row gathers of a
//    batch of them before using any.
//  * Windows: only heavy windows (at least heavy_nnz nonzeros, the
//    hot rows of a power-law mode) are summed in the shared-memory tile and
//    written once.  A run of consecutive light windows is one flat range: the
//    running row sum of a worker goes to the output with a vector atomic when
//    the row changes, with no per-window barrier or tile write, so the many
//    small windows of a long tail cost no more than their nonzeros.
//
// Per-lane constants; product modes a, b (mats_order[1], [2]) and, for
// order 4, c ([3]).
struct Win2Ctx {
    const uint8_t *e_m, *e_a, *e_b, *e_c;
    const uint32_t *b_m, *b_a, *b_b, *b_c;
    const char *Fa, *Fb, *Fc;   // factor rows, offset to this lane's columns
    uint32_t rb;      // bytes per factor row (stride * 4 <= 512)
    uint32_t lim_a, lim_b, lim_c, rows_w, st;
    int sl, wk, c0;
    bool col_ok, m0, m1, m2, m3;
    uint32_t mrot;    // column mask m0 | m1 << 1 | m2 << 2 | m3 << 3 rotated right by wk mod 4
};

// One worker's positions [r_beg, r_end) of the blocks [klo, khi) of the
// schedule, for NP product modes (2: order 3, 3: order 4).  Records are
// staged as {row, row of a, row of b, value} (NP = 2) or as {row of a, row
// of b, row of c, value} with the output row in s_row (NP = 3).  TILE: rows
// are window rows (row0 + r) summed in `tile`; otherwise output rows,
// flushed with vector atomics.  FULL: the stride is
// exactly 4W columns, so every lane holds stored columns and the factor rows
// are gathered without a select (an empty record carries rows 0, in range).
// AC (with FULL): the rank equals the stride, so no column is padding and the
// row flushes need no column masks.  EB: records per gather batch.
template <int W, int NP, bool TILE, bool FULL, bool AC, int EB = 2>
__device__ __forceinline__ void win2_range(const sptgb_hicoo_args &a, const Win2Ctx &x, uint4 *s_rec,
                                           uint32_t *s_row, float *tile,
                                           uint32_t row0, uint64_t klo, uint64_t khi, uint32_t r_beg,
                                           uint32_t r_end) {
    uint32_t cur = NONE;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    auto put = [&]() {
        if (cur == NONE || (!FULL && !x.col_ok)) return;
        if (TILE) {
            // worker k adds its four columns starting at column k mod 4: at
            // each step the workers of a warp hit four different bank classes
            // (no bank conflict for a 32-float row, and no same-address
            // serialisation when two workers hold the same row)
            float *t = tile + cur * x.st + x.c0;
            float4 v = acc;   // rotated left by wk mod 4
            if (x.wk & 1) v = make_float4(v.y, v.z, v.w, v.x);
            if (x.wk & 2) v = make_float4(v.z, v.w, v.x, v.y);
            const int r = x.wk & 3;
            if (AC || (x.mrot & 1)) atomicAdd(t + (r & 3), v.x);
            if (AC || (x.mrot & 2)) atomicAdd(t + ((r + 1) & 3), v.y);
            if (AC || (x.mrot & 4)) atomicAdd(t + ((r + 2) & 3), v.z);
            if (AC || (x.mrot & 8)) atomicAdd(t + ((r + 3) & 3), v.w);
        } else {
            const float4 v = AC ? acc
                                : make_float4(x.m0 ? acc.x : 0.f, x.m1 ? acc.y : 0.f, x.m2 ? acc.z : 0.f,
                                              x.m3 ? acc.w : 0.f);
            atomicAdd(reinterpret_cast<float4 *>(a.out + (size_t)cur * x.st) + x.sl, v);
        }
    };
    // block positions and element offsets fit in 32 bits: the launcher
    // takes this kernel only for nb and nnz below 2^32 - 2^12, and bptr was
    // checked to rise from 0 to nnz
    const uint32_t khi32 = (uint32_t)khi;
    uint32_t kb = (uint32_t)klo;
    uint32_t kst = 0;
    if (r_beg < r_end) {
        kb = (uint32_t)block_at(a.pnnz, klo, khi, r_beg);
        kst = a.pnnz[kb];
    }
    const uint32_t rounds = __reduce_max_sync(0xffffffffu, (r_end - r_beg + W - 1) / W);
    for (uint32_t it = 0; it < rounds; ++it) {
        const uint32_t p = r_beg + it * W + x.sl;
        const bool valid = p < r_end;
        // lane's block: kb + (boundaries pnnz[kb+1 ..] <= p), searched over
        // the W boundaries the worker's lanes load; boundaries past khi read
        // as 0xffffffff, so the loop ends after at most (khi - kb) / W + 1
        // rounds (more than one only when blocks are empty)
        uint32_t myk = kb;
        uint32_t mystart = kst;
        bool todo = valid;
        uint32_t base = kb;
        uint32_t bstart = kst;
        for (uint32_t guard = 0; guard < (1u << 26) && __any_sync(0xffffffffu, todo); ++guard) {
            const uint32_t idx = base + 1 + x.sl;
            const uint32_t bv = idx <= khi32 ? a.pnnz[idx] : 0xffffffffu;
            uint32_t c = 0;
#pragma unroll
            for (int step = W / 2; step >= 1; step >>= 1) {
                const uint32_t t = __shfl_sync(0xffffffffu, bv, (int)(c + step - 1), W);
                if (todo && t <= p) c += step;
            }
            const uint32_t last = __shfl_sync(0xffffffffu, bv, W - 1, W);
            if (todo && c == W - 1 && last <= p) c = W;   // all W boundaries passed
            const uint32_t prev = __shfl_sync(0xffffffffu, bv, (int)(c > 0 ? c - 1 : 0), W);
            if (todo && c < W) {
                myk = base + c;
                mystart = c ? prev : bstart;
                todo = false;
            }
            bstart = last;
            base += W;
        }
        // an empty record: row NONE, product rows 0 (in range for the
        // unconditional gathers)
        uint4 r = make_uint4(NP == 2 ? NONE : 0u, 0u, 0u, 0u);
        uint32_t rrow = NONE;
        if (valid && !todo) {
            const uint32_t b = a.perm[myk];
            const uint32_t e = (uint32_t)a.bptr[b] + (p - mystart);
            bool ok = e < a.nnz;
            if (ok) {
                const uint32_t rl = x.e_m[e];
                const uint32_t row = TILE ? rl : (x.b_m[b] << a.sb_bits) + rl;
                const uint32_t ra = (x.b_a[b] << a.sb_bits) + x.e_a[e];
                const uint32_t rr = (x.b_b[b] << a.sb_bits) + x.e_b[e];
                if constexpr (NP == 2) {
                    ok = rl < x.rows_w && (TILE ? row0 + rl : row) < a.out_rows && ra < x.lim_a && rr < x.lim_b;
                    if (ok) r = make_uint4(row, ra, rr, __float_as_uint(a.vals[e]));
                } else {
                    const uint32_t rc = (x.b_c[b] << a.sb_bits) + x.e_c[e];
                    ok = rl < x.rows_w && (TILE ? row0 + rl : row) < a.out_rows && ra < x.lim_a && rr < x.lim_b &&
                         rc < x.lim_c;
                    if (ok) {
                        r = make_uint4(ra, rr, rc, __float_as_uint(a.vals[e]));
                        rrow = row;
                    }
                }
            }
            if (!ok) atomicOr(a.err, 1u);
        } else if (valid) {
            atomicOr(a.err, 1u);
        }
        // the next round of this worker starts in its last lane's block
        kb = __shfl_sync(0xffffffffu, myk, W - 1, W);
        kst = __shfl_sync(0xffffffffu, mystart, W - 1, W);
        s_rec[threadIdx.x & 31] = r;
        if constexpr (NP == 3) s_row[threadIdx.x & 31] = rrow;
        __syncwarp();
#pragma unroll
        for (int j0 = 0; j0 < W; j0 += EB) {
            if constexpr (NP == 2) {
                uint4 q4[EB];
                float4 fa[EB], fb[EB];
#pragma unroll
                for (int t = 0; t < EB; ++t) q4[t] = s_rec[x.wk * W + j0 + t];
#pragma unroll
                for (int t = 0; t < EB; ++t) {
                    if (FULL) {
                        fa[t] = __ldg(reinterpret_cast<const float4 *>(x.Fa + (size_t)q4[t].y * x.rb));
                        fb[t] = __ldg(reinterpret_cast<const float4 *>(x.Fb + (size_t)q4[t].z * x.rb));
                    } else {
                        const bool use = q4[t].x != NONE && x.col_ok;
                        fa[t] = use ? __ldg(reinterpret_cast<const float4 *>(x.Fa + (size_t)q4[t].y * x.rb))
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
                        fb[t] = use ? __ldg(reinterpret_cast<const float4 *>(x.Fb + (size_t)q4[t].z * x.rb))
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
#pragma unroll
                for (int t = 0; t < EB; ++t) {
                    if (q4[t].x == NONE) continue;
                    if (q4[t].x != cur) {
                        put();
                        cur = q4[t].x;
                        acc = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    const float v = __uint_as_float(q4[t].w);
                    acc.x += v * fa[t].x * fb[t].x;
                    acc.y += v * fa[t].y * fb[t].y;
                    acc.z += v * fa[t].z * fb[t].z;
                    acc.w += v * fa[t].w * fb[t].w;
                }
            } else {
                // order 4: v * U_a * U_b * U_c in mats_order
                uint4 q4[EB];
                uint32_t qr[EB];
                float4 fa[EB], fb[EB], fc[EB];
#pragma unroll
                for (int t = 0; t < EB; ++t) {
                    q4[t] = s_rec[x.wk * W + j0 + t];
                    qr[t] = s_row[x.wk * W + j0 + t];
                }
#pragma unroll
                for (int t = 0; t < EB; ++t) {
                    const bool use = FULL || (qr[t] != NONE && x.col_ok);
                    fa[t] = use ? __ldg(reinterpret_cast<const float4 *>(x.Fa + (size_t)q4[t].x * x.rb))
                                : make_float4(0.f, 0.f, 0.f, 0.f);
                    fb[t] = use ? __ldg(reinterpret_cast<const float4 *>(x.Fb + (size_t)q4[t].y * x.rb))
                                : make_float4(0.f, 0.f, 0.f, 0.f);
                    fc[t] = use ? __ldg(reinterpret_cast<const float4 *>(x.Fc + (size_t)q4[t].z * x.rb))
                                : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int t = 0; t < EB; ++t) {
                    if (qr[t] == NONE) continue;
                    if (qr[t] != cur) {
                        put();
                        cur = qr[t];
                        acc = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    const float v = __uint_as_float(q4[t].w);
                    acc.x += v * fa[t].x * fb[t].x * fc[t].x;
                    acc.y += v * fa[t].y * fb[t].y * fc[t].y;
                    acc.z += v * fa[t].z * fb[t].z * fc[t].z;
                    acc.w += v * fa[t].w * fb[t].w * fc[t].w;
                }
            }
        }
        __syncwarp();
    }
    put();
}

// The per-lane constants of a worker (lane sl of worker wk in its warp).
template <int W, int NP>
__device__ __forceinline__ void win2_ctx(const sptgb_hicoo_args &a, Win2Ctx &x) {
    const int lane = threadIdx.x & 31;
    x.sl = lane % W;
    x.wk = lane / W;
    x.rows_w = 1u << a.sb_bits;
    x.st = a.stride;
    x.col_ok = (uint32_t)(x.sl * 4) < x.st;
    x.c0 = x.sl * 4;
    x.m0 = x.c0 + 0 < (int)a.rank;
    x.m1 = x.c0 + 1 < (int)a.rank;
    x.m2 = x.c0 + 2 < (int)a.rank;
    x.m3 = x.c0 + 3 < (int)a.rank;
    {
        const uint32_t mb = (uint32_t)x.m0 | (uint32_t)x.m1 << 1 | (uint32_t)x.m2 << 2 | (uint32_t)x.m3 << 3;
        const uint32_t r = (uint32_t)x.wk & 3u;
        x.mrot = ((mb >> r) | (mb << (4 - r))) & 15u;
    }
    const uint32_t mode = a.mode, pa = a.order[1], pb = a.order[2];
    x.e_m = a.einds[mode];
    x.e_a = a.einds[pa];
    x.e_b = a.einds[pb];
    x.b_m = a.binds[mode];
    x.b_a = a.binds[pa];
    x.b_b = a.binds[pb];
    x.lim_a = a.ndims[pa];
    x.lim_b = a.ndims[pb];
    x.Fa = reinterpret_cast<const char *>(a.fac[pa]) + (size_t)x.sl * 16;
    x.Fb = reinterpret_cast<const char *>(a.fac[pb]) + (size_t)x.sl * 16;
    if constexpr (NP == 3) {
        const uint32_t pc = a.order[3];
        x.e_c = a.einds[pc];
        x.b_c = a.binds[pc];
        x.lim_c = a.ndims[pc];
        x.Fc = reinterpret_cast<const char *>(a.fac[pc]) + (size_t)x.sl * 16;
    }
    x.rb = x.st * 4u;
}

// A schedule without heavy windows (no output window holds heavy_nnz
// nonzeros, e.g. every window of a uniform mode) is one flat light range:
// this kernel has no tile, so it needs no shared memory beyond the record
// staging (the L1 keeps the rest) and fewer registers than k_hicoo_win2.
constexpr int LIGHT_MINB = 6;   // CTAs per SM the register budget is set for (order 3)
constexpr int LIGHT_EB = 2;     // records per gather batch
// CTAs per SM of the window kernels: order 4 gathers a third factor row per
// record and gets the registers of 4 CTAs per SM
constexpr int win_minb(int np, bool light) { return np == 2 ? (light ? LIGHT_MINB : 5) : 4; }
template <int W, int NP, bool FULL, bool AC>
__global__ void __launch_bounds__(BLOCK, win_minb(NP, true))
    k_hicoo_light(sptgb_hicoo_args a, uint32_t chunk, uint32_t total) {
    constexpr int NWARP = BLOCK / 32;
    constexpr uint32_t NWC = BLOCK / W;   // workers per CTA
    __shared__ uint4 s_rec[NWARP][32];
    __shared__ uint32_t s_row[NP == 3 ? NWARP : 1][32];   // output rows of the staged order-4 records
    const int warp = threadIdx.x >> 5;
    Win2Ctx x;
    win2_ctx<W, NP>(a, x);
    const uint32_t gw = (uint32_t)(warp * (32 / W) + x.wk);
    const uint64_t lo64 = (uint64_t)blockIdx.x * chunk;
    if (lo64 >= total) return;
    const uint32_t lo = (uint32_t)lo64, hi = (uint32_t)min((uint64_t)total, lo64 + chunk);
    const uint32_t per = (hi - lo + NWC - 1) / NWC;
    const uint32_t r_beg = lo + min(hi - lo, gw * per);
    win2_range<W, NP, false, FULL, AC, LIGHT_EB>(a, x, s_rec[warp], s_row[NP == 3 ? warp : 0], nullptr, 0u, 0u,
                                                 a.nb, r_beg, min(hi, r_beg + per));
}

template <int W, int NP, bool FULL, bool AC>
__global__ void __launch_bounds__(BLOCK, win_minb(NP, false))
    k_hicoo_win2(sptgb_hicoo_args a, uint32_t chunk, uint32_t total) {
    extern __shared__ float tile[];   // [1 << sb][stride]
    constexpr int NWARP = BLOCK / 32;
    constexpr int NWK = 32 / W;              // workers per warp
    constexpr uint32_t NWC = BLOCK / W;      // workers per CTA
    __shared__ uint4 s_rec[NWARP][32];
    __shared__ uint32_t s_row[NP == 3 ? NWARP : 1][32];   // output rows of the staged order-4 records
    const int warp = threadIdx.x >> 5;
    Win2Ctx x;
    win2_ctx<W, NP>(a, x);
    const uint32_t mode = a.mode;
    const uint32_t st4 = x.st / 4;
    const uint32_t gw = (uint32_t)(warp * NWK + x.wk);

    const uint64_t lo64 = (uint64_t)blockIdx.x * chunk;
    if (lo64 >= total) return;
    const uint32_t lo = (uint32_t)lo64, hi = (uint32_t)min((uint64_t)total, lo64 + chunk);
    for (uint32_t i = threadIdx.x; i < x.rows_w * x.st; i += BLOCK) tile[i] = 0.f;
    uint32_t wlo = 0, whi = a.nwin;   // first window: last w with pnnz[wst[w]] <= lo
    while (whi - wlo > 1) {
        const uint32_t mid = (wlo + whi) >> 1;
        if (a.pnnz[a.wst[mid]] <= lo) wlo = mid;
        else whi = mid;
    }
    uint32_t w = wlo;
    uint32_t q = lo;
    __syncthreads();
    while (q < hi) {
        const uint64_t k0 = a.wst[w], k1 = a.wst[w + 1];
        const uint32_t wbeg = a.pnnz[k0], wend = a.pnnz[k1];
        if (wend - wbeg < a.heavy_nnz) {
            // a run of light windows, up to the next heavy one
            uint32_t hl = 0, hh = a.nheavy;   // first heavy window > w
            while (hl < hh) {
                const uint32_t mid = (hl + hh) >> 1;
                if (a.heavy[mid] <= w) hl = mid + 1;
                else hh = mid;
            }
            const uint32_t wh = hl < a.nheavy ? (uint32_t)a.heavy[hl] : a.nwin;
            const uint64_t kend = a.wst[wh];
            const uint32_t rend = a.pnnz[kend];
            const uint32_t s0 = q, s1 = hi < rend ? hi : rend;
            const uint32_t per = (s1 - s0 + NWC - 1) / NWC;
            const uint32_t r_beg = s0 + min(s1 - s0, gw * per);
            win2_range<W, NP, false, FULL, AC>(a, x, s_rec[warp], s_row[NP == 3 ? warp : 0], tile, 0u, k0, kend,
                                               r_beg, min(s1, r_beg + per));
            q = s1;
            w = wh;
            continue;
        }
        const uint32_t s0 = q > wbeg ? q : wbeg, s1 = hi < wend ? hi : wend;
        const uint32_t row0 = a.binds[mode][a.perm[k0]] << a.sb_bits;
        const uint32_t per = (s1 - s0 + NWC - 1) / NWC;
        const uint32_t r_beg = s0 + min(s1 - s0, gw * per);
        win2_range<W, NP, true, FULL, AC>(a, x, s_rec[warp], s_row[NP == 3 ? warp : 0], tile, row0, k0, k1, r_beg,
                                          min(s1, r_beg + per));
        __syncthreads();
        // one write of the window: plain when this CTA covered all of it
        const bool owned = s0 == wbeg && s1 == wend;
        float4 *t4 = reinterpret_cast<float4 *>(tile);
        for (uint32_t i = threadIdx.x; i < x.rows_w * st4; i += BLOCK) {
            const uint32_t r = i / st4, c = i % st4;
            const float4 v = t4[i];
            t4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (row0 + r >= a.out_rows) continue;
            float4 *o = reinterpret_cast<float4 *>(a.out + (size_t)(row0 + r) * x.st) + c;
            if (owned) *o = v;
            else if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd(o, v);
        }
        __syncthreads();
        q = s1;
        ++w;
    }
}

// flags[w] = 1 when output window w holds at least `heavy` nonzeros.
__global__ void k_window_heavy(const uint64_t *__restrict__ wst, const uint32_t *__restrict__ pnnz, uint32_t nwin,
                               uint32_t heavy, uint32_t *__restrict__ flags) {
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwin; w += gridDim.x * blockDim.x)
        flags[w] = pnnz[wst[w + 1]] - pnnz[wst[w]] >= heavy;
}

__global__ void k_block_sizes(const uint32_t *__restrict__ perm, const uint64_t *__restrict__ bptr, uint64_t nb,
                              uint32_t *__restrict__ sizes) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nb; k += (uint64_t)gridDim.x * blockDim.x)
        sizes[k] = (uint32_t)(bptr[perm[k] + 1] - bptr[perm[k]]);
}

template <int W, int NP, bool FULL, bool AC>
cudaError_t launch_win2_k(const sptgb_hicoo_args &a, cudaStream_t s) {
    const size_t smem = ((size_t)1 << a.sb_bits) * a.stride * sizeof(float);
    if (smem > 180 * 1024) return cudaErrorInvalidValue;
    // once per process: a function-local static is initialised by one thread
    // while the others wait (a failure shows up as the launch's error)
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_hicoo_win2<W, NP, FULL, AC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 180 * 1024);
    (void)attr;
    const int nsm = sptgb_sm_count();
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_hicoo_win2<W, NP, FULL, AC>, BLOCK, smem);
    if (per < 1) per = 1;
    if (a.nnz == 0 || a.nnz >= 0xffffffffull) return a.nnz ? cudaErrorInvalidValue : cudaSuccess;
    const uint32_t total = (uint32_t)a.nnz;
    const uint64_t grid = (uint64_t)nsm * per * 2;
    const uint32_t chunk = (uint32_t)((total + grid - 1) / grid);
    const uint32_t ngrid = (total + chunk - 1) / chunk;
    k_hicoo_win2<W, NP, FULL, AC><<<ngrid, BLOCK, smem, s>>>(a, chunk, total);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

template <int W, int NP, bool FULL, bool AC>
cudaError_t launch_light_k(const sptgb_hicoo_args &a, cudaStream_t s) {
    static const int per = [] {
        int p = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_hicoo_light<W, NP, FULL, AC>, BLOCK, 0);
        return p < 1 ? 1 : p;
    }();
    const int nsm = sptgb_sm_count();
    if (a.nnz == 0 || a.nnz >= 0xffffffffull) return a.nnz ? cudaErrorInvalidValue : cudaSuccess;
    const uint32_t total = (uint32_t)a.nnz;
    const uint64_t grid = (uint64_t)nsm * per * 2;
    const uint32_t chunk = (uint32_t)((total + grid - 1) / grid);
    const uint32_t ngrid = (total + chunk - 1) / chunk;
    k_hicoo_light<W, NP, FULL, AC><<<ngrid, BLOCK, 0, s>>>(a, chunk, total);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

template <int W, int NP>
cudaError_t launch_win2(const sptgb_hicoo_args &a, cudaStream_t s) {
    if (a.nheavy == 0) {
        if (a.stride != 4u * W) return launch_light_k<W, NP, false, false>(a, s);
        return a.rank == a.stride ? launch_light_k<W, NP, true, true>(a, s) : launch_light_k<W, NP, true, false>(a, s);
    }
    if (a.stride != 4u * W) return launch_win2_k<W, NP, false, false>(a, s);
    return a.rank == a.stride ? launch_win2_k<W, NP, true, true>(a, s) : launch_win2_k<W, NP, true, false>(a, s);
}

// *err = 1 when an element's coordinate is outside its mode or its element
// offset is not below 2^sb (one thread per block).
__global__ void k_hicoo_check(const uint64_t *__restrict__ bptr, sptgb_hicoo_args a, uint64_t nb) {
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < nb; b += (uint64_t)gridDim.x * blockDim.x) {
        bool bad = false;
        for (uint64_t e = bptr[b]; e < bptr[b + 1] && !bad; ++e)
            for (uint32_t m = 0; m < a.nmodes; ++m) {
                const uint32_t el = a.einds[m][e];
                bad |= (el >> a.sb_bits) != 0 || (a.binds[m][b] << a.sb_bits) + el >= a.ndims[m];
            }
        if (bad) *a.err = 1u;
    }
}

template <int W>
cudaError_t launch(const sptgb_hicoo_args &a, cudaStream_t s) {
    static const int per_sm = [] {
        int p = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_mttkrp_hicoo<W>, BLOCK, 0);
        return p < 1 ? 1 : p;
    }();
    const int max_blocks = per_sm * sptgb_sm_count();
    const uint64_t wpb = BLOCK / W;
    uint64_t blocks = (a.nb + wpb - 1) / wpb;
    if (blocks > (uint64_t)max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    k_mttkrp_hicoo<W><<<(unsigned)blocks, BLOCK, 0, s>>>(a);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

}  // namespace

extern "C" cudaError_t sptgb_mttkrp_hicoo(const sptgb_hicoo_args *a, cudaStream_t s) {
    if (a->stride % 8 != 0 || a->stride > 128 || a->nmodes < 2 || a->nmodes > SPTGB_MAX_MODES)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a->out, 0, (size_t)a->out_rows * a->stride * sizeof(float), s);
    if (e != cudaSuccess || a->nb == 0) return e;
    const uint32_t c4 = a->stride / 4;
    // the window kernels count positions and blocks in 32 bits
    if (a->perm && (a->nmodes == 3 || a->nmodes == 4) && a->nnz < 0xfffff000ull) {
        if (a->nmodes == 3) {
            if (c4 <= 2) return launch_win2<2, 2>(*a, s);
            if (c4 <= 4) return launch_win2<4, 2>(*a, s);
            if (c4 <= 8) return launch_win2<8, 2>(*a, s);
            if (c4 <= 16) return launch_win2<16, 2>(*a, s);
            return launch_win2<32, 2>(*a, s);
        }
        if (c4 <= 2) return launch_win2<2, 3>(*a, s);
        if (c4 <= 4) return launch_win2<4, 3>(*a, s);
        if (c4 <= 8) return launch_win2<8, 3>(*a, s);
        if (c4 <= 16) return launch_win2<16, 3>(*a, s);
        return launch_win2<32, 3>(*a, s);
    }
    if (c4 <= 2) return launch<2>(*a, s);
    if (c4 <= 4) return launch<4>(*a, s);
    if (c4 <= 8) return launch<8>(*a, s);
    if (c4 <= 16) return launch<16>(*a, s);
    return launch<32>(*a, s);
}

extern "C" cudaError_t sptgb_hicoo_schedule(const uint32_t *binds_mode, const uint64_t *bptr, uint64_t nb,
                                            int window_bits, uint32_t heavy_nnz, const sptgb_hicoo_sched_scratch *w, uint32_t *perm,
                                            uint32_t *pnnz, uint64_t *wst, uint32_t *nwin_out, uint64_t *heavy,
                                            uint32_t *nheavy_out, cudaStream_t s) {
    *nwin_out = 0;
    *nheavy_out = 0;
    if (nb == 0) return cudaMemsetAsync(pnnz, 0, sizeof(uint32_t), s);
    cudaError_t e = cudaMemcpyAsync(w->keys[0], binds_mode, nb * 4, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = sptgb_iota_u32(w->vals[0], nb, 0, s);
    uint32_t *keys[2] = {w->keys[0], w->keys[1]}, *vals[2] = {w->vals[0], w->vals[1]};
    int which = 0;
    if (e == cudaSuccess && window_bits > 0) e = sptgb_radix_sort_u32(keys, vals, nb, window_bits, w->rtmp, &which, s);
    if (e != cudaSuccess) return e;
    const uint32_t *skeys = keys[which];
    e = cudaMemcpyAsync(perm, vals[which], nb * 4, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    uint64_t g = (nb + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    k_block_sizes<<<(unsigned)g, 256, 0, s>>>(perm, bptr, nb, w->flags);
    sptgb_count_launch(1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = sptgb_exclusive_scan_u32(w->flags, pnnz, nb, pnnz + nb, w->stmp, s);
    const uint32_t *ia[1] = {skeys};
    if (e == cudaSuccess) e = sptgb_mark_groups(ia, 1, 0, nb, w->flags, s);
    uint32_t *dn = w->pos + nb;   // pos has nb + 1 entries
    if (e == cudaSuccess) e = sptgb_exclusive_scan_u32(w->flags, w->pos, nb, dn, w->stmp, s);
    if (e == cudaSuccess) e = sptgb_compact_starts(w->flags, w->pos, nb, wst, s);
    uint32_t nwin = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nwin, dn, sizeof nwin, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    const uint64_t end = nb;
    e = cudaMemcpyAsync(wst + nwin, &end, sizeof end, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    *nwin_out = nwin;
    // the heavy windows, ascending
    uint64_t gw = (nwin + 255) / 256;
    if (gw > (uint64_t)sptgb_sm_count() * 16) gw = (uint64_t)sptgb_sm_count() * 16;
    k_window_heavy<<<(unsigned)gw, 256, 0, s>>>(wst, pnnz, nwin, heavy_nnz, w->flags);
    sptgb_count_launch(1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = sptgb_exclusive_scan_u32(w->flags, w->pos, nwin, dn, w->stmp, s);
    if (e == cudaSuccess) e = sptgb_compact_starts(w->flags, w->pos, nwin, heavy, s);
    uint32_t nh = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nh, dn, sizeof nh, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) *nheavy_out = nh;
    return e;
}

// *bad = 1 unless bptr[0] == 0, bptr[nb] == nnz and bptr is non-decreasing.
__global__ void k_bptr_check(const uint64_t *__restrict__ bptr, uint64_t nb, uint64_t nnz, unsigned int *bad) {
    unsigned int b = 0;
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i0 == 0) b = bptr[0] != 0 || bptr[nb] != nnz;
    for (uint64_t i = i0; i < nb; i += (uint64_t)gridDim.x * blockDim.x) b |= bptr[i + 1] < bptr[i];
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1u);
}

extern "C" cudaError_t sptgb_hicoo_check_bptr(const uint64_t *bptr, uint64_t nb, uint64_t nnz, unsigned int *bad,
                                              cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess || nb == 0) return e;
    uint64_t g = (nb + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    k_bptr_check<<<(unsigned)g, 256, 0, s>>>(bptr, nb, nnz, bad);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_hicoo_check(const sptgb_hicoo_args *a, cudaStream_t s) {
    if (a->nb == 0) return cudaSuccess;
    uint64_t g = (a->nb + 255) / 256;
    if (g > (uint64_t)sptgb_sm_count() * 16) g = (uint64_t)sptgb_sm_count() * 16;
    k_hicoo_check<<<(unsigned)g, 256, 0, s>>>(a->bptr, *a, a->nb);
    sptgb_count_launch(1);
    return cudaGetLastError();
}
