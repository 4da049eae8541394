// HiCOO MTTKRP for sm_103a (sptMTTKRPHiCOO, src/sptensor/hicoo/mttkrp.c:53-144).
//
// A worker (W lanes, one float4 column group per lane) owns one HiCOO block
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

template <int W>
cudaError_t launch(const sptgb_hicoo_args &a, cudaStream_t s) {
    static int max_blocks = 0;
    if (max_blocks == 0) {
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mttkrp_hicoo<W>, BLOCK, 0);
        max_blocks = (per_sm < 1 ? 1 : per_sm) * nsm;
    }
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
    if (c4 <= 2) return launch<2>(*a, s);
    if (c4 <= 4) return launch<4>(*a, s);
    if (c4 <= 8) return launch<8>(*a, s);
    if (c4 <= 16) return launch<16>(*a, s);
    return launch<32>(*a, s);
}
