// Sparse tensor times matrix on the GPU (sptSparseTensorMulMatrix,
// src/sptensor/mmul.c:37-97).
//
// X is sorted with `mode` last, so the nonzeros of one output fiber (equal
// coordinates in every other mode) are consecutive: fiber f owns nonzeros
// [starts[f], starts[f+1]).  A worker of W lanes takes one fiber; lane l
// holds output columns 4l..4l+3 (+ 4W per further pass when ncols > 4W) and
// accumulates y = y + v * U[i_mode, :] over the fiber's nonzeros in order,
// with the multiply and the add rounded separately, which is the reference's
// loop (mmul.c:81-89) operation for operation.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"

namespace {

constexpr int BLOCK = 256;

template <int W>
__global__ void __launch_bounds__(BLOCK) k_ttm(const uint64_t *__restrict__ starts, uint64_t nfib, uint64_t nnz,
                                               const uint32_t *__restrict__ rows, const float *__restrict__ vals,
                                               const float *__restrict__ U, uint32_t ustride, uint32_t ncols,
                                               float *__restrict__ Y, uint32_t ystride) {
    const int sl = (threadIdx.x & 31) % W;
    const uint64_t worker = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) / W;
    const uint64_t nworkers = ((uint64_t)gridDim.x * BLOCK) / W;
    for (uint64_t f = worker; f < nfib; f += nworkers) {
        const uint64_t z0 = starts[f], z1 = f + 1 < nfib ? starts[f + 1] : nnz;
        for (uint32_t c0 = (uint32_t)sl * 4; c0 < ncols; c0 += 4 * W) {
            float y0 = 0.f, y1 = 0.f, y2 = 0.f, y3 = 0.f;
            for (uint64_t z = z0; z < z1; ++z) {
                const float v = vals[z];
                const float *u = U + (size_t)rows[z] * ustride + c0;
                y0 = __fadd_rn(y0, __fmul_rn(v, __ldg(u + 0)));
                if (c0 + 1 < ncols) y1 = __fadd_rn(y1, __fmul_rn(v, __ldg(u + 1)));
                if (c0 + 2 < ncols) y2 = __fadd_rn(y2, __fmul_rn(v, __ldg(u + 2)));
                if (c0 + 3 < ncols) y3 = __fadd_rn(y3, __fmul_rn(v, __ldg(u + 3)));
            }
            float *y = Y + (size_t)f * ystride + c0;
            y[0] = y0;
            if (c0 + 1 < ncols) y[1] = y1;
            if (c0 + 2 < ncols) y[2] = y2;
            if (c0 + 3 < ncols) y[3] = y3;
        }
    }
}

template <int W>
cudaError_t launch(const uint64_t *starts, uint64_t nfib, uint64_t nnz, const uint32_t *rows, const float *vals,
                   const float *U, uint32_t ustride, uint32_t ncols, float *Y, uint32_t ystride, cudaStream_t s) {
    uint64_t blocks = (nfib * W + BLOCK - 1) / BLOCK;
    if (blocks > (uint64_t)sptgb_sm_count() * 8) blocks = (uint64_t)sptgb_sm_count() * 8;
    if (blocks < 1) blocks = 1;
    k_ttm<W><<<(unsigned)blocks, BLOCK, 0, s>>>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

}  // namespace

extern "C" cudaError_t sptgb_ttm(const uint64_t *starts, uint64_t nfib, uint64_t nnz, const uint32_t *rows,
                                 const float *vals, const float *U, uint32_t ustride, uint32_t ncols, float *Y,
                                 uint32_t ystride, cudaStream_t s) {
    if (nfib == 0 || ncols == 0) return cudaSuccess;
    const uint32_t c4 = (ncols + 3) / 4;
    if (c4 <= 2) return launch<2>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride, s);
    if (c4 <= 4) return launch<4>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride, s);
    if (c4 <= 8) return launch<8>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride, s);
    if (c4 <= 16) return launch<16>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride, s);
    return launch<32>(starts, nfib, nnz, rows, vals, U, ustride, ncols, Y, ystride, s);
}
