// Squared Frobenius norm of a COO tensor's values without any device
// allocation.
//
// Who needs this: a caller whose device memory is owned by someone else --
// an application that reserves the whole device memory pool up front for its
// own allocator and forbids further cudaMalloc calls, or a latency-critical
// caller that cannot afford the implicit synchronisation and cost of
// cudaMalloc/cudaFree on every call -- still wants ||X||^2 (the first term of
// the CP-ALS fit).  The allocating entry point, SparseTensorFrobeniusNormSquared,
// allocates a device copy of the values and its reduction partials per call;
// this variant stages both in one fixed array that is part of the library
// image instead.
//
// The scratch is a file-scope static __device__ array of 16 MiB + 2688 bytes
// (room for 4,194,304 float values, 304 partial sums and the result): every GPU
// that loads the library holds it until the process exits.  Host code cannot
// use the array's name as a device address (on the host it names a stand-in),
// so every call looks the address up with cudaGetSymbolAddress on the device
// (and CUDA context) current in the calling thread; the lookup is cheap once
// the module is loaded, and no address outlives a context.  All calls share
// the array and it keeps the last call's contents: each call overwrites every
// partial slot and the result slot it reads, so nothing has to start at zero,
// and calls that overlap on the GPU (different streams or threads at the same
// time) race on the array and must be serialised by the caller.  Every call
// ends by synchronising its stream and copying the result into host memory,
// so it cannot be called while that stream is capturing a CUDA graph.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"
#include "../../../include/sptgb.h"

#define NA_MAX_VALUES (4u * 1024u * 1024u)
#define NA_BLOCKS SPTGB_NPART
#define NA_THREADS 256
#define NA_VALUES_BYTES ((size_t)NA_MAX_VALUES * sizeof(float))
#define NA_PART_OFFSET NA_VALUES_BYTES
#define NA_RESULT_OFFSET (NA_PART_OFFSET + (size_t)NA_BLOCKS * sizeof(double))
#define NA_SCRATCH_BYTES (NA_RESULT_OFFSET + 256)

static __device__ __align__(256) unsigned char g_sptgb_noalloc_scratch[NA_SCRATCH_BYTES];

namespace {

// Each of the NA_BLOCKS blocks writes its own partial slot (zero when it has
// no values), so no slot keeps a previous call's value.
__global__ void __launch_bounds__(NA_THREADS)
k_na_sumsq_partial(const float *__restrict__ v, uint64_t n, double *__restrict__ part) {
    __shared__ double red[NA_THREADS];
    double s = 0.0;
    // FP32 products summed in FP64, as src/sptensor/sptensor.c:96-107
    for (uint64_t i = blockIdx.x * (uint64_t)NA_THREADS + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * NA_THREADS) {
        const float x = v[i];
        s += (double)__fmul_rn(x, x);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = NA_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_na_sum_final(const double *__restrict__ part, double *__restrict__ out) {
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < NA_BLOCKS; ++b) s += part[b];
        *out = s;
    }
}

// Device address of the scratch array in the current device's context,
// looked up on every call.
int na_scratch(unsigned char **ptr) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sptgb_noalloc_scratch);
    if (e != cudaSuccess) return sptgb_cuda_fail(e, "SpTns NormSq no-alloc", __FILE__, __LINE__);
    *ptr = static_cast<unsigned char *>(p);
    return 0;
}

}  // namespace

extern "C" int sptgbSparseTensorFrobeniusNormSquaredNoAlloc(sptSparseTensor const *spten, double *normsq,
                                                            void *stream) {
    const char *module = "SpTns NormSq no-alloc";
    const uint64_t n = spten->nnz;
    if (n > NA_MAX_VALUES) {
        spt_ComplainError(module, SPTERR_VALUE_ERROR, __FILE__, __LINE__,
                          "nnz exceeds the no-allocation limit of 4194304 values");
        return SPTERR_VALUE_ERROR;
    }
    unsigned char *base = nullptr;
    int r = na_scratch(&base);
    if (r) return r;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    float *dv = reinterpret_cast<float *>(base);
    double *part = reinterpret_cast<double *>(base + NA_PART_OFFSET);
    double *res = reinterpret_cast<double *>(base + NA_RESULT_OFFSET);
    cudaError_t e = cudaSuccess;
    if (n) e = cudaMemcpyAsync(dv, spten->values.data, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_na_sumsq_partial<<<NA_BLOCKS, NA_THREADS, 0, s>>>(dv, n, part);
        k_na_sum_final<<<1, 32, 0, s>>>(part, res);
        sptgb_count_launch(2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(normsq, res, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return sptgb_cuda_fail(e, module, __FILE__, __LINE__);
    return 0;
}
