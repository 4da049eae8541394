// Text tensor ingest on the device (sptLoadSparseTensor, src/sptensor/load.c:31-84).
//
// The reference reads whitespace-separated tokens with fscanf: N unsigned
// indices and one double per nonzero, line breaks carry no meaning.  Here a
// chunk of the file body is copied to the device; token starts (a non-space
// byte after a space) are flagged, scanned and compacted; then one thread
// parses one token into (record, field) = (token / (N+1), token % (N+1)).
//   indices: optional '+', decimal digits, value < 2^32 (else the token is
//            invalid);
//   values:  [sign] digits [. digits] [e|E [sign] digits]; when the decimal
//            significand has at most 19 digits, fits 2^53 and the power of ten
//            is at most 22 in magnitude, value = m * 10^e (or m / 10^-e) in
//            double is the correctly rounded result (both operands exact, one
//            rounding); any other value token is handed to the host, which
//            parses it as fscanf("%lf") would (strtod on the token).
// The first invalid token ends the tensor, as a failing fscanf does.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../sptgb_internal.h"

namespace {

__device__ __forceinline__ bool is_space(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

__global__ void k_token_flags(const unsigned char *__restrict__ buf, uint64_t n, uint32_t *__restrict__ flags) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        flags[i] = !is_space(buf[i]) && (i == 0 || is_space(buf[i - 1]));
}

__device__ const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                      1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// 0: parsed; 1: needs the host parser; 2: invalid.
__device__ int parse_double(const unsigned char *p, const unsigned char *end, double *out) {
    bool neg = false;
    if (p < end && (*p == '+' || *p == '-')) {
        neg = *p == '-';
        ++p;
    }
    if (p < end && !(*p >= '0' && *p <= '9') && *p != '.') return 1;   // inf, nan, hex: host
    uint64_t m = 0;
    int digits = 0, exp10 = 0;
    bool any = false, exact = true;
    while (p < end && *p >= '0' && *p <= '9') {
        any = true;
        if (m == 0 && *p == '0') {
            ++p;
            continue;
        }
        if (digits < 19) {
            m = m * 10 + (*p - '0');
            ++digits;
        } else {
            exact = false;
            ++exp10;
        }
        ++p;
    }
    if (p < end && *p == '.') {
        ++p;
        while (p < end && *p >= '0' && *p <= '9') {
            any = true;
            if (m == 0 && *p == '0') {
                --exp10;
                ++p;
                continue;
            }
            if (digits < 19) {
                m = m * 10 + (*p - '0');
                ++digits;
                --exp10;
            } else {
                exact = false;
            }
            ++p;
        }
    }
    if (!any) return 2;
    if (p < end && (*p == 'e' || *p == 'E')) {
        ++p;
        bool eneg = false;
        if (p < end && (*p == '+' || *p == '-')) {
            eneg = *p == '-';
            ++p;
        }
        if (p >= end || !(*p >= '0' && *p <= '9')) return 1;
        int e = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            if (e < 100000) e = e * 10 + (*p - '0');
            ++p;
        }
        exp10 += eneg ? -e : e;
    }
    if (p != end) return 2;
    if (m == 0) {
        *out = neg ? -0.0 : 0.0;
        return 0;
    }
    if (!exact || m > (1ull << 53) || exp10 > 22 || exp10 < -22) return 1;
    double v = (double)m;
    v = exp10 >= 0 ? v * kPow10[exp10] : v / kPow10[-exp10];
    *out = neg ? -v : v;
    return 0;
}

__device__ int parse_u32(const unsigned char *p, const unsigned char *end, uint32_t *out) {
    if (p < end && *p == '+') ++p;
    if (p >= end) return 2;
    uint64_t v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        if (v > 0xffffffffull) return 2;
        ++p;
    }
    if (p != end) return 2;
    *out = (uint32_t)v;
    return 0;
}

__global__ void k_parse_tokens(const unsigned char *__restrict__ buf, uint64_t n, const uint64_t *__restrict__ starts,
                               uint64_t ntok, uint64_t base_tok, sptgb_ingest_out o) {
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntok;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t gt = base_tok + t;
        const uint64_t rec = gt / (o.nmodes + 1);
        const uint32_t f = (uint32_t)(gt % (o.nmodes + 1));
        if (rec >= o.max_records) continue;
        const unsigned char *p = buf + starts[t];
        const unsigned char *end = p;
        while (end < buf + n && !is_space(*end)) ++end;
        if (f < o.nmodes) {
            uint32_t v = 0;
            if (parse_u32(p, end, &v) != 0) {
                atomicMin(reinterpret_cast<unsigned long long *>(o.first_bad), (unsigned long long)gt);
                continue;
            }
            if (v < o.start_index) atomicMin(reinterpret_cast<unsigned long long *>(o.first_below), (unsigned long long)gt);
            o.inds[f][rec] = v - o.start_index;
        } else {
            double d = 0.0;
            const int r = parse_double(p, end, &d);
            if (r != 0) {   // other spellings (hex, inf, nan, trailing bytes): the host decides
                const unsigned long long k = atomicAdd(reinterpret_cast<unsigned long long *>(o.nslow), 1ull);
                if (k < o.slow_cap) {
                    o.slow_rec[k] = rec;
                    o.slow_off[k] = o.base_off + starts[t];
                }
            } else {
                o.vals[rec] = (float)d;
            }
        }
    }
}

__global__ void k_segment_sums(const uint64_t *__restrict__ starts, uint64_t ng, uint64_t n,
                               const float *__restrict__ vals, float *__restrict__ out) {
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < ng; g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = g + 1 < ng ? starts[g + 1] : n;
        float acc = 0.f;
        for (uint64_t i = starts[g]; i < e; ++i) acc += vals[i];
        out[g] = acc;
    }
}

unsigned grid_for(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    if (b > (uint64_t)sptgb_sm_count() * 16) b = (uint64_t)sptgb_sm_count() * 16;
    return b ? (unsigned)b : 1u;
}

}  // namespace

extern "C" cudaError_t sptgb_ingest_token_starts(const void *buf, uint64_t n, uint32_t *flags, uint32_t *pos,
                                                 uint32_t *ntok, void *scan_tmp, uint64_t *starts, cudaStream_t s) {
    if (n == 0) return cudaMemsetAsync(ntok, 0, sizeof(uint32_t), s);
    k_token_flags<<<grid_for(n), 256, 0, s>>>(static_cast<const unsigned char *>(buf), n, flags);
    sptgb_count_launch(1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = sptgb_exclusive_scan_u32(flags, pos, n, ntok, scan_tmp, s);
    if (e == cudaSuccess) e = sptgb_compact_starts(flags, pos, n, starts, s);
    return e;
}

extern "C" cudaError_t sptgb_ingest_parse(const void *buf, uint64_t n, const uint64_t *starts, uint64_t ntok,
                                          uint64_t base_tok, const sptgb_ingest_out *o, cudaStream_t s) {
    if (ntok == 0) return cudaSuccess;
    k_parse_tokens<<<grid_for(ntok), 256, 0, s>>>(static_cast<const unsigned char *>(buf), n, starts, ntok, base_tok,
                                                  *o);
    sptgb_count_launch(1);
    return cudaGetLastError();
}

extern "C" cudaError_t sptgb_segment_sums(const uint64_t *starts, uint64_t ng, uint64_t n, const float *vals, float *out,
                                          cudaStream_t s) {
    if (ng == 0) return cudaSuccess;
    k_segment_sums<<<grid_for(ng), 256, 0, s>>>(starts, ng, n, vals, out);
    sptgb_count_launch(1);
    return cudaGetLastError();
}
