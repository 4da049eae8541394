// One work unit of the record-based segmented MTTKRP, shared by the
// single-tensor kernel (mttkrp_coo.cu) and the batched kernel (batch.cu).
//
// A worker of W lanes (lane sl holds columns [4sl, 4sl+4)) walks the records
// [start, start+len) of a mode-sorted copy in order:
//   NF = 2 (order 3): record {row, a, b, value bits}
//   NF = 3 (order 4): record {row, a, b, c}, value in vals[k]
// computes value * F_a[a] * F_b[b] (* F_c[c]) with packed FP32x2 arithmetic,
// keeps the running row sum in registers and writes a row when the output
// coordinate changes: a plain store for rows inside the unit, a vector atomic
// for the unit's first row when the previous unit ends in it and for its last
// row when the next unit starts in it (the output must be zero beforehand).
// Record batches of BATCH are software-pipelined: the next batch is loaded while
// the current batch's factor rows are gathered.  Padding columns (past the
// rank) are written as zero.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sptgb_mttkrp {

constexpr uint32_t NO_ROW = 0xffffffffu;

__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    uint64_t ra = *reinterpret_cast<uint64_t *>(&a), rb = *reinterpret_cast<uint64_t *>(&b), rd;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2 *>(&rd);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    uint64_t ra = *reinterpret_cast<uint64_t *>(&a), rb = *reinterpret_cast<uint64_t *>(&b);
    uint64_t rc = *reinterpret_cast<uint64_t *>(&c), rd;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    return *reinterpret_cast<float2 *>(&rd);
}

// COH: the rows may have been written earlier in the same kernel (the
// persistent batched step), so they are read through the coherent path
// instead of the read-only one.
template <bool BF16, bool COH = false>
__device__ __forceinline__ float4 gather_row(const char *base, uint32_t row, uint32_t row_bytes) {
    if (!BF16 && COH) return __ldca(reinterpret_cast<const float4 *>(base + (size_t)row * row_bytes));
    if (!BF16) return __ldg(reinterpret_cast<const float4 *>(base + (size_t)row * row_bytes));
    const uint2 u = __ldg(reinterpret_cast<const uint2 *>(base + (size_t)row * row_bytes));
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                       __uint_as_float(u.y & 0xffff0000u));
}

__device__ __forceinline__ void put_row(float *out, uint32_t row, uint32_t stride, int sl, float4 v, bool shared) {
    float4 *p = reinterpret_cast<float4 *>(out + (size_t)row * stride) + sl;
    if (shared)
        atomicAdd(p, v);
    else
        *p = v;
}

// F[i]: factor base already offset by this lane's columns (bytes).
template <bool BF16, bool FULL, int NF, int BATCH = 4, bool COH = false>
__device__ __forceinline__ void unit(const uint4 *__restrict__ rec, const float *__restrict__ vals,
                                     const char *const *F, uint32_t row_bytes, float *__restrict__ out, uint64_t nnz,
                                     uint64_t start, uint32_t len, uint32_t stride, uint32_t rank, int sl) {
    const bool col_ok = FULL || (uint32_t)(sl * 4) < stride;
    const bool masked = rank < stride;
    const int c0 = sl * 4;
    const uint4 *r0 = rec + start;
    const uint32_t prev = start > 0 ? rec[start - 1].x : NO_ROW;
    const uint32_t next = start + len < nnz ? rec[start + len].x : NO_ROW;
    uint32_t cur = r0[0].x;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);

    auto flush = [&](bool shared) {
        if (!col_ok) return;
        float4 v = acc;
        if (masked) {
            const int rk = (int)rank;
            v = make_float4(c0 + 0 < rk ? v.x : 0.f, c0 + 1 < rk ? v.y : 0.f, c0 + 2 < rk ? v.z : 0.f,
                            c0 + 3 < rk ? v.w : 0.f);
        }
        put_row(out, cur, stride, sl, v, shared);
    };
    auto gather = [&](const uint4 &q, float4 *f) {
        f[0] = col_ok ? gather_row<BF16, COH>(F[0], q.y, row_bytes) : make_float4(0.f, 0.f, 0.f, 0.f);
        f[1] = col_ok ? gather_row<BF16, COH>(F[1], q.z, row_bytes) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (NF == 3) f[2] = col_ok ? gather_row<BF16, COH>(F[2], q.w, row_bytes) : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    auto consume = [&](const uint4 &q, float v, const float4 *f) {
        if (q.x != cur) {
            flush(cur == prev);
            acc = make_float4(0.f, 0.f, 0.f, 0.f);
            cur = q.x;
        }
        float2 p0 = mul2(make_float2(v, v), make_float2(f[0].x, f[0].y));
        float2 p1 = mul2(make_float2(v, v), make_float2(f[0].z, f[0].w));
        if (NF == 3) {
            p0 = mul2(p0, make_float2(f[1].x, f[1].y));
            p1 = mul2(p1, make_float2(f[1].z, f[1].w));
        }
        const float4 &fl = f[NF - 1];
        const float2 s0 = fma2(p0, make_float2(fl.x, fl.y), make_float2(acc.x, acc.y));
        const float2 s1 = fma2(p1, make_float2(fl.z, fl.w), make_float2(acc.z, acc.w));
        acc = make_float4(s0.x, s0.y, s1.x, s1.y);
    };
    auto value = [&](const uint4 &q, uint32_t k) -> float { return NF == 2 ? __uint_as_float(q.w) : __ldg(vals + start + k); };

    uint32_t k = 0;
    uint4 qn[BATCH];
    if (len >= BATCH) {
#pragma unroll
        for (int j = 0; j < BATCH; ++j) qn[j] = __ldg(r0 + j);
    }
    for (; k + BATCH <= len; k += BATCH) {
        uint4 q[BATCH];
        float4 f[BATCH][NF];
#pragma unroll
        for (int j = 0; j < BATCH; ++j) q[j] = qn[j];
#pragma unroll
        for (int j = 0; j < BATCH; ++j) gather(q[j], f[j]);
        if (k + 2 * BATCH <= len) {
#pragma unroll
            for (int j = 0; j < BATCH; ++j) qn[j] = __ldg(r0 + k + BATCH + j);
        }
#pragma unroll
        for (int j = 0; j < BATCH; ++j) consume(q[j], value(q[j], k + j), f[j]);
    }
    for (; k < len; ++k) {
        const uint4 q = __ldg(r0 + k);
        float4 f[NF];
        gather(q, f);
        consume(q, value(q, k), f);
    }
    flush(cur == prev || cur == next);
}

}  // namespace sptgb_mttkrp
