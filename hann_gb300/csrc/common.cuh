// common.cuh -- shared device helpers for the hann_gb300 PQIVF kernels.
//
// Exact FP32 distances on the device reproduce the summation order of the
// reference's NEON tier (core/simd_kernels.inc.h:64-102 instantiated by
// core/simd_kernels_neon.inc.h): element i of the unrolled part accumulates
// into chain (u, l) = ((i % 16) / 4, i % 4) with a fused multiply-add; the
// one-vector cleanup loop continues chain (0, l); the chains combine as
// (c0 + c1) + (c2 + c3) per lane, the four lanes as (l0 + l1) + (l2 + l3),
// and the scalar tail adds (a - b)^2 as a separate multiply and add. The
// Grace host that sits beside the GB300 runs exactly this tier, so a device
// distance is bit-identical to the reference's CPU distance on that host.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hann {

// ---------------------------------------------------------------------------
// Reference-order squared Euclidean distance, generic length.
// a and b may live in any address space; the loop order is fixed.
template <typename PA, typename PB>
__device__ __forceinline__ float sqeuclid_ref(PA a, PB b, int n) {
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[u][l] = 0.0f;
    int i = 0;
    const int lim4 = n - (n % 16);
    for (; i < lim4; i += 16) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int l = 0; l < 4; l++) {
                float d = a[i + 4 * u + l] - b[i + 4 * u + l];
                acc[u][l] = __fmaf_rn(d, d, acc[u][l]);
            }
    }
    const int lim = n - (n % 4);
    for (; i < lim; i += 4) {
#pragma unroll
        for (int l = 0; l < 4; l++) {
            float d = a[i + l] - b[i + l];
            acc[0][l] = __fmaf_rn(d, d, acc[0][l]);
        }
    }
    float v[4];
#pragma unroll
    for (int l = 0; l < 4; l++)
        v[l] = __fadd_rn(__fadd_rn(acc[0][l], acc[1][l]), __fadd_rn(acc[2][l], acc[3][l]));
    float sum = __fadd_rn(__fadd_rn(v[0], v[1]), __fadd_rn(v[2], v[3]));
    for (; i < n; i++) {
        float d = a[i] - b[i];
        sum = __fadd_rn(sum, __fmul_rn(d, d));
    }
    return sum;
}

// sqeuclid_ref with b read as float4 (b 16-byte aligned, as every row of a
// row-major matrix with dim % 4 == 0 is): same arithmetic, same order, fewer
// and wider loads.
template <typename PA>
__device__ __forceinline__ float sqeuclid_ref_v4(PA a, const float* __restrict__ b, int n) {
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[u][l] = 0.0f;
    const float4* b4 = reinterpret_cast<const float4*>(b);
    int i = 0;
    const int lim4 = n - (n % 16);
    for (; i < lim4; i += 16) {
        float bb[16];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float4 v = __ldg(b4 + (i >> 2) + u);
            bb[4 * u + 0] = v.x;
            bb[4 * u + 1] = v.y;
            bb[4 * u + 2] = v.z;
            bb[4 * u + 3] = v.w;
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int l = 0; l < 4; l++) {
                float d = a[i + 4 * u + l] - bb[4 * u + l];
                acc[u][l] = __fmaf_rn(d, d, acc[u][l]);
            }
    }
    const int lim = n - (n % 4);
    for (; i < lim; i += 4) {
        const float4 v = __ldg(b4 + (i >> 2));
        const float bb[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int l = 0; l < 4; l++) {
            float d = a[i + l] - bb[l];
            acc[0][l] = __fmaf_rn(d, d, acc[0][l]);
        }
    }
    float v[4];
#pragma unroll
    for (int l = 0; l < 4; l++)
        v[l] = __fadd_rn(__fadd_rn(acc[0][l], acc[1][l]), __fadd_rn(acc[2][l], acc[3][l]));
    float sum = __fadd_rn(__fadd_rn(v[0], v[1]), __fadd_rn(v[2], v[3]));
    for (; i < n; i++) {
        float d = a[i] - b[i];
        sum = __fadd_rn(sum, __fmul_rn(d, d));
    }
    return sum;
}

// Reference-order Manhattan distance (core/simd_kernels.inc.h:115-149, NEON).
template <typename PA, typename PB>
__device__ __forceinline__ float manhattan_ref(PA a, PB b, int n) {
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[u][l] = 0.0f;
    int i = 0;
    const int lim4 = n - (n % 16);
    for (; i < lim4; i += 16) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int l = 0; l < 4; l++)
                acc[u][l] = __fadd_rn(acc[u][l], fabsf(a[i + 4 * u + l] - b[i + 4 * u + l]));
    }
    const int lim = n - (n % 4);
    for (; i < lim; i += 4) {
#pragma unroll
        for (int l = 0; l < 4; l++) acc[0][l] = __fadd_rn(acc[0][l], fabsf(a[i + l] - b[i + l]));
    }
    float v[4];
#pragma unroll
    for (int l = 0; l < 4; l++)
        v[l] = __fadd_rn(__fadd_rn(acc[0][l], acc[1][l]), __fadd_rn(acc[2][l], acc[3][l]));
    float sum = __fadd_rn(__fadd_rn(v[0], v[1]), __fadd_rn(v[2], v[3]));
    for (; i < n; i++) sum = __fadd_rn(sum, fabsf(a[i] - b[i]));
    return sum;
}

// Reference-order dot product of the cosine kernel's accumulations
// (core/simd_kernels.inc.h:153-219, NEON); the scalar tail is fused there.
template <typename PA, typename PB>
__device__ __forceinline__ float dot_ref(PA a, PB b, int n) {
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 4; l++) acc[u][l] = 0.0f;
    int i = 0;
    const int lim4 = n - (n % 16);
    for (; i < lim4; i += 16) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int l = 0; l < 4; l++) acc[u][l] = __fmaf_rn(a[i + 4 * u + l], b[i + 4 * u + l], acc[u][l]);
    }
    const int lim = n - (n % 4);
    for (; i < lim; i += 4) {
#pragma unroll
        for (int l = 0; l < 4; l++) acc[0][l] = __fmaf_rn(a[i + l], b[i + l], acc[0][l]);
    }
    float v[4];
#pragma unroll
    for (int l = 0; l < 4; l++)
        v[l] = __fadd_rn(__fadd_rn(acc[0][l], acc[1][l]), __fadd_rn(acc[2][l], acc[3][l]));
    float sum = __fadd_rn(__fadd_rn(v[0], v[1]), __fadd_rn(v[2], v[3]));
    for (; i < n; i++) sum = __fmaf_rn(a[i], b[i], sum);
    return sum;
}

// Cosine distance from the three reference-order accumulations: zero norm
// gives 1, the similarity is clamped to [-1, 1] (core/simd_kernels.inc.h:220-228).
__device__ __forceinline__ float cosine_from_parts(float dot, float na, float nb) {
    float A = __fsqrt_rn(na), B = __fsqrt_rn(nb);
    if (A == 0.0f || B == 0.0f) return 1.0f;
    float s = __fdiv_rn(dot, __fmul_rn(A, B));
    s = fminf(fmaxf(s, -1.0f), 1.0f);
    return __fsub_rn(1.0f, s);
}

// ---------------------------------------------------------------------------
// Order-preserving map of a float to an unsigned key (smaller float, smaller
// key), so thresholds can be kept with integer atomics.
__device__ __forceinline__ uint32_t float_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Candidates rescored exactly per query: k + 32 for the reference's PQ
// distances (mode 0), max(4k, 64) for the raw-vector rerank (mode 1), a
// multiple of 32; `fixed` > 0 overrides. A query's depth depends only on its
// own k, so its result does not depend on the batch it runs in.
__host__ __device__ __forceinline__ int rerank_depth_for(int k, int mode, int fixed) {
    if (fixed > 0) return fixed > k ? fixed : k;
    const int r = mode == 0 ? k + 32 : (4 * k > 64 ? 4 * k : 64);
    return (r + 31) / 32 * 32;
}

// Bound on |s~ - s| for the BF16 ranking score s = ||b||^2 - 2<a, b>
// (an = |a|, ar = |a - a~|, bmax = max|b|, brmax = max|b - b~|, a~ and b~
// the BF16 roundings, kp the padded length):
//   operand rounding      2 (ar bmax + |a~| brmax)       (Cauchy-Schwarz)
//   FP32 accumulation     2 kp 2^-22 |a~| |b~|
//   FP32 ||b||^2          kp 2^-23 bmax^2
//   score rounding        2^-22 (bmax^2 + 2 |a~| bmax)
__host__ __device__ __forceinline__ float bf16_score_eps(float an, float ar, float bmax, float brmax, int kp) {
    const float at = an + ar, bt = bmax + brmax;
    const float u22 = 2.384185791015625e-7f, u23 = 1.1920928955078125e-7f;
    return 2.0f * (ar * bmax + at * brmax) + 2.0f * (float)kp * u22 * at * bt + (float)kp * u23 * bmax * bmax +
           u22 * (bmax * bmax + 2.0f * at * bmax);
}

}  // namespace hann
