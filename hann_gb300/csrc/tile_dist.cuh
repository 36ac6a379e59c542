// tile_dist.cuh -- register-tiled exact FP32 distances in the reference's
// summation order, shared by k-means assignment and the batched k-NN.
//
// A thread owns 4 rows x 4 columns. Rows sit in shared memory element-major
// (Xs[i * TP + row]), columns likewise (Cs[i * TC + col]); per element one
// float4 of rows and one float4 of columns feed all 16 pairs. The sixteen
// accumulation chains of the reference's NEON tier (core/simd_kernels.inc.h:
// 64-102, LANES = 4, four accumulators) are walked one chain at a time for
// all 16 pairs, so every pair sees exactly the reference's order:
//   element i of the unrolled part -> chain (u, l) = ((i % 16) / 4, i % 4)
//   one-vector cleanup             -> chain (0, l)
//   combine                        -> ((c0 + c1) + (c2 + c3)) per lane,
//                                     (l0 + l1) + (l2 + l3) over lanes
//   scalar tail                    -> added one element at a time.
// OP selects the per-element step:
//   OP_SQDIFF  d = a - b; acc = fma(d, d, acc); tail acc + d*d (unfused)
//   OP_ABSDIFF acc = acc + |a - b|; tail the same
//   OP_DOT     acc = fma(a, b, acc); tail fused as well
#pragma once

#include "common.cuh"

namespace hann {

constexpr int OP_SQDIFF = 0;
constexpr int OP_ABSDIFF = 1;
constexpr int OP_DOT = 2;

template <int OP>
__device__ __forceinline__ float tile_step(float a, float b, float acc) {
    if (OP == OP_SQDIFF) {
        const float d = a - b;
        return __fmaf_rn(d, d, acc);
    } else if (OP == OP_ABSDIFF) {
        return __fadd_rn(acc, fabsf(a - b));
    } else {
        return __fmaf_rn(a, b, acc);
    }
}

template <int OP>
__device__ __forceinline__ float tile_tail(float a, float b, float acc) {
    if (OP == OP_SQDIFF) {
        const float d = a - b;
        return __fadd_rn(acc, __fmul_rn(d, d));
    } else if (OP == OP_ABSDIFF) {
        return __fadd_rn(acc, fabsf(a - b));
    } else {
        return __fmaf_rn(a, b, acc);
    }
}

struct Acc16 {
    float v[4][4];
};

template <int OP, int TP, int TC>
__device__ __forceinline__ void chain16(const float* __restrict__ Xs, const float* __restrict__ Cs, int tp, int tc,
                                        int u, int l, int t16, int lim4, int s4, Acc16& acc) {
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc.v[a][b] = 0.0f;
    for (int t = 0; t < t16; t++) {
        const int i = 16 * t + 4 * u + l;
        const float4 xp = *reinterpret_cast<const float4*>(Xs + i * TP + 4 * tp);
        const float4 cc = *reinterpret_cast<const float4*>(Cs + i * TC + 4 * tc);
        const float xa[4] = {xp.x, xp.y, xp.z, xp.w};
        const float cb[4] = {cc.x, cc.y, cc.z, cc.w};
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc.v[a][b] = tile_step<OP>(xa[a], cb[b], acc.v[a][b]);
    }
    if (u == 0) {
        for (int s = 0; s < s4; s++) {
            const int i = lim4 + 4 * s + l;
            const float4 xp = *reinterpret_cast<const float4*>(Xs + i * TP + 4 * tp);
            const float4 cc = *reinterpret_cast<const float4*>(Cs + i * TC + 4 * tc);
            const float xa[4] = {xp.x, xp.y, xp.z, xp.w};
            const float cb[4] = {cc.x, cc.y, cc.z, cc.w};
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc.v[a][b] = tile_step<OP>(xa[a], cb[b], acc.v[a][b]);
        }
    }
}

// Reference-order results of the thread's 16 pairs for the current tiles.
template <int OP, int TP, int TC>
__device__ __forceinline__ void tile_pairs(const float* __restrict__ Xs, const float* __restrict__ Cs, int tp,
                                           int tc, int dim, float out[4][4]) {
    const int lim4 = dim - (dim % 16);
    const int lim = dim - (dim % 4);
    const int t16 = lim4 / 16;
    const int s4 = (lim - lim4) / 4;
    Acc16 acc, c01, c2;
    float v01[4][4], v2[4][4];
#pragma unroll 1
    for (int l = 0; l < 4; l++) {
        chain16<OP, TP, TC>(Xs, Cs, tp, tc, 0, l, t16, lim4, s4, acc);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) c01.v[a][b] = acc.v[a][b];
        chain16<OP, TP, TC>(Xs, Cs, tp, tc, 1, l, t16, lim4, s4, acc);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) c01.v[a][b] = __fadd_rn(c01.v[a][b], acc.v[a][b]);
        chain16<OP, TP, TC>(Xs, Cs, tp, tc, 2, l, t16, lim4, s4, acc);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) c2.v[a][b] = acc.v[a][b];
        chain16<OP, TP, TC>(Xs, Cs, tp, tc, 3, l, t16, lim4, s4, acc);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) {
                float vl = __fadd_rn(c01.v[a][b], __fadd_rn(c2.v[a][b], acc.v[a][b]));
                if (l == 0) v01[a][b] = vl;
                else if (l == 1) v01[a][b] = __fadd_rn(v01[a][b], vl);
                else if (l == 2) v2[a][b] = vl;
                else out[a][b] = __fadd_rn(v01[a][b], __fadd_rn(v2[a][b], vl));
            }
    }
    for (int i = lim; i < dim; i++) {
        const float4 xp = *reinterpret_cast<const float4*>(Xs + i * TP + 4 * tp);
        const float4 cc = *reinterpret_cast<const float4*>(Cs + i * TC + 4 * tc);
        const float xa[4] = {xp.x, xp.y, xp.z, xp.w};
        const float cb[4] = {cc.x, cc.y, cc.z, cc.w};
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) out[a][b] = tile_tail<OP>(xa[a], cb[b], out[a][b]);
    }
}

// Stage rows [0, valid) of a row-major matrix (leading dimension dim) into
// an element-major tile T[i * TR + r] (TR rows wide), zero past `valid`
// (valid >= 1). Consecutive threads take consecutive rows, so the
// shared-memory stores are conflict-free; when dim is a multiple of 4 and
// the rows are 16-byte aligned each thread moves a float4. src(r) gives the
// global row pointer of tile row r (all rows share one base).
template <int TR, int THREADS, typename RowPtr>
__device__ __forceinline__ void stage_tile(float* __restrict__ T, int dim, int valid, RowPtr src) {
    if ((dim & 3) == 0 && (reinterpret_cast<uintptr_t>(src(0)) & 15) == 0) {
        const int d4 = dim >> 2;
        for (int e = threadIdx.x; e < TR * d4; e += THREADS) {
            const int r = e % TR, i4 = e / TR;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (r < valid) v = *reinterpret_cast<const float4*>(src(r) + 4 * i4);
            T[(4 * i4 + 0) * TR + r] = v.x;
            T[(4 * i4 + 1) * TR + r] = v.y;
            T[(4 * i4 + 2) * TR + r] = v.z;
            T[(4 * i4 + 3) * TR + r] = v.w;
        }
    } else {
        for (int e = threadIdx.x; e < TR * dim; e += THREADS) {
            const int r = e % TR, i = e / TR;
            T[i * TR + r] = r < valid ? src(r)[i] : 0.0f;
        }
    }
}

}  // namespace hann
