// kernels_train.cu -- k-means assignment, FP64 centroid update, product
// quantizer assignment and encoding.
//
// Every argmin here uses the reference-order FP32 squared Euclidean distance
// (common.cuh) and lets the lowest index win a tie, as assignPoints and
// encodeWithCodebooks do (pqivf/index.go:641-666, 738-789). Centroid sums are
// FP64 on the device (the reference sums in FP32 in point order,
// pqivf/index.go:816-843); the mean is rounded once to FP32.
#include "hann_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "tile_dist.cuh"

#include <algorithm>

namespace hann {

// ---------------------------------------------------------------------------
// Tiled exact distances (tile_dist.cuh). A block owns TP points and walks
// every centroid in tiles of TC; each thread owns 4 points x 4 centroids.
constexpr int TD_THREADS = 256;
constexpr int TD_TP = 128;
constexpr int TD_TC = 32;
constexpr int TD_DMAX = 128;

// MODE 0: argmin per point. MODE 1: full distance matrix.
// The centroid range is split over gridDim.y blocks (tiles_per_split tiles
// each); with more than one split an argmin is combined across blocks by a
// 64-bit atomicMin on (distance key, index), which keeps the lowest index on
// a tie.
template <int MODE>
__global__ void __launch_bounds__(TD_THREADS) tile_dist_kernel(const float* __restrict__ x, int64_t n, int dim,
                                                               const float* __restrict__ cent, int k,
                                                               int tiles_per_split,
                                                               int32_t* __restrict__ out_idx,
                                                               float* __restrict__ out_dist,
                                                               float* __restrict__ out_mat,
                                                               unsigned long long* __restrict__ out_key) {
    extern __shared__ __align__(16) float sm[];
    float* Xs = sm;
    float* Cs = sm + dim * TD_TP;
    __shared__ float red_d[8][TD_TP];
    __shared__ int red_i[8][TD_TP];
    const int tid = threadIdx.x;
    const int tp = tid & 31, tc = tid >> 5;
    const int64_t p0 = (int64_t)blockIdx.x * TD_TP;
    stage_tile<TD_TP, TD_THREADS>(Xs, dim, (int)min((int64_t)TD_TP, n - p0),
                                  [&](int r) { return x + (p0 + r) * dim; });
    float best_d[4];
    int best_i[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        best_d[a] = __int_as_float(0x7f800000);
        best_i[a] = 0x7fffffff;
    }
    const int c_begin = blockIdx.y * tiles_per_split * TD_TC;
    const int c_end = min(k, c_begin + tiles_per_split * TD_TC);
    for (int c0 = c_begin; c0 < c_end; c0 += TD_TC) {
        __syncthreads();
        stage_tile<TD_TC, TD_THREADS>(Cs, dim, min(TD_TC, k - c0),
                                      [&](int r) { return cent + (int64_t)(c0 + r) * dim; });
        __syncthreads();
        float dd[4][4];
        tile_pairs<OP_SQDIFF, TD_TP, TD_TC>(Xs, Cs, tp, tc, dim, dd);
        if (MODE == 0) {
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int c = c0 + 4 * tc + b;
                    if (c < k && dd[a][b] < best_d[a]) {
                        best_d[a] = dd[a][b];
                        best_i[a] = c;
                    }
                }
        } else {
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int64_t gp = p0 + 4 * tp + a;
                if (gp >= n) continue;
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int c = c0 + 4 * tc + b;
                    if (c < k) out_mat[gp * k + c] = dd[a][b];
                }
            }
        }
    }
    if (MODE == 0) {
#pragma unroll
        for (int a = 0; a < 4; a++) {
            red_d[tc][4 * tp + a] = best_d[a];
            red_i[tc][4 * tp + a] = best_i[a];
        }
        __syncthreads();
        if (tid < TD_TP) {
            float bd = red_d[0][tid];
            int bi = red_i[0][tid];
            for (int w = 1; w < 8; w++) {
                const float d = red_d[w][tid];
                const int i = red_i[w][tid];
                if (d < bd || (d == bd && i < bi)) {
                    bd = d;
                    bi = i;
                }
            }
            const int64_t gp = p0 + tid;
            if (gp < n) {
                if (gridDim.y > 1) {
                    if (bi != 0x7fffffff)
                        atomicMin(&out_key[gp], ((unsigned long long)float_key(bd) << 32) | (uint32_t)bi);
                } else {
                    // No finite distance at all (NaN input): the reference
                    // keeps index 0 (pqivf/index.go:772-778).
                    out_idx[gp] = bi == 0x7fffffff ? 0 : bi;
                    if (out_dist) out_dist[gp] = bd;
                }
            }
        }
    }
}

// Generic path for dimensions above the tile limit: one thread per point.
template <int MODE>
__global__ void rowwise_dist_kernel(const float* __restrict__ x, int64_t n, int dim, const float* __restrict__ cent,
                                    int k, int32_t* __restrict__ out_idx, float* __restrict__ out_dist,
                                    float* __restrict__ out_mat) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* xp = x + p * dim;
    float bd = __int_as_float(0x7f800000);
    int bi = 0;
    for (int c = 0; c < k; c++) {
        const float d = sqeuclid_ref(xp, cent + (int64_t)c * dim, dim);
        if (MODE == 0) {
            if (c == 0 || d < bd) {
                bd = d;
                bi = c;
            }
        } else {
            out_mat[p * k + c] = d;
        }
    }
    if (MODE == 0) {
        out_idx[p] = bi;
        if (out_dist) out_dist[p] = bd;
    }
}

__global__ void unpack_argmin_kernel(const unsigned long long* __restrict__ key, int64_t n, int32_t* __restrict__ idx,
                                     float* __restrict__ dist) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const unsigned long long v = key[p];
    const bool none = v == ~0ull;
    idx[p] = none ? 0 : (int32_t)(uint32_t)(v & 0xffffffffull);
    if (dist) dist[p] = none ? __int_as_float(0x7fc00000) : key_float((uint32_t)(v >> 32));
}

template <int MODE>
static cudaError_t launch_tile(const float* x, int64_t n, int dim, const float* cent, int k, int32_t* out_idx,
                               float* out_dist, float* out_mat, unsigned long long* key_scratch, cudaStream_t s) {
    if (n <= 0 || k <= 0) return cudaSuccess;
    if (dim <= TD_DMAX) {
        const size_t smem = (size_t)dim * (TD_TP + TD_TC) * sizeof(float);
        static bool attr_set = false;
        if (!attr_set) {
            cudaError_t e = cudaFuncSetAttribute(tile_dist_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)((size_t)TD_DMAX * (TD_TP + TD_TC) * sizeof(float)));
            if (e != cudaSuccess) return e;
            attr_set = true;
        }
        const int64_t blocks = ceil_div(n, TD_TP);
        const int tiles = (int)ceil_div(k, TD_TC);
        // Enough blocks for two waves of one block per SM.
        int splits = (int)std::min<int64_t>(tiles, std::max<int64_t>(1, ceil_div(2 * 152, blocks)));
        if (MODE == 0 && key_scratch == nullptr) splits = 1;
        const int per = (int)ceil_div(tiles, splits);
        splits = (int)ceil_div(tiles, per);
        if (MODE == 0 && splits > 1) {
            cudaError_t e = cudaMemsetAsync(key_scratch, 0xff, (size_t)n * sizeof(unsigned long long), s);
            if (e != cudaSuccess) return e;
        }
        tile_dist_kernel<MODE><<<dim3((unsigned)blocks, (unsigned)splits), TD_THREADS, smem, s>>>(
            x, n, dim, cent, k, per, out_idx, out_dist, out_mat, key_scratch);
        if (MODE == 0 && splits > 1)
            unpack_argmin_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(key_scratch, n, out_idx, out_dist);
    } else {
        rowwise_dist_kernel<MODE><<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(x, n, dim, cent, k, out_idx, out_dist,
                                                                            out_mat);
    }
    return cudaGetLastError();
}

cudaError_t launch_assign_exact(const float* x, int64_t n, int dim, const float* cent, int k, int32_t* out_idx,
                                float* out_dist, unsigned long long* key_scratch, cudaStream_t s) {
    return launch_tile<0>(x, n, dim, cent, k, out_idx, out_dist, nullptr, key_scratch, s);
}

cudaError_t launch_dist_matrix(const float* q, int64_t nq, int dim, const float* cent, int k, float* out,
                               cudaStream_t s) {
    return launch_tile<1>(q, nq, dim, cent, k, nullptr, nullptr, out, nullptr, s);
}

// ---------------------------------------------------------------------------
// k-means update: FP64 sums by global atomics, then mean rounded to FP32.
__global__ void kmeans_accumulate_kernel(const float* __restrict__ x, int64_t n, int dim,
                                         const int32_t* __restrict__ assign, double* __restrict__ sums,
                                         int64_t* __restrict__ counts) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * dim) return;
    const int64_t p = e / dim;
    const int i = (int)(e - p * dim);
    const int c = assign[p];
    atomicAdd(&sums[(int64_t)c * dim + i], (double)x[e]);
    if (i == 0) atomicAdd(reinterpret_cast<unsigned long long*>(&counts[c]), 1ull);
}

cudaError_t launch_kmeans_accumulate(const float* x, int64_t n, int dim, const int32_t* assign, double* sums,
                                     int64_t* counts, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    kmeans_accumulate_kernel<<<(unsigned)ceil_div(n * dim, 256), 256, 0, s>>>(x, n, dim, assign, sums, counts);
    return cudaGetLastError();
}

__global__ void kmeans_finalize_kernel(const double* __restrict__ sums, const int64_t* __restrict__ counts, int k,
                                       int dim, float* __restrict__ cent) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)k * dim) return;
    const int64_t c = e / dim;
    const int64_t cnt = counts[c];
    if (cnt > 0) cent[e] = (float)(sums[e] / (double)cnt);
}

cudaError_t launch_kmeans_finalize(const double* sums, const int64_t* counts, int k, int dim, float* cent,
                                   cudaStream_t s) {
    if (k <= 0) return cudaSuccess;
    kmeans_finalize_kernel<<<(unsigned)ceil_div((int64_t)k * dim, 256), 256, 0, s>>>(sums, counts, k, dim, cent);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Product quantizer assignment: block = 256 points of one subquantizer, the
// codebook in shared memory, the sub-vector in registers.
template <int DSUB>
__global__ void __launch_bounds__(256) pq_assign_kernel(const float* __restrict__ res, int64_t n, int M,
                                                        const float* __restrict__ cb, int pqK, int m_begin,
                                                        int32_t* __restrict__ out) {
    extern __shared__ __align__(16) float scb[];
    const int m = m_begin + blockIdx.y;
    const int dim = M * DSUB;
    for (int e = threadIdx.x; e < pqK * DSUB; e += blockDim.x) scb[e] = cb[(int64_t)m * pqK * DSUB + e];
    __syncthreads();
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float sub[DSUB];
#pragma unroll
    for (int e = 0; e < DSUB; e++) sub[e] = res[p * dim + m * DSUB + e];
    float bd = sqeuclid_ref(sub, scb, DSUB);
    int bi = 0;
    for (int j = 1; j < pqK; j++) {
        const float d = sqeuclid_ref(sub, scb + j * DSUB, DSUB);
        if (d < bd) {
            bd = d;
            bi = j;
        }
    }
    out[p * M + m] = bi;
}

// Packed form for sub-dimensions 4, 8 and 16: two points a thread, every
// distance computed with the FP32x2 instructions (sub/mul/fma/add.rn.f32x2,
// each half rounded as the scalar instruction rounds it) in sqeuclid_ref's
// order. The codebook sits in shared memory with every float stored twice,
// so one 16-byte broadcast load gives two codeword coordinates already
// paired for both points. Every square is sqeuclid_ref's fma into a zero
// accumulator, written as that fma: a separate packed multiply followed by
// a packed add was fused into one fma by the compiler (one assignment in
// 300,000 moved by an ulp), which an fma cannot be. sqeuclid_ref's
// additions of the untouched zero accumulators for sub-dimensions below 16
// leave a sum of squares unchanged and are left out: the distances are
// sqeuclid_ref's bits.
using u64 = unsigned long long;
__device__ __forceinline__ u64 pk_sub(u64 a, u64 b) {
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// d * d rounded once, as fma(d, d, +0): exact for every d (d * d is never -0)
__device__ __forceinline__ u64 pk_sq(u64 d) {
    u64 r;
    asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(r) : "l"(d), "l"(0ull));
    return r;
}
__device__ __forceinline__ u64 pk_fma(u64 a, u64 b, u64 c) {
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ u64 pk_add(u64 a, u64 b) {
    u64 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 pk_pair(float lo, float hi) {
    return (u64)__float_as_uint(lo) | ((u64)__float_as_uint(hi) << 32);
}

template <int DSUB>
__device__ __forceinline__ u64 pk_sqeuclid(const u64 (&s)[DSUB], const ulonglong2* __restrict__ c) {
    u64 d[DSUB];
#pragma unroll
    for (int q = 0; q < DSUB / 2; q++) {
        const ulonglong2 w = c[q];
        d[2 * q] = pk_sub(s[2 * q], w.x);
        d[2 * q + 1] = pk_sub(s[2 * q + 1], w.y);
    }
    u64 v[4];
    if (DSUB == 4) {
#pragma unroll
        for (int l = 0; l < 4; l++) v[l] = pk_sq(d[l]);
    } else if (DSUB == 8) {
#pragma unroll
        for (int l = 0; l < 4; l++) v[l] = pk_fma(d[4 + l], d[4 + l], pk_sq(d[l]));
    } else {
#pragma unroll
        for (int l = 0; l < 4; l++)
            v[l] = pk_add(pk_add(pk_sq(d[l]), pk_sq(d[4 + l])), pk_add(pk_sq(d[8 + l]), pk_sq(d[12 + l])));
    }
    return pk_add(pk_add(v[0], v[1]), pk_add(v[2], v[3]));
}

constexpr int PQ_PACK_THREADS = 256;

template <int DSUB>
__global__ void __launch_bounds__(PQ_PACK_THREADS) pq_assign_packed_kernel(const float* __restrict__ res, int64_t n,
                                                                           int M, const float* __restrict__ cb,
                                                                           int pqK, int m_begin,
                                                                           int32_t* __restrict__ out) {
    extern __shared__ __align__(16) float scb2[];  // [pqK][DSUB][2]
    const int m = m_begin + blockIdx.y;
    const int dim = M * DSUB;
    for (int e = threadIdx.x; e < pqK * DSUB; e += blockDim.x) {
        const float v = cb[(int64_t)m * pqK * DSUB + e];
        scb2[2 * e] = v;
        scb2[2 * e + 1] = v;
    }
    __syncthreads();
    const int64_t p0 = (int64_t)blockIdx.x * (2 * PQ_PACK_THREADS) + threadIdx.x;
    const int64_t p1 = p0 + PQ_PACK_THREADS;
    if (p0 >= n) return;
    const bool has1 = p1 < n;
    u64 s[DSUB];
#pragma unroll
    for (int e = 0; e < DSUB; e++)
        s[e] = pk_pair(res[p0 * dim + m * DSUB + e], has1 ? res[p1 * dim + m * DSUB + e] : 0.0f);
    const ulonglong2* c2 = reinterpret_cast<const ulonglong2*>(scb2);
    u64 d = pk_sqeuclid<DSUB>(s, c2);
    float b0 = __uint_as_float((uint32_t)d), b1 = __uint_as_float((uint32_t)(d >> 32));
    int i0 = 0, i1 = 0;
#pragma unroll 4
    for (int j = 1; j < pqK; j++) {
        d = pk_sqeuclid<DSUB>(s, c2 + j * (DSUB / 2));
        const float e0 = __uint_as_float((uint32_t)d), e1 = __uint_as_float((uint32_t)(d >> 32));
        if (e0 < b0) {
            b0 = e0;
            i0 = j;
        }
        if (e1 < b1) {
            b1 = e1;
            i1 = j;
        }
    }
    out[p0 * M + m] = i0;
    if (has1) out[p1 * M + m] = i1;
}

// The packed assignment fused with the k-means accumulation of the same
// iteration: a grid of at most four blocks an SM walks the rows in tiles of
// 2 x 256; each row's sub-vector, already in registers, is added in FP64 to
// its codeword's sum in shared memory (an odd stride of DSUB + 1 doubles a
// codeword, so the lanes adding the same coordinate for random codewords
// spread over all 16 bank pairs), and every block adds its sums and counts
// to the global ones once. Same assignments as pq_assign_packed_kernel; the sums are FP64
// additions of the same values, in another order.
template <int DSUB>
__global__ void __launch_bounds__(PQ_PACK_THREADS) pq_assign_accumulate_kernel(
    const float* __restrict__ res, int64_t n, int M, const float* __restrict__ cb, int pqK, int m,
    int32_t* __restrict__ out, double* __restrict__ sums, unsigned long long* __restrict__ counts) {
    extern __shared__ __align__(16) float scb2[];  // [pqK][DSUB][2], then sums, then counts
    double* ssum = reinterpret_cast<double*>(scb2 + 2 * pqK * DSUB);  // [pqK][DSUB + 1]
    unsigned long long* scnt = reinterpret_cast<unsigned long long*>(ssum + pqK * (DSUB + 1));
    const int dim = M * DSUB;
    for (int e = threadIdx.x; e < pqK * DSUB; e += blockDim.x) {
        const float v = cb[(int64_t)m * pqK * DSUB + e];
        scb2[2 * e] = v;
        scb2[2 * e + 1] = v;
    }
    for (int e = threadIdx.x; e < pqK * (DSUB + 1); e += blockDim.x) ssum[e] = 0.0;
    for (int e = threadIdx.x; e < pqK; e += blockDim.x) scnt[e] = 0ull;
    __syncthreads();
    const ulonglong2* c2 = reinterpret_cast<const ulonglong2*>(scb2);
    for (int64_t t0 = (int64_t)blockIdx.x * (2 * PQ_PACK_THREADS); t0 < n;
         t0 += (int64_t)gridDim.x * (2 * PQ_PACK_THREADS)) {
        const int64_t p0 = t0 + threadIdx.x, p1 = p0 + PQ_PACK_THREADS;
        if (p0 >= n) continue;
        const bool has1 = p1 < n;
        float v0[DSUB], v1[DSUB];
        u64 s[DSUB];
#pragma unroll
        for (int e = 0; e < DSUB; e++) {
            v0[e] = res[p0 * dim + m * DSUB + e];
            v1[e] = has1 ? res[p1 * dim + m * DSUB + e] : 0.0f;
            s[e] = pk_pair(v0[e], v1[e]);
        }
        u64 d = pk_sqeuclid<DSUB>(s, c2);
        float b0 = __uint_as_float((uint32_t)d), b1 = __uint_as_float((uint32_t)(d >> 32));
        int i0 = 0, i1 = 0;
#pragma unroll 4
        for (int j = 1; j < pqK; j++) {
            d = pk_sqeuclid<DSUB>(s, c2 + j * (DSUB / 2));
            const float e0 = __uint_as_float((uint32_t)d), e1 = __uint_as_float((uint32_t)(d >> 32));
            if (e0 < b0) {
                b0 = e0;
                i0 = j;
            }
            if (e1 < b1) {
                b1 = e1;
                i1 = j;
            }
        }
        out[p0 * M + m] = i0;
#pragma unroll
        for (int e = 0; e < DSUB; e++) atomicAdd(&ssum[i0 * (DSUB + 1) + e], (double)v0[e]);
        atomicAdd(&scnt[i0], 1ull);
        if (has1) {
            out[p1 * M + m] = i1;
#pragma unroll
            for (int e = 0; e < DSUB; e++) atomicAdd(&ssum[i1 * (DSUB + 1) + e], (double)v1[e]);
            atomicAdd(&scnt[i1], 1ull);
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < pqK * DSUB; e += blockDim.x) {
        const double v = ssum[(e / DSUB) * (DSUB + 1) + e % DSUB];
        if (v != 0.0) atomicAdd(&sums[e], v);
    }
    for (int e = threadIdx.x; e < pqK; e += blockDim.x)
        if (scnt[e]) atomicAdd(&counts[e], scnt[e]);
}

// Generic sub-dimension: sub-vector read from global memory.
__global__ void __launch_bounds__(256) pq_assign_generic_kernel(const float* __restrict__ res, int64_t n, int M,
                                                                int dsub, const float* __restrict__ cb, int pqK,
                                                                int m_begin, int32_t* __restrict__ out) {
    extern __shared__ __align__(16) float scb[];
    const int m = m_begin + blockIdx.y;
    const int dim = M * dsub;
    for (int e = threadIdx.x; e < pqK * dsub; e += blockDim.x) scb[e] = cb[(int64_t)m * pqK * dsub + e];
    __syncthreads();
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* sub = res + p * dim + m * dsub;
    float bd = sqeuclid_ref(sub, scb, dsub);
    int bi = 0;
    for (int j = 1; j < pqK; j++) {
        const float d = sqeuclid_ref(sub, scb + j * dsub, dsub);
        if (d < bd) {
            bd = d;
            bi = j;
        }
    }
    out[p * M + m] = bi;
}

cudaError_t launch_pq_assign(const float* res, int64_t n, int M, int dsub, const float* codebooks, int pqK,
                             int m_begin, int m_end, int32_t* out, cudaStream_t s) {
    if (n <= 0 || m_end <= m_begin) return cudaSuccess;
    const size_t smem = (size_t)pqK * dsub * sizeof(float);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(pq_assign_generic_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    const size_t smem2 = 2 * smem;
    if ((dsub == 4 || dsub == 8 || dsub == 16) && smem2 <= 48 * 1024) {
        dim3 g2((unsigned)ceil_div(n, 2 * PQ_PACK_THREADS), (unsigned)(m_end - m_begin));
        if (dsub == 4)
            pq_assign_packed_kernel<4><<<g2, PQ_PACK_THREADS, smem2, s>>>(res, n, M, codebooks, pqK, m_begin, out);
        else if (dsub == 8)
            pq_assign_packed_kernel<8><<<g2, PQ_PACK_THREADS, smem2, s>>>(res, n, M, codebooks, pqK, m_begin, out);
        else
            pq_assign_packed_kernel<16><<<g2, PQ_PACK_THREADS, smem2, s>>>(res, n, M, codebooks, pqK, m_begin, out);
        return cudaGetLastError();
    }
    dim3 grid((unsigned)ceil_div(n, 256), (unsigned)(m_end - m_begin));
    switch (smem > 48 * 1024 ? 0 : dsub) {
    case 1: pq_assign_kernel<1><<<grid, 256, smem, s>>>(res, n, M, codebooks, pqK, m_begin, out); break;
    case 2: pq_assign_kernel<2><<<grid, 256, smem, s>>>(res, n, M, codebooks, pqK, m_begin, out); break;
    case 4: pq_assign_kernel<4><<<grid, 256, smem, s>>>(res, n, M, codebooks, pqK, m_begin, out); break;
    case 8: pq_assign_kernel<8><<<grid, 256, smem, s>>>(res, n, M, codebooks, pqK, m_begin, out); break;
    case 16: pq_assign_kernel<16><<<grid, 256, smem, s>>>(res, n, M, codebooks, pqK, m_begin, out); break;
    default:
        pq_assign_generic_kernel<<<grid, 256, smem, s>>>(res, n, M, dsub, codebooks, pqK, m_begin, out);
        break;
    }
    return cudaGetLastError();
}

__global__ void pq_accumulate_kernel(const float* __restrict__ res, int64_t n, int M, int dsub,
                                     const int32_t* __restrict__ codes, int pqK, int m_begin, int m_cnt,
                                     double* __restrict__ sums, int64_t* __restrict__ counts) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per_point = (int64_t)m_cnt * dsub;
    if (e >= n * per_point) return;
    const int64_t p = e / per_point;
    const int r = (int)(e - p * per_point);
    const int m = m_begin + r / dsub;
    const int i = r % dsub;
    const int dim = M * dsub;
    const int c = codes[p * M + m];
    atomicAdd(&sums[((int64_t)m * pqK + c) * dsub + i], (double)res[p * dim + m * dsub + i]);
    if (i == 0) atomicAdd(reinterpret_cast<unsigned long long*>(&counts[(int64_t)m * pqK + c]), 1ull);
}

// One subquantizer's sums, accumulated per block in shared memory (FP64)
// and added to the global sums once per block: every codeword is hit by
// thousands of points, so direct global atomics serialise on it.
__global__ void pq_accumulate_smem_kernel(const float* __restrict__ res, int64_t n, int M, int dsub,
                                          const int32_t* __restrict__ codes, int pqK, int m,
                                          double* __restrict__ sums, int64_t* __restrict__ counts) {
    extern __shared__ __align__(16) double psum[];  // [pqK * dsub], then pqK counts
    unsigned long long* pcnt = reinterpret_cast<unsigned long long*>(psum + pqK * dsub);
    for (int i = threadIdx.x; i < pqK * dsub; i += blockDim.x) psum[i] = 0.0;
    for (int i = threadIdx.x; i < pqK; i += blockDim.x) pcnt[i] = 0ull;
    __syncthreads();
    const int dim = M * dsub;
    const int64_t per = ceil_div(n, gridDim.x);
    const int64_t p0 = blockIdx.x * per, p1 = min(n, p0 + per);
    for (int64_t e = p0 * dsub + threadIdx.x; e < p1 * dsub; e += blockDim.x) {
        const int64_t p = e / dsub;
        const int i = (int)(e - p * dsub);
        const int c = codes[p * M + m];
        atomicAdd(&psum[c * dsub + i], (double)res[p * dim + m * dsub + i]);
        if (i == 0) atomicAdd(&pcnt[c], 1ull);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < pqK * dsub; i += blockDim.x)
        if (psum[i] != 0.0) atomicAdd(&sums[(int64_t)m * pqK * dsub + i], psum[i]);
    for (int i = threadIdx.x; i < pqK; i += blockDim.x)
        if (pcnt[i]) atomicAdd(reinterpret_cast<unsigned long long*>(&counts[(int64_t)m * pqK + i]), pcnt[i]);
}

cudaError_t launch_pq_accumulate(const float* res, int64_t n, int M, int dsub, const int32_t* codes, int pqK,
                                 int m_begin, int m_end, double* sums, int64_t* counts, cudaStream_t s) {
    if (n <= 0 || m_end <= m_begin) return cudaSuccess;
    const size_t smem = (size_t)pqK * dsub * sizeof(double) + (size_t)pqK * sizeof(unsigned long long);
    if (m_end - m_begin == 1 && smem <= 48 * 1024 && n >= 4096) {
        const unsigned blocks = (unsigned)std::min<int64_t>(4 * 152, ceil_div(n, 1024));
        pq_accumulate_smem_kernel<<<blocks, 256, smem, s>>>(res, n, M, dsub, codes, pqK, m_begin, sums, counts);
        return cudaGetLastError();
    }
    const int64_t total = n * (int64_t)(m_end - m_begin) * dsub;
    pq_accumulate_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(res, n, M, dsub, codes, pqK, m_begin,
                                                                       m_end - m_begin, sums, counts);
    return cudaGetLastError();
}

size_t pq_assign_accumulate_smem(int dsub, int pqK) {
    return (size_t)pqK * dsub * 2 * sizeof(float) + (size_t)pqK * (dsub + 1) * sizeof(double) +
           (size_t)pqK * sizeof(unsigned long long);
}

bool pq_assign_accumulate_supported(int dsub, int pqK) {
    return (dsub == 4 || dsub == 8 || dsub == 16) && pqK >= 1 && pqK <= 256;
}

cudaError_t launch_pq_assign_accumulate(const float* res, int64_t n, int M, int dsub, const float* codebooks,
                                        int pqK, int m, int32_t* out, double* sums_m, int64_t* counts_m,
                                        cudaStream_t s) {
    if (!pq_assign_accumulate_supported(dsub, pqK)) return cudaErrorNotSupported;
    if (n <= 0) return cudaSuccess;
    const size_t smem = pq_assign_accumulate_smem(dsub, pqK);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto* cnt = reinterpret_cast<unsigned long long*>(counts_m);
    cudaError_t e = cudaSuccess;
    // up to four resident blocks an SM, as many as the shared memory allows
#define HANN_PQ_FUSED(D)                                                                                       \
    {                                                                                                          \
        e = cudaFuncSetAttribute(pq_assign_accumulate_kernel<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                 (int)smem);                                                                   \
        if (e != cudaSuccess) return e;                                                                        \
        int occ = 1;                                                                                           \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pq_assign_accumulate_kernel<D>,                \
                                                          PQ_PACK_THREADS, smem);                              \
        if (e != cudaSuccess) return e;                                                                        \
        const unsigned blocks = (unsigned)std::min<int64_t>((int64_t)std::max(1, std::min(occ, 4)) * sms,      \
                                                            ceil_div(n, 2 * PQ_PACK_THREADS));                 \
        pq_assign_accumulate_kernel<D><<<blocks, PQ_PACK_THREADS, smem, s>>>(res, n, M, codebooks, pqK, m, out, \
                                                                             sums_m, cnt);                     \
    }
    if (dsub == 4) {
        HANN_PQ_FUSED(4)
    } else if (dsub == 8) {
        HANN_PQ_FUSED(8)
    } else {
        HANN_PQ_FUSED(16)
    }
#undef HANN_PQ_FUSED
    return cudaGetLastError();
}

__global__ void residuals_kernel(const float* __restrict__ x, const int64_t* __restrict__ src,
                                 const int32_t* __restrict__ cluster, int64_t n, int dim,
                                 const float* __restrict__ coarse, float* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * dim) return;
    const int64_t r = e / dim;
    const int i = (int)(e - r * dim);
    const int64_t sr = src ? src[r] : r;
    out[e] = x[sr * dim + i] - coarse[(int64_t)cluster[r] * dim + i];
}

cudaError_t launch_residuals(const float* x, const int64_t* src, const int32_t* cluster, int64_t n, int dim,
                             const float* coarse, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    residuals_kernel<<<(unsigned)ceil_div(n * dim, 256), 256, 0, s>>>(x, src, cluster, n, dim, coarse, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Encoding: one thread per row, one subquantizer codebook at a time in
// shared memory. The residual is x - c in FP32 (vectorSub,
// pqivf/index.go:692-702); each code is the reference-order argmin.
__global__ void __launch_bounds__(256) encode_kernel(const float* __restrict__ x, const int64_t* __restrict__ rows,
                                                     const int32_t* __restrict__ cluster, int64_t n, int dim,
                                                     const float* __restrict__ coarse,
                                                     const float* __restrict__ cb, int M, int pqK,
                                                     uint8_t* __restrict__ codes, int code_stride,
                                                     float* __restrict__ term) {
    extern __shared__ __align__(16) float scb[];
    const int dsub = dim / M;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    const int64_t p = live ? (rows ? rows[i] : i) : 0;
    const int cl = live ? cluster[p] : 0;
    const float* xp = x + p * dim;
    const float* cp = coarse + (int64_t)cl * dim;
    float tsum = 0.0f;
    struct Res {
        const float* a;
        const float* b;
        __device__ float operator[](int t) const { return a[t] - b[t]; }
    };
    for (int m = 0; m < M; m++) {
        __syncthreads();
        for (int e = threadIdx.x; e < pqK * dsub; e += blockDim.x) scb[e] = cb[(int64_t)m * pqK * dsub + e];
        __syncthreads();
        if (!live) continue;
        const Res rs{xp + m * dsub, cp + m * dsub};
        float bd = sqeuclid_ref(rs, scb, dsub);
        int bi = 0;
        for (int j = 1; j < pqK; j++) {
            const float d = sqeuclid_ref(rs, scb + j * dsub, dsub);
            if (d < bd) {
                bd = d;
                bi = j;
            }
        }
        codes[p * code_stride + m] = (uint8_t)bi;
        const float* w = scb + bi * dsub;
        for (int e = 0; e < dsub; e++) tsum += w[e] * (w[e] + 2.0f * cp[m * dsub + e]);
    }
    if (live) {
        for (int m = M; m < code_stride; m++) codes[p * code_stride + m] = 0;
        term[p] = tsum;
    }
}

// encode_kernel with the sub-vector length known at compile time: each
// residual sub-vector (FP32 x - c, as the reference's residual) is formed once
// in registers instead of at every codeword.
template <int DSUB>
__global__ void __launch_bounds__(256) encode_fixed_kernel(const float* __restrict__ x,
                                                           const int64_t* __restrict__ rows,
                                                           const int32_t* __restrict__ cluster, int64_t n, int dim,
                                                           const float* __restrict__ coarse,
                                                           const float* __restrict__ cb, int M, int pqK,
                                                           uint8_t* __restrict__ codes, int code_stride,
                                                           float* __restrict__ term) {
    extern __shared__ __align__(16) float scb[];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    const int64_t p = live ? (rows ? rows[i] : i) : 0;
    const int cl = live ? cluster[p] : 0;
    const float* xp = x + p * dim;
    const float* cp = coarse + (int64_t)cl * dim;
    float tsum = 0.0f;
    for (int m = 0; m < M; m++) {
        __syncthreads();
        for (int e = threadIdx.x; e < pqK * DSUB; e += blockDim.x) scb[e] = cb[(int64_t)m * pqK * DSUB + e];
        __syncthreads();
        if (!live) continue;
        float r[DSUB];
#pragma unroll
        for (int e = 0; e < DSUB; e++) r[e] = xp[m * DSUB + e] - cp[m * DSUB + e];
        float bd = sqeuclid_ref(r, scb, DSUB);
        int bi = 0;
        for (int j = 1; j < pqK; j++) {
            const float d = sqeuclid_ref(r, scb + j * DSUB, DSUB);
            if (d < bd) {
                bd = d;
                bi = j;
            }
        }
        codes[p * code_stride + m] = (uint8_t)bi;
        const float* w = scb + bi * DSUB;
        for (int e = 0; e < DSUB; e++) tsum += w[e] * (w[e] + 2.0f * cp[m * DSUB + e]);
    }
    if (live) {
        for (int m = M; m < code_stride; m++) codes[p * code_stride + m] = 0;
        term[p] = tsum;
    }
}

cudaError_t launch_encode(const float* x, const int64_t* rows, const int32_t* cluster, int64_t n, int dim,
                          const float* coarse, const float* codebooks, int M, int pqK, uint8_t* codes,
                          int code_stride, float* term, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int dsub = dim / M;
    const size_t smem = (size_t)pqK * dsub * sizeof(float);
    const unsigned grid = (unsigned)ceil_div(n, 256);
    if (smem <= 48 * 1024) {
        switch (dsub) {
        case 1:
            encode_fixed_kernel<1><<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                          codes, code_stride, term);
            return cudaGetLastError();
        case 2:
            encode_fixed_kernel<2><<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                          codes, code_stride, term);
            return cudaGetLastError();
        case 4:
            encode_fixed_kernel<4><<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                          codes, code_stride, term);
            return cudaGetLastError();
        case 8:
            encode_fixed_kernel<8><<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                          codes, code_stride, term);
            return cudaGetLastError();
        case 16:
            encode_fixed_kernel<16><<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                          codes, code_stride, term);
            return cudaGetLastError();
        default: break;
        }
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    encode_kernel<<<grid, 256, smem, s>>>(x, rows, cluster, n, dim, coarse, codebooks, M, pqK, codes, code_stride,
                                          term);
    return cudaGetLastError();
}

__global__ void term_kernel(const uint8_t* __restrict__ codes, const int64_t* __restrict__ rows,
                            const int32_t* __restrict__ cluster, int64_t n, int dim, const float* __restrict__ coarse,
                            const float* __restrict__ cb, int M, int pqK, int code_stride, float* __restrict__ term) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t p = rows ? rows[i] : i;
    const int dsub = dim / M;
    const float* cp = coarse + (int64_t)cluster[p] * dim;
    float tsum = 0.0f;
    for (int m = 0; m < M; m++) {
        const float* w = cb + ((int64_t)m * pqK + codes[p * code_stride + m]) * dsub;
        for (int e = 0; e < dsub; e++) tsum += w[e] * (w[e] + 2.0f * cp[m * dsub + e]);
    }
    term[p] = tsum;
}

cudaError_t launch_term(const uint8_t* codes, const int64_t* rows, const int32_t* cluster, int64_t n, int dim,
                        const float* coarse, const float* codebooks, int M, int pqK, int code_stride, float* term,
                        cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    term_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(codes, rows, cluster, n, dim, coarse, codebooks, M, pqK,
                                                           code_stride, term);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Row movement.
__global__ void copy_words_kernel(const uint32_t* __restrict__ in, const int64_t* __restrict__ src,
                                  uint32_t* __restrict__ out, const int64_t* __restrict__ dst, int64_t n, int width) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * width) return;
    const int64_t r = e / width;
    const int j = (int)(e - r * width);
    const int64_t sr = src ? src[r] : r;
    const int64_t dr = dst ? dst[r] : r;
    out[dr * width + j] = in[sr * width + j];
}

cudaError_t launch_copy_words(const void* in, const int64_t* src, void* out, const int64_t* dst, int64_t n, int width,
                              cudaStream_t s) {
    if (n <= 0 || width <= 0) return cudaSuccess;
    copy_words_kernel<<<(unsigned)ceil_div(n * width, 256), 256, 0, s>>>(
        static_cast<const uint32_t*>(in), src, static_cast<uint32_t*>(out), dst, n, width);
    return cudaGetLastError();
}

__global__ void gather2_kernel(const float* __restrict__ a, const float* __restrict__ b,
                               const int64_t* __restrict__ src, int64_t n, int dim, float* __restrict__ out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * dim) return;
    const int64_t r = e / dim;
    const int j = (int)(e - r * dim);
    const int64_t s = src[r];
    out[e] = s >= 0 ? a[s * dim + j] : b[(-s - 1) * dim + j];
}

cudaError_t launch_gather2(const float* a, const float* b, const int64_t* src, int64_t n, int dim, float* out,
                           cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    gather2_kernel<<<(unsigned)ceil_div(n * dim, 256), 256, 0, s>>>(a, b, src, n, dim, out);
    return cudaGetLastError();
}

__global__ void gather_cols_kernel(const float* __restrict__ in, int64_t ld, int off, const int64_t* __restrict__ src,
                                   const int32_t* __restrict__ dst, int64_t n, int w, float* __restrict__ out,
                                   int64_t ldo) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * w) return;
    const int64_t r = e / w;
    const int j = (int)(e - r * w);
    const int64_t dr = dst ? dst[r] : r;
    out[dr * ldo + j] = in[src[r] * ld + off + j];
}

cudaError_t launch_gather_cols(const float* in, int64_t ld, int off, const int64_t* src, const int32_t* dst, int64_t n,
                               int w, float* out, int64_t ldo, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    gather_cols_kernel<<<(unsigned)ceil_div(n * w, 256), 256, 0, s>>>(in, ld, off, src, dst, n, w, out, ldo);
    return cudaGetLastError();
}

__global__ void tombstone_kernel(const int64_t* __restrict__ rows, int64_t n, float* __restrict__ term,
                                 int64_t* __restrict__ row_id) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    term[rows[i]] = __int_as_float(0x7f800000);
    row_id[rows[i]] = -1;
}

// One block per list: the list's slots [src, src + len) move, in order, to
// [dst, ...); with compact set only live slots (row id >= 0) move, so the
// tombstones disappear. Rows go 256 at a time: the block ranks the live
// slots with ballots, then copies the chunk's vector and code words with
// consecutive threads on consecutive words.
__global__ void __launch_bounds__(256) relayout_lists_kernel(
    const int64_t* __restrict__ src_start, const int32_t* __restrict__ src_len, const int64_t* __restrict__ dst_start,
    const int32_t* __restrict__ compact, int dim, int cwords, const float* __restrict__ vin, float* __restrict__ vout,
    const uint32_t* __restrict__ cin, uint32_t* __restrict__ cout, const float* __restrict__ tin,
    float* __restrict__ tout, const int64_t* __restrict__ rin, int64_t* __restrict__ rout,
    const int32_t* __restrict__ clin, int32_t* __restrict__ clout) {
    __shared__ int pos[256];
    __shared__ int wcnt[8];
    const int l = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t src = src_start[l], dst = dst_start[l];
    const int len = src_len[l];
    const bool cmp = compact[l] != 0;
    int out = 0;
    for (int c0 = 0; c0 < len; c0 += 256) {
        const int j = c0 + tid;
        const bool live = j < len && (!cmp || rin[src + j] >= 0);
        const unsigned b = __ballot_sync(0xffffffffu, live);
        if (lane == 0) wcnt[w] = __popc(b);
        __syncthreads();
        int before = 0, tot = 0;
        for (int ww = 0; ww < 8; ww++) {
            if (ww < w) before += wcnt[ww];
            tot += wcnt[ww];
        }
        const int p = live ? out + before + __popc(b & ((1u << lane) - 1u)) : -1;
        pos[tid] = p;
        if (live) {
            tout[dst + p] = tin[src + j];
            rout[dst + p] = rin[src + j];
            clout[dst + p] = clin[src + j];
        }
        __syncthreads();
        const int rows = min(256, len - c0);
        for (int e = tid; e < rows * dim; e += 256) {
            const int r = e / dim, i = e - r * dim;
            if (pos[r] >= 0) vout[(dst + pos[r]) * dim + i] = vin[(src + c0 + r) * dim + i];
        }
        for (int e = tid; e < rows * cwords; e += 256) {
            const int r = e / cwords, i = e - r * cwords;
            if (pos[r] >= 0) cout[(dst + pos[r]) * cwords + i] = cin[(src + c0 + r) * cwords + i];
        }
        out += tot;
        __syncthreads();
    }
}

cudaError_t launch_relayout_lists(int nlist, const int64_t* src_start, const int32_t* src_len,
                                  const int64_t* dst_start, const int32_t* compact, int dim, int cwords,
                                  const float* vin, float* vout, const void* cin, void* cout, const float* tin,
                                  float* tout, const int64_t* rin, int64_t* rout, const int32_t* clin, int32_t* clout,
                                  cudaStream_t s) {
    if (nlist <= 0) return cudaSuccess;
    relayout_lists_kernel<<<(unsigned)nlist, 256, 0, s>>>(src_start, src_len, dst_start, compact, dim, cwords, vin,
                                                         vout, static_cast<const uint32_t*>(cin),
                                                         static_cast<uint32_t*>(cout), tin, tout, rin, rout, clin,
                                                         clout);
    return cudaGetLastError();
}

cudaError_t launch_tombstone(const int64_t* rows, int64_t n, float* term, int64_t* row_id, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    tombstone_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(rows, n, term, row_id);
    return cudaGetLastError();
}

}  // namespace hann

// Subquantizer assignment of host residuals: res [n][M * dsub], codebooks
// [M][pqK][dsub], out [n][M] the nearest codeword of every row and
// subquantizer, as one k-means iteration of training computes it; with sums
// and counts, also the iteration's FP64 codeword sums [M][pqK][dsub] and
// counts [M][pqK], through the kernels training runs.
extern "C" int hann_gpu_pq_assign(const float* res, int64_t n, int32_t M, int32_t dsub, const float* codebooks,
                                  int32_t pqK, int32_t* out, double* sums, int64_t* counts) {
    using namespace hann;
    if (n <= 0 || M <= 0 || dsub <= 0 || pqK <= 0 || pqK > 256 || !res || !codebooks || !out ||
        (sums == nullptr) != (counts == nullptr))
        return HANN_E_INVALID;
    float *dr = nullptr, *dc = nullptr;
    int32_t* dout = nullptr;
    double* dsum = nullptr;
    int64_t* dcnt = nullptr;
    int rc = HANN_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == HANN_OK) rc = HANN_E_CUDA;
        return e == cudaSuccess;
    };
    const size_t nr = (size_t)n * M * dsub, nc = (size_t)M * pqK * dsub;
    if (ok(cudaMalloc(&dr, sizeof(float) * nr)) && ok(cudaMalloc(&dc, sizeof(float) * nc)) &&
        ok(cudaMalloc(&dout, sizeof(int32_t) * (size_t)n * M)) &&
        (!sums || (ok(cudaMalloc(&dsum, sizeof(double) * nc)) && ok(cudaMalloc(&dcnt, sizeof(int64_t) * M * pqK))))) {
        ok(cudaMemcpy(dr, res, sizeof(float) * nr, cudaMemcpyHostToDevice));
        ok(cudaMemcpy(dc, codebooks, sizeof(float) * nc, cudaMemcpyHostToDevice));
        if (sums) {
            ok(cudaMemset(dsum, 0, sizeof(double) * nc));
            ok(cudaMemset(dcnt, 0, sizeof(int64_t) * M * pqK));
        }
        for (int m = 0; m < M && rc == HANN_OK; m++) {
            if (!sums) {
                ok(launch_pq_assign(dr, n, M, dsub, dc, pqK, m, m + 1, dout, nullptr));
            } else if (pq_assign_accumulate_supported(dsub, pqK)) {
                ok(launch_pq_assign_accumulate(dr, n, M, dsub, dc, pqK, m, dout, dsum + (size_t)m * pqK * dsub,
                                               dcnt + (size_t)m * pqK, nullptr));
            } else {
                ok(launch_pq_assign(dr, n, M, dsub, dc, pqK, m, m + 1, dout, nullptr));
                ok(launch_pq_accumulate(dr, n, M, dsub, dout, pqK, m, m + 1, dsum, dcnt, nullptr));
            }
        }
        ok(cudaDeviceSynchronize());
        ok(cudaMemcpy(out, dout, sizeof(int32_t) * (size_t)n * M, cudaMemcpyDeviceToHost));
        if (sums) {
            ok(cudaMemcpy(sums, dsum, sizeof(double) * nc, cudaMemcpyDeviceToHost));
            ok(cudaMemcpy(counts, dcnt, sizeof(int64_t) * M * pqK, cudaMemcpyDeviceToHost));
        }
    }
    cudaFree(dr);
    cudaFree(dc);
    cudaFree(dout);
    cudaFree(dsum);
    cudaFree(dcnt);
    return rc;
}
