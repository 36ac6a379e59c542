// kernels_rescore.cu -- exact answers from the BF16 tensor-core scores.
//
// The GEMM in kernels_gemm.cu ranks columns by s~(a, b) = ||b||^2 - 2<a, b>
// computed from BF16 operands; |s~ - s| <= eps(a) with eps(a) from
// bf16_score_eps (common.cuh). Both kernels
// here rescore, with the reference's exact FP32 distance (common.cuh,
// sqeuclid_ref), every column whose approximate score can still reach the
// boundary, so their outputs equal the exact SIMT path's:
//   * probe_select_band: the nprobe nearest lists of a query. With T~ the
//     nprobe-th smallest approximate score, every list of the exact top
//     nprobe has s~ <= T~ + 2 eps; all of those are rescored exactly and the
//     best nprobe by (exact distance, index) are kept (nearestCentroids,
//     pqivf/index.go:184-206). More than PS_MAX of them (a degenerate band)
//     falls back to rescoring the whole row.
//   * rescore_top8: the argmin for k-means and Add (assignPoints,
//     pqivf/index.go:738-789). The GEMM kept each row's 8 smallest scores;
//     if the 8th is still inside the band [s~min, s~min + 2 eps] the band may
//     hold more columns and the row is listed for the exact tiled kernel,
//     otherwise the exact argmin (lowest index on a tie) is among the 8.
#include "common.cuh"
#include "kernels.h"
#include "select.cuh"

namespace hann {
namespace {

constexpr int PB_THREADS = 256;
constexpr int PB_MAX = 4096;
constexpr int QMAX = 128;

__global__ void __launch_bounds__(PB_THREADS) probe_select_band_kernel(
    float* __restrict__ S, const float* __restrict__ Q, const float* __restrict__ qn2,
    const float* __restrict__ qres, int dim, int kp, const float* __restrict__ coarse,
    const float* __restrict__ cmax_p, int nlist, const int32_t* __restrict__ nprobe,
    int np_max, const int32_t* __restrict__ kq, const int32_t* __restrict__ list_len, int allow_fb,
    int32_t* __restrict__ probe_ids, float* __restrict__ probe_d, int32_t* __restrict__ fallback,
    unsigned long long* __restrict__ fb_count, int row_in_smem) {
    __shared__ uint32_t s_key[PB_MAX];
    __shared__ int32_t s_idx[PB_MAX];
    __shared__ float qv[QMAX];
    __shared__ uint32_t s_prefix, s_rem, s_and, s_or;
    __shared__ int s_cnt, s_cnt2;
    __shared__ unsigned long long s_total;
    __shared__ unsigned int whist[(PB_THREADS / 32) * 256];
    extern __shared__ __align__(16) float srow[];
    const int tid = threadIdx.x;
    const int64_t q = blockIdx.x;
    float* row = S + q * nlist;
    if (row_in_smem) {
        // one read of the score row; every pass below runs on shared memory
        const float4* g4 = reinterpret_cast<const float4*>(row);
        float4* s4 = reinterpret_cast<float4*>(srow);
        const int n4 = (nlist & 3) == 0 ? nlist >> 2 : 0;
        for (int i = tid; i < n4; i += PB_THREADS) s4[i] = g4[i];
        for (int i = 4 * n4 + tid; i < nlist; i += PB_THREADS) srow[i] = row[i];
        row = srow;
    }
    const int np = min(nprobe[q], nlist);
    for (int e = tid; e < dim; e += PB_THREADS) qv[e] = Q[q * dim + e];
    if (tid == 0) {
        s_cnt = 0;
        s_cnt2 = 0;
        s_total = 0;
    }
    radix_nth_fast<PB_THREADS>(row, nlist, np, whist, &s_prefix, &s_rem, &s_and, &s_or);
    const float eps = bf16_score_eps(sqrtf(qn2[q]), qres[q], cmax_p[0], cmax_p[1], kp);
    const float tA = key_float(s_prefix);
    // plus twice the FP32 rounding of a reference-order distance (about
    // dim * 2^-24 of its size, covered by 2e-5 here for dim <= 128)
    const float thr = tA + 2.0f * eps + 2e-5f * (fabsf(tA) + qn2[q]);
    for (int c = tid; c < nlist; c += PB_THREADS) {
        if (row[c] <= thr) {
            const int pos = atomicAdd(&s_cnt, 1);
            if (pos < PB_MAX) s_idx[pos] = c;
        }
    }
    __syncthreads();
    int C = s_cnt;
    if (C > PB_MAX) {
        // Degenerate band: rescore the whole row exactly, then select on it.
        for (int c = tid; c < nlist; c += PB_THREADS) row[c] = sqeuclid_ref(qv, coarse + (int64_t)c * dim, dim);
        __syncthreads();
        radix_nth_fast<PB_THREADS>(row, nlist, np, whist, &s_prefix, &s_rem, &s_and, &s_or);
        const uint32_t T = s_prefix;
        for (int c = tid; c < nlist; c += PB_THREADS) {
            const uint32_t key = float_key(row[c]);
            if (key <= T) {
                const int pos = atomicAdd(&s_cnt2, 1);
                if (pos < PB_MAX) {
                    s_key[pos] = key;
                    s_idx[pos] = c;
                }
            }
        }
        __syncthreads();
        C = min(s_cnt2, PB_MAX);
    } else {
        for (int i = tid; i < C; i += PB_THREADS)
            s_key[i] = float_key(sqeuclid_ref(qv, coarse + (int64_t)s_idx[i] * dim, dim));
    }
    int P = 1;
    while (P < C) P <<= 1;
    for (int i = C + tid; i < P; i += PB_THREADS) {
        s_key[i] = 0xffffffffu;
        s_idx[i] = 0x7fffffff;
    }
    __syncthreads();
    sort_ki(s_key, s_idx, P);
    unsigned long long part = 0;
    for (int i = tid; i < np; i += PB_THREADS) {
        probe_ids[q * np_max + i] = s_idx[i];
        probe_d[q * np_max + i] = key_float(s_key[i]);
        part += (unsigned long long)list_len[s_idx[i]];
    }
    atomicAdd(&s_total, part);
    __syncthreads();
    if (tid == 0) {
        const int fb = (allow_fb && s_total < (unsigned long long)kq[q]) ? 1 : 0;
        fallback[q] = fb;
        if (fb) atomicAdd(fb_count, 1ull);
    }
}

constexpr int PFW_CAP = 256;  // band lists up to this length finish on one warp
constexpr int PFW_WARPS = 8;

// One warp per query when its band holds at most PFW_CAP lists (the usual
// case: about nprobe plus a few): the same result as probe_final_kernel
// without block barriers. Other queries are left to probe_final_kernel.
__global__ void __launch_bounds__(PFW_WARPS * 32) probe_final_warp_kernel(
    const float* __restrict__ Q, int64_t nq, int dim, const float* __restrict__ coarse, int nlist,
    const int32_t* __restrict__ nprobe, int np_max, const int32_t* __restrict__ kq,
    const int32_t* __restrict__ list_len, int allow_fb, int lcap, const unsigned long long* __restrict__ band,
    const int32_t* __restrict__ lcount, const int32_t* __restrict__ need_exact, int32_t* __restrict__ probe_ids,
    float* __restrict__ probe_d, int32_t* __restrict__ fallback, unsigned long long* __restrict__ fb_count,
    int32_t* __restrict__ todo, int32_t* __restrict__ todo_count) {
    __shared__ float qv_all[PFW_WARPS][QMAX];
    __shared__ unsigned long long keys_all[PFW_WARPS][PFW_CAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * PFW_WARPS + w;
    if (q >= nq) return;
    const int L = lcount[q];
    if (need_exact[q] || L > PFW_CAP) {
        // left to probe_final_kernel
        if (lane == 0) todo[atomicAdd(todo_count, 1)] = (int32_t)q;
        return;
    }
    float* qv = qv_all[w];
    unsigned long long* keys = keys_all[w];
    for (int e = lane; e < dim; e += 32) qv[e] = Q[q * dim + e];
    __syncwarp();
    const int np = min(nprobe[q], nlist);
    int P = 1;
    while (P < L) P <<= 1;
    for (int i = lane; i < P; i += 32) {
        unsigned long long key = ~0ull;
        if (i < L) {
            const uint32_t c = (uint32_t)(band[q * lcap + i] & 0xffffffffull);
            const float* cr = coarse + (int64_t)c * dim;
            const float d = (dim & 3) == 0 ? sqeuclid_ref_v4(qv, cr, dim) : sqeuclid_ref(qv, cr, dim);
            key = ((unsigned long long)float_key(d) << 32) | c;
        }
        keys[i] = key;
    }
    __syncwarp();
    warp_sort_u64(keys, P);
    unsigned long long part = 0;
    for (int i = lane; i < np; i += 32) {
        const int c = (int)(keys[i] & 0xffffffffull);
        probe_ids[q * np_max + i] = c;
        probe_d[q * np_max + i] = key_float((uint32_t)(keys[i] >> 32));
        part += (unsigned long long)list_len[c];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) {
        const int fb = (allow_fb && part < (unsigned long long)kq[q]) ? 1 : 0;
        fallback[q] = fb;
        if (fb) atomicAdd(fb_count, 1ull);
    }
}

// Final step of the screened probe. Per query, the band list (every list
// whose screened score can still reach the np-th) is rescored with the
// reference-order FP32 distance and the best np by (distance, list) are
// written ascending. A query whose band overflowed (need_exact) computes its
// whole exact row into Drow (global scratch, nlist per query) and selects on
// it, ties at the cut taken in list order. Also sets the fallback flag like
// probe_select_band.
__device__ __forceinline__ void probe_final_row(
    int64_t q, const float* __restrict__ Q, int dim, const float* __restrict__ coarse, int nlist,
    const int32_t* __restrict__ nprobe, int np_max, const int32_t* __restrict__ kq,
    const int32_t* __restrict__ list_len, int allow_fb, int lcap, const unsigned long long* __restrict__ band,
    const int32_t* __restrict__ lcount, const int32_t* __restrict__ need_exact, float* __restrict__ Drow,
    int32_t* __restrict__ probe_ids, float* __restrict__ probe_d, int32_t* __restrict__ fallback,
    unsigned long long* __restrict__ fb_count) {
    extern __shared__ __align__(16) unsigned long long keys[];  // [lcap + P]
    __shared__ float qv[QMAX];
    __shared__ unsigned int hist[256];
    __shared__ unsigned int whist[(PB_THREADS / 32) * 256];
    __shared__ unsigned long long s_and, s_or, s_prefix;
    __shared__ uint32_t s_p32, s_rem, s_a32, s_o32;
    __shared__ int s_pos, s_wsum[PB_THREADS / 32];
    __shared__ unsigned long long s_total;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (!need_exact[q] && lcount[q] <= PFW_CAP) return;  // done by probe_final_warp_kernel
    const int np = min(nprobe[q], nlist);
    for (int e = tid; e < dim; e += PB_THREADS) qv[e] = Q[q * dim + e];
    if (tid == 0) {
        s_pos = 0;
        s_total = 0;
    }
    __syncthreads();
    int P = 1;
    while (P < np) P <<= 1;
    unsigned long long* out;
    if (need_exact[q]) {
        float* row = Drow + q * nlist;
        for (int c = tid; c < nlist; c += PB_THREADS) row[c] = sqeuclid_ref(qv, coarse + (int64_t)c * dim, dim);
        __syncthreads();
        radix_nth_fast<PB_THREADS>(row, nlist, np, whist, &s_p32, &s_rem, &s_a32, &s_o32);
        const uint32_t T = s_p32, rem = s_rem;
        out = keys;
        // below the cut: order-free
        for (int c = tid; c < nlist; c += PB_THREADS) {
            const uint32_t key = float_key(row[c]);
            if (key < T) out[atomicAdd(&s_pos, 1)] = ((unsigned long long)key << 32) | (uint32_t)c;
        }
        // at the cut: the first rem lists in list order
        uint32_t taken = 0;
        for (int c0 = 0; c0 < nlist && taken < rem; c0 += PB_THREADS) {
            const int c = c0 + tid;
            const bool eq = c < nlist && float_key(row[c]) == T;
            const unsigned b = __ballot_sync(0xffffffffu, eq);
            if (lane == 0) s_wsum[w] = __popc(b);
            __syncthreads();
            uint32_t before = 0, tot = 0;
            for (int ww = 0; ww < PB_THREADS / 32; ww++) {
                if (ww < w) before += s_wsum[ww];
                tot += s_wsum[ww];
            }
            const uint32_t rank = taken + before + __popc(b & ((1u << lane) - 1u));
            if (eq && rank < rem) out[atomicAdd(&s_pos, 1)] = ((unsigned long long)T << 32) | (uint32_t)c;
            taken += tot;
            __syncthreads();
        }
    } else {
        const int L = lcount[q];
        for (int i = tid; i < L; i += PB_THREADS) {
            const uint32_t c = (uint32_t)(band[q * lcap + i] & 0xffffffffull);
            keys[i] = ((unsigned long long)float_key(sqeuclid_ref(qv, coarse + (int64_t)c * dim, dim)) << 32) | c;
        }
        __syncthreads();
        out = keys + L;
        if (L > np) {
            const unsigned long long K = radix_nth_u64(keys, L, np, hist, &s_and, &s_or, &s_prefix, &s_p32);
            for (int i = tid; i < L; i += PB_THREADS)
                if (keys[i] <= K) out[atomicAdd(&s_pos, 1)] = keys[i];
        } else {
            for (int i = tid; i < L; i += PB_THREADS) out[i] = keys[i];
        }
    }
    __syncthreads();
    for (int i = np + tid; i < P; i += PB_THREADS) out[i] = ~0ull;
    __syncthreads();
    if (P > 1) sort_u64(out, P);
    unsigned long long part = 0;
    for (int i = tid; i < np; i += PB_THREADS) {
        const int c = (int)(out[i] & 0xffffffffull);
        probe_ids[q * np_max + i] = c;
        probe_d[q * np_max + i] = key_float((uint32_t)(out[i] >> 32));
        part += (unsigned long long)list_len[c];
    }
    atomicAdd(&s_total, part);
    __syncthreads();
    if (tid == 0) {
        const int fb = (allow_fb && s_total < (unsigned long long)kq[q]) ? 1 : 0;
        fallback[q] = fb;
        if (fb) atomicAdd(fb_count, 1ull);
    }
}

// The queries probe_final_warp_kernel left, todo[0, *todo_count).
__global__ void __launch_bounds__(PB_THREADS) probe_final_kernel(
    const float* __restrict__ Q, int dim, const float* __restrict__ coarse, int nlist,
    const int32_t* __restrict__ nprobe, int np_max, const int32_t* __restrict__ kq,
    const int32_t* __restrict__ list_len, int allow_fb, int lcap, const unsigned long long* __restrict__ band,
    const int32_t* __restrict__ lcount, const int32_t* __restrict__ need_exact, float* __restrict__ Drow,
    int32_t* __restrict__ probe_ids, float* __restrict__ probe_d, int32_t* __restrict__ fallback,
    unsigned long long* __restrict__ fb_count, const int32_t* __restrict__ todo,
    const int32_t* __restrict__ todo_count) {
    const int n = *todo_count;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        probe_final_row(todo[i], Q, dim, coarse, nlist, nprobe, np_max, kq, list_len, allow_fb, lcap, band, lcount,
                        need_exact, Drow, probe_ids, probe_d, fallback, fb_count);
        __syncthreads();
    }
}

__global__ void rescore_top8_kernel(const float* __restrict__ x, const float* __restrict__ xn2,
                                    const float* __restrict__ xres, int64_t n, int dim, int kp,
                                    const float* __restrict__ cent, int k, const float* __restrict__ cmax_p,
                                    const int32_t* __restrict__ cand_idx, const float* __restrict__ cand_val,
                                    int32_t* __restrict__ out_idx, float* __restrict__ out_d2,
                                    int64_t* __restrict__ overflow_rows, int* __restrict__ n_overflow) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float eps = bf16_score_eps(sqrtf(xn2[r]), xres[r], cmax_p[0], cmax_p[1], kp);
    const float v0 = cand_val[r * 8];
    const float thr = v0 + 2.0f * eps + 2e-5f * (fabsf(v0) + xn2[r]);
    if (k > 8 && cand_val[r * 8 + 7] <= thr) {
        const int pos = atomicAdd(n_overflow, 1);
        overflow_rows[pos] = r;
        return;
    }
    const float* xr = x + r * dim;
    float bd = __int_as_float(0x7f800000);
    int bi = 0x7fffffff;
    for (int c = 0; c < 8; c++) {
        const int idx = cand_idx[r * 8 + c];
        if (idx < 0 || cand_val[r * 8 + c] > thr) break;
        const float* cr = cent + (int64_t)idx * dim;
        const float d = (dim & 3) == 0 ? sqeuclid_ref_v4(xr, cr, dim) : sqeuclid_ref(xr, cr, dim);
        if (d < bd || (d == bd && idx < bi)) {
            bd = d;
            bi = idx;
        }
    }
    out_idx[r] = bi == 0x7fffffff ? 0 : bi;
    if (out_d2) out_d2[r] = bd;
}

// How far each centroid moved since the previous assignment: ||new - old||
// (FP32, rounded up by a relative 1e-5 so it bounds the exact norm). One warp
// per centroid.
__global__ void centroid_shift_kernel(const float* __restrict__ cnew, const float* __restrict__ cold, int k, int dim,
                                      float* __restrict__ shift) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= k) return;
    float acc = 0.0f;
    for (int e = lane; e < dim; e += 32) {
        const float t = cnew[(int64_t)c * dim + e] - cold[(int64_t)c * dim + e];
        acc = fmaf(t, t, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) shift[c] = sqrtf(acc) * 1.00001f + 1e-30f;
}

// The warm filter's bound on each row's best screened score. The row's
// previous centroid c was at squared distance d2 (the reference-order FP32
// value); it has moved by at most shift[c], so its exact score now, ||c||^2 -
// 2 <x, c> = dist^2 - ||x||^2, is at most (sqrt(d2) + shift)^2 - ||x||^2, and
// so is the exact score of the row's nearest centroid; its screened score
// exceeds that by at most the screen's eps. The FP32 roundings of d2, the
// shift and ||x||^2 (relative 1e-5 here, about 128 x 2^-24 at most) and of
// the reference's distance (the 2e-5 slack the top-8 rescore uses) are
// added on top.
__global__ void warm_bound_kernel(const float* __restrict__ d2, const int32_t* __restrict__ prev,
                                  const float* __restrict__ shift, const float* __restrict__ xn2,
                                  const float* __restrict__ xres, const float* __restrict__ cmax_p, int kp, int64_t n,
                                  float* __restrict__ rthr) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float eps = bf16_score_eps(sqrtf(xn2[r]), xres[r], cmax_p[0], cmax_p[1], kp);
    const float rt = sqrtf(fmaxf(d2[r], 0.0f) * 1.00001f) + shift[prev[r]] * 1.00001f;
    const float u = rt * rt * 1.00001f - xn2[r] * 0.99999f;
    rthr[r] = u + eps + 2e-5f * (fabsf(u) + xn2[r]);
}

// The exact nearest centroid of every row among its filtered candidates
// (cand_id [n][cap], count cnt[r]): reference-order FP32 distances, the
// lowest index on a tie. The filter kept every centroid whose screened score
// is under the row's warm bound, the nearest one among them; rows whose
// count passed cap (or is 0) go to the exact kernel.
__global__ void rescore_filtered_kernel(const float* __restrict__ x, int64_t n, int dim, const float* __restrict__ cent,
                                        const int32_t* __restrict__ cnt, const int32_t* __restrict__ cand_id, int cap,
                                        int32_t* __restrict__ out_idx, float* __restrict__ out_d2,
                                        int64_t* __restrict__ overflow_rows, int* __restrict__ n_overflow) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int c = cnt[r];
    if (c <= 0 || c > cap) {
        overflow_rows[atomicAdd(n_overflow, 1)] = r;
        return;
    }
    const float* xr = x + r * dim;
    float bd = __int_as_float(0x7f800000);
    int bi = 0x7fffffff;
    for (int i = 0; i < c; i++) {
        const int idx = cand_id[r * cap + i];
        const float* cr = cent + (int64_t)idx * dim;
        const float d = (dim & 3) == 0 ? sqeuclid_ref_v4(xr, cr, dim) : sqeuclid_ref(xr, cr, dim);
        if (d < bd || (d == bd && idx < bi)) {
            bd = d;
            bi = idx;
        }
    }
    out_idx[r] = bi;
    out_d2[r] = bd;
}

__global__ void norm_maxes_kernel(const float* __restrict__ v, const float* __restrict__ res, int n,
                                  float* __restrict__ out) {
    __shared__ float red[256], red2[256];
    float m = 0.0f, m2 = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        m = fmaxf(m, sqrtf(fmaxf(v[i], 0.0f)));
        m2 = fmaxf(m2, res[i]);
    }
    red[threadIdx.x] = m;
    red2[threadIdx.x] = m2;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
            red2[threadIdx.x] = fmaxf(red2[threadIdx.x], red2[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = red[0] * 1.0001f;
        out[1] = red2[0];
    }
}

__global__ void scatter_i32_kernel(const int32_t* __restrict__ src, const int64_t* __restrict__ rows, const int* n,
                                   int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *n) out[rows[i]] = src[i];
}

}  // namespace

cudaError_t launch_probe_select_band(float* S, const float* Q, const float* qn2, const float* qres, int64_t nq,
                                     int dim, int kp, const float* coarse, const float* cmax, int nlist,
                                     const int32_t* nprobe,
                                     int np_max, const int32_t* k, const int32_t* list_len, int allow_fallback,
                                     int32_t* probe_ids, float* probe_d, int32_t* fallback,
                                     unsigned long long* fallback_count, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (np_max > PB_MAX || dim > QMAX) return cudaErrorInvalidValue;
    // The score row lives in shared memory when it fits beside the 34 KiB of
    // static buffers.
    const size_t row_bytes = (size_t)nlist * sizeof(float);
    const int in_smem = row_bytes <= 160 * 1024 ? 1 : 0;
    const size_t dyn = in_smem ? row_bytes : 0;
    // static buffers (about 34 KiB) plus the row can pass the 48 KiB default
    cudaError_t e = cudaFuncSetAttribute(probe_select_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         160 * 1024);
    if (e != cudaSuccess) return e;
    probe_select_band_kernel<<<(unsigned)nq, PB_THREADS, dyn, s>>>(S, Q, qn2, qres, dim, kp, coarse, cmax, nlist,
                                                                  nprobe,
                                                                  np_max, k, list_len, allow_fallback, probe_ids,
                                                                  probe_d, fallback, fallback_count, in_smem);
    return cudaGetLastError();
}

size_t probe_final_smem(int lcap, int np_max) {
    int P = 1;
    while (P < np_max) P <<= 1;
    return (size_t)(lcap + P) * sizeof(unsigned long long);
}

cudaError_t launch_probe_final(const float* Q, int64_t nq, int dim, const float* coarse, int nlist,
                               const int32_t* nprobe, int np_max, const int32_t* k, const int32_t* list_len,
                               int allow_fallback, int lcap, const unsigned long long* band, const int32_t* lcount,
                               const int32_t* need_exact, float* Drow, int32_t* probe_ids, float* probe_d,
                               int32_t* fallback, unsigned long long* fallback_count, int32_t* todo, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (np_max > PB_MAX || dim > QMAX || lcap < np_max) return cudaErrorInvalidValue;
    const size_t smem = probe_final_smem(lcap, np_max);
    cudaError_t e = cudaFuncSetAttribute(probe_final_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int32_t* todo_count = todo + nq;
    e = cudaMemsetAsync(todo_count, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    probe_final_warp_kernel<<<(unsigned)ceil_div(nq, PFW_WARPS), PFW_WARPS * 32, 0, s>>>(
        Q, nq, dim, coarse, nlist, nprobe, np_max, k, list_len, allow_fallback, lcap, band, lcount, need_exact,
        probe_ids, probe_d, fallback, fallback_count, todo, todo_count);
    // the queries the warp form left: a grid of a few blocks per SM walks the list
    probe_final_kernel<<<(unsigned)std::min<int64_t>(nq, 4 * 152), PB_THREADS, smem, s>>>(
        Q, dim, coarse, nlist, nprobe, np_max, k, list_len, allow_fallback, lcap, band, lcount, need_exact, Drow,
        probe_ids, probe_d, fallback, fallback_count, todo, todo_count);
    return cudaGetLastError();
}

cudaError_t launch_rescore_top8(const float* x, const float* xn2, const float* xres, int64_t n, int dim, int kp,
                                const float* cent, int k, const float* cmax, const int32_t* cand_idx,
                                const float* cand_val, int32_t* out_idx, float* out_d2, int64_t* overflow_rows,
                                int* n_overflow, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    rescore_top8_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(x, xn2, xres, n, dim, kp, cent, k, cmax, cand_idx,
                                                                   cand_val, out_idx, out_d2, overflow_rows,
                                                                   n_overflow);
    return cudaGetLastError();
}

cudaError_t launch_centroid_shift(const float* cnew, const float* cold, int k, int dim, float* shift,
                                  cudaStream_t s) {
    if (k <= 0) return cudaSuccess;
    centroid_shift_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, s>>>(cnew, cold, k, dim, shift);
    return cudaGetLastError();
}

cudaError_t launch_warm_bound(const float* d2, const int32_t* prev, const float* shift, const float* xn2,
                              const float* xres, const float* cmax, int kp, int64_t n, float* rthr, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    warm_bound_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(d2, prev, shift, xn2, xres, cmax, kp, n, rthr);
    return cudaGetLastError();
}

cudaError_t launch_rescore_filtered(const float* x, int64_t n, int dim, const float* cent, const int32_t* cnt,
                                    const int32_t* cand_id, int cap, int32_t* out_idx, float* out_d2,
                                    int64_t* overflow_rows, int* n_overflow, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    rescore_filtered_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(x, n, dim, cent, cnt, cand_id, cap, out_idx,
                                                                       out_d2, overflow_rows, n_overflow);
    return cudaGetLastError();
}

cudaError_t launch_norm_maxes(const float* sqnorm, const float* resid, int n, float* out, cudaStream_t s) {
    norm_maxes_kernel<<<1, 256, 0, s>>>(sqnorm, resid, n, out);
    return cudaGetLastError();
}

cudaError_t launch_scatter_i32(const int32_t* src, const int64_t* rows, const int* n, int64_t cap, int32_t* out,
                               cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    scatter_i32_kernel<<<(unsigned)ceil_div(cap, 256), 256, 0, s>>>(src, rows, n, out);
    return cudaGetLastError();
}

}  // namespace hann
