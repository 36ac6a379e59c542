// kernels_knn.cu -- batched exact k-nearest-neighbour search over a flat base
// (testutil.BruteForceKNN, internal/testutil/data.go:66-93, over the batch
// distance kernels simd_<metric>_batch, core/simd_kernels.inc.h:235-264).
//
// Results are ordered by (distance, row) with the distance exactly the
// reference's FP32 value for the metric, so ids and distances equal the
// reference's on any input. Two ways produce them:
//
//   * exact SIMT: knn_filter_kernel computes reference-order distances in
//     register tiles (tile_dist.cuh) for one chunk of base rows and keeps,
//     per query, only the pairs whose (distance, row) key is below the key of
//     the query's current k-th neighbour; knn_merge_exact_kernel folds them
//     into the query's sorted top-k list. Keys compare (distance, row), so the
//     filter is exact in any chunk order.
//   * tensor-core screen: the BF16 GEMM (kernels_gemm.cu, filter mode) ranks
//     rows by an approximate score s~ with |s~ - s| <= eps; per query a band
//     list keeps every row with s~ <= T~ + 2 eps + slack, T~ the k-th
//     smallest s~ seen (knn_merge_band_kernel); knn_final_band_kernel
//     rescores the band with the exact metric and keeps the best k. The exact
//     top k always lies in the band (see knn_merge_band_kernel).
#include "common.cuh"
#include "kernels.h"
#include "select.cuh"
#include "tile_dist.cuh"

#include <algorithm>

namespace hann {
namespace {

constexpr int KF_THREADS = 256;
constexpr int KF_TP = 128;  // query rows per block
constexpr int KF_TC = 32;   // base rows per tile
constexpr int KM_THREADS = 256;

template <int METRIC>
struct MetricOp {
    static constexpr int op = METRIC == 2 ? OP_ABSDIFF : (METRIC == 3 ? OP_DOT : OP_SQDIFF);
};

// Output distance from the tile accumulation: squared Euclidean as is,
// Euclidean as its FP32 square root, Manhattan as is, cosine from the dot
// product and the two reference-order squared norms.
template <int METRIC>
__device__ __forceinline__ float finish(float acc, float qn, float bn) {
    if (METRIC == 1) return __fsqrt_rn(acc);
    if (METRIC == 3) return cosine_from_parts(acc, qn, bn);
    return acc;
}

__device__ __forceinline__ unsigned long long dkey(float d, uint32_t row) {
    return ((unsigned long long)float_key(d) << 32) | row;
}

template <int METRIC>
__device__ __forceinline__ float metric_ref(const float* q, const float* b, int dim, float qn, float bn) {
    if (METRIC == 0) return (dim & 3) == 0 ? sqeuclid_ref_v4(q, b, dim) : sqeuclid_ref(q, b, dim);
    if (METRIC == 1) return __fsqrt_rn((dim & 3) == 0 ? sqeuclid_ref_v4(q, b, dim) : sqeuclid_ref(q, b, dim));
    if (METRIC == 2) return manhattan_ref(q, b, dim);
    return cosine_from_parts(dot_ref(q, b, dim), qn, bn);
}

// Filter (MATRIX false) or distance matrix (MATRIX true) over base rows
// [c_begin, c_end). Block row r stands for query qi = qlist ? qlist[r] : r,
// which indexes the query vector and every per-query array (threshold,
// counter, candidate buffer); with MATRIX the distance goes to
// out_mat[r * ld + (col - c_begin)].
template <int METRIC, bool MATRIX>
__global__ void __launch_bounds__(KF_THREADS) knn_filter_kernel(
    const float* __restrict__ queries, const int32_t* __restrict__ qlist, int nrows, int dim,
    const float* __restrict__ base, int64_t c_begin, int64_t c_end, int tiles_per_split,
    const float* __restrict__ qnorm, const float* __restrict__ bnorm, const unsigned long long* __restrict__ thr,
    int cap, int32_t* __restrict__ cnt, int32_t* __restrict__ cand_id, float* __restrict__ cand_d,
    double* __restrict__ out_mat, int64_t ld) {
    constexpr int OP = MetricOp<METRIC>::op;
    extern __shared__ __align__(16) float sm[];
    float* Xs = sm;
    float* Cs = sm + dim * KF_TP;
    const int tid = threadIdx.x;
    const int tp = tid & 31, tc = tid >> 5;
    const int r0 = blockIdx.x * KF_TP;
    stage_tile<KF_TP, KF_THREADS>(Xs, dim, min(KF_TP, nrows - r0), [&](int p) {
        const int64_t qi = qlist ? qlist[r0 + p] : r0 + p;
        return queries + qi * dim;
    });
    unsigned long long t_row[4];
    float qn[4];
    int64_t qrow[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int r = r0 + 4 * tp + a;
        t_row[a] = 0ull;
        qn[a] = 0.0f;
        qrow[a] = r;
        if (r < nrows) {
            const int64_t qi = qlist ? qlist[r] : r;
            qrow[a] = qi;
            if (!MATRIX) t_row[a] = thr[qi];
            if (METRIC == 3) qn[a] = qnorm[qi];
        }
    }
    const int64_t cb0 = c_begin + (int64_t)blockIdx.y * tiles_per_split * KF_TC;
    const int64_t cb1 = min(c_end, cb0 + (int64_t)tiles_per_split * KF_TC);
    for (int64_t c0 = cb0; c0 < cb1; c0 += KF_TC) {
        __syncthreads();
        stage_tile<KF_TC, KF_THREADS>(Cs, dim, (int)min((int64_t)KF_TC, cb1 - c0),
                                      [&](int c) { return base + (c0 + c) * dim; });
        __syncthreads();
        float dd[4][4];
        tile_pairs<OP, KF_TP, KF_TC>(Xs, Cs, tp, tc, dim, dd);
        float bn[4];
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int64_t col = c0 + 4 * tc + b;
            bn[b] = (METRIC == 3 && col < cb1) ? bnorm[col] : 0.0f;
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int r = r0 + 4 * tp + a;
            if (r >= nrows) continue;
            float d[4];
            unsigned pass = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int64_t col = c0 + 4 * tc + b;
                d[b] = finish<METRIC>(dd[a][b], qn[a], bn[b]);
                if (col < cb1) {
                    if (MATRIX) out_mat[(int64_t)r * ld + (col - c_begin)] = (double)d[b];
                    else if (dkey(d[b], (uint32_t)col) < t_row[a]) pass |= 1u << b;
                }
            }
            if (!MATRIX && pass) {
                const int64_t qi = qrow[a];
                int pos = atomicAdd(&cnt[qi], __popc(pass));
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    if (pass & (1u << b)) {
                        if (pos < cap) {
                            cand_id[qi * cap + pos] = (int32_t)(c0 + 4 * tc + b);
                            cand_d[qi * cap + pos] = d[b];
                        }
                        pos++;
                    }
                }
            }
        }
    }
}

// One thread per (query row, base row) pair, for dimensions beyond the tile
// limit. Same outputs as knn_filter_kernel.
template <int METRIC, bool MATRIX>
__global__ void knn_filter_generic_kernel(const float* __restrict__ queries, const int32_t* __restrict__ qlist,
                                          int nrows, int dim, const float* __restrict__ base, int64_t c_begin,
                                          int64_t c_end, const float* __restrict__ qnorm,
                                          const float* __restrict__ bnorm,
                                          const unsigned long long* __restrict__ thr, int cap,
                                          int32_t* __restrict__ cnt, int32_t* __restrict__ cand_id,
                                          float* __restrict__ cand_d, double* __restrict__ out_mat, int64_t ld) {
    const int64_t width = c_end - c_begin;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= width * nrows) return;
    const int r = (int)(e / width);
    const int64_t col = c_begin + (e - (int64_t)r * width);
    const int64_t qi = qlist ? qlist[r] : r;
    const float d = metric_ref<METRIC>(queries + qi * dim, base + col * dim, dim, METRIC == 3 ? qnorm[qi] : 0.0f,
                                       METRIC == 3 ? bnorm[col] : 0.0f);
    if (MATRIX) {
        out_mat[(int64_t)r * ld + (col - c_begin)] = (double)d;
    } else if (dkey(d, (uint32_t)col) < thr[qi]) {
        const int pos = atomicAdd(&cnt[qi], 1);
        if (pos < cap) {
            cand_id[qi * cap + pos] = (int32_t)col;
            cand_d[qi * cap + pos] = d;
        }
    }
}

// Fold one chunk's candidates into each query's sorted top-k list of
// (distance, row) keys. A row whose candidates overflowed the buffer keeps
// its list and is flagged so the chunk can be rerun in smaller pieces.
__global__ void __launch_bounds__(KM_THREADS) knn_merge_exact_kernel(
    const int32_t* __restrict__ qlist, int k, int cap, int32_t* __restrict__ cnt, const int32_t* __restrict__ cand_id,
    const float* __restrict__ cand_d, unsigned long long* __restrict__ list, int32_t* __restrict__ lcount,
    unsigned long long* __restrict__ thr, int32_t* __restrict__ redo, int* __restrict__ redo_count) {
    extern __shared__ __align__(16) unsigned long long keys[];
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_and, s_or, s_prefix;
    __shared__ unsigned int s_rem;
    __shared__ int s_pos;
    const int64_t r = qlist ? (int64_t)qlist[blockIdx.x] : (int64_t)blockIdx.x;
    const int c = cnt[r];
    if (c == 0) return;
    if (c > cap) {
        if (threadIdx.x == 0) {
            redo[r] = 1;
            atomicAdd(redo_count, 1);
            cnt[r] = 0;
        }
        return;
    }
    const int L = lcount[r];
    for (int i = threadIdx.x; i < L; i += KM_THREADS) keys[i] = list[r * k + i];
    for (int i = threadIdx.x; i < c; i += KM_THREADS)
        keys[L + i] = dkey(cand_d[r * cap + i], (uint32_t)cand_id[r * cap + i]);
    const int T = L + c;
    int P = 1;
    while (P < min(T, k)) P <<= 1;
    unsigned long long* out = keys + T;
    __syncthreads();
    if (T > k) {
        const unsigned long long K = radix_nth_u64(keys, T, k, hist, &s_and, &s_or, &s_prefix, &s_rem);
        if (threadIdx.x == 0) s_pos = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < T; i += KM_THREADS) {
            if (keys[i] <= K) out[atomicAdd(&s_pos, 1)] = keys[i];
        }
    } else {
        for (int i = threadIdx.x; i < T; i += KM_THREADS) out[i] = keys[i];
    }
    const int m = min(T, k);
    for (int i = m + threadIdx.x; i < P; i += KM_THREADS) out[i] = ~0ull;
    __syncthreads();
    sort_u64(out, P);
    for (int i = threadIdx.x; i < m; i += KM_THREADS) list[r * k + i] = out[i];
    if (threadIdx.x == 0) {
        lcount[r] = m;
        thr[r] = m == k ? out[k - 1] : ~0ull;
        cnt[r] = 0;
    }
}

// Band merge for the tensor-core screen. Keys are (float_key(s~), row).
// Invariant: after every merge the list holds every row seen so far with
// s~ <= thr = T~ + e2 + 2e-5 (|T~| + a), T~ the k-th smallest s~ seen, e2 =
// 2 eps. Rows the GEMM dropped had s~ above an earlier, larger threshold, and
// the threshold only falls, so the final list holds every row with s~ <= the
// final threshold. The exact top k lies inside it: k rows have s~ <= T~, so
// their exact scores are <= T~ + eps, so the k-th exact score is too, and any
// row at or below it has s~ <= T~ + 2 eps (plus the FP32 rounding of the
// reference's distance, covered by the relative slack).
// A list that would exceed lcap, or a candidate buffer that overflowed,
// sends the query to the exact SIMT path (need_exact) and stops its screen.
// krow (optional) gives a per-row k, capped at k.
__device__ __forceinline__ void merge_band_row(
    int64_t r, int k, const int32_t* __restrict__ krow, int cap, int lcap, int32_t* __restrict__ cnt,
    const int32_t* __restrict__ cand_id,
    const float* __restrict__ cand_s, const float* __restrict__ e2, const float* __restrict__ asl,
    unsigned long long* __restrict__ list, int32_t* __restrict__ lcount, float* __restrict__ thr,
    int32_t* __restrict__ need_exact) {
    extern __shared__ __align__(16) unsigned long long keys[];
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_and, s_or, s_prefix;
    __shared__ unsigned int s_rem;
    __shared__ int s_pos;
    const int c = cnt[r];
    if (c == 0) return;
    if (need_exact[r] || c > cap) {
        if (threadIdx.x == 0) {
            need_exact[r] = 1;
            thr[r] = -__int_as_float(0x7f800000);
            cnt[r] = 0;
        }
        return;
    }
    const int L = lcount[r];
    const int kr = krow ? max(1, min(krow[r], k)) : k;
    for (int i = threadIdx.x; i < L; i += KM_THREADS) keys[i] = list[r * lcap + i];
    for (int i = threadIdx.x; i < c; i += KM_THREADS)
        keys[L + i] = dkey(cand_s[r * cap + i], (uint32_t)cand_id[r * cap + i]);
    const int T = L + c;
    __syncthreads();
    float t_new = __int_as_float(0x7f800000);
    if (T >= kr) {
        const unsigned long long K = radix_nth_u64(keys, T, kr, hist, &s_and, &s_or, &s_prefix, &s_rem);
        const float tk = key_float((uint32_t)(K >> 32));
        t_new = tk + e2[r] + 2e-5f * (fabsf(tk) + asl[r]);
    }
    if (threadIdx.x == 0) s_pos = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < T; i += KM_THREADS) {
        const unsigned long long key = keys[i];
        if (key_float((uint32_t)(key >> 32)) <= t_new) {
            const int pos = atomicAdd(&s_pos, 1);
            if (pos < lcap) list[r * lcap + pos] = key;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int m = s_pos;
        if (m > lcap) {
            need_exact[r] = 1;
            thr[r] = -__int_as_float(0x7f800000);
        } else {
            lcount[r] = m;
            thr[r] = t_new;
        }
        cnt[r] = 0;
    }
}

// Block merge of the rows in todo[0, *todo_count) (the rows the warp form
// left), or of row blockIdx.x when todo is null.
__global__ void __launch_bounds__(KM_THREADS) knn_merge_band_kernel(
    int k, const int32_t* __restrict__ krow, int cap, int lcap, int32_t* __restrict__ cnt,
    const int32_t* __restrict__ cand_id,
    const float* __restrict__ cand_s, const float* __restrict__ e2, const float* __restrict__ asl,
    unsigned long long* __restrict__ list, int32_t* __restrict__ lcount, float* __restrict__ thr,
    int32_t* __restrict__ need_exact, const int32_t* __restrict__ todo, const int32_t* __restrict__ todo_count) {
    if (!todo) {
        merge_band_row(blockIdx.x, k, krow, cap, lcap, cnt, cand_id, cand_s, e2, asl, list, lcount, thr, need_exact);
        return;
    }
    const int n = *todo_count;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        merge_band_row(todo[i], k, krow, cap, lcap, cnt, cand_id, cand_s, e2, asl, list, lcount, thr, need_exact);
        __syncthreads();
    }
}

// Warp merge capacities: band list + candidates up to which one warp merges
// a row. The small form (8 warps a block) serves the probe's bands; rows of
// a k-NN with k > 32 carry about 8 k keys after a chunk, for the large form
// (4 warps a block, 16 KB of keys each).
constexpr int MW_MAX = 512;
constexpr int MW_WARPS = 8;
constexpr int MW_MAX_L = 2048;
constexpr int MW_WARPS_L = 4;
template <int CAPK, int WARPS>
constexpr size_t merge_warp_smem() {
    return (size_t)WARPS * CAPK * sizeof(unsigned long long) + (size_t)WARPS * 256 * sizeof(unsigned int);
}

// One warp per row when the row's band list and new candidates together
// hold at most CAPK keys: the same merge as knn_merge_band_kernel without
// block barriers. A row it merges has its candidate count reset, so the
// block kernel launched after it skips the row; rows it leaves (larger, or
// flagged) go to the block kernel.
template <int CAPK, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) knn_merge_band_warp_kernel(
    int nrows, int k, const int32_t* __restrict__ krow, int cap, int lcap, int32_t* __restrict__ cnt,
    const int32_t* __restrict__ cand_id, const float* __restrict__ cand_s, const float* __restrict__ e2,
    const float* __restrict__ asl, unsigned long long* __restrict__ list, int32_t* __restrict__ lcount,
    float* __restrict__ thr, const int32_t* __restrict__ need_exact, int32_t* __restrict__ todo,
    int32_t* __restrict__ todo_count) {
    extern __shared__ __align__(16) unsigned long long mw_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned int* hist = reinterpret_cast<unsigned int*>(mw_smem + WARPS * CAPK) + w * 256;
    const int64_t r = (int64_t)blockIdx.x * WARPS + w;
    if (r >= nrows) return;
    const int c = cnt[r];
    const int L = lcount[r];
    if (c == 0) return;
    if (need_exact[r] || c > cap || L + c > CAPK) {
        // left to the block kernel
        if (lane == 0) todo[atomicAdd(todo_count, 1)] = (int32_t)r;
        return;
    }
    unsigned long long* keys = mw_smem + w * CAPK;
    const int kr = krow ? max(1, min(krow[r], k)) : k;
    // the band list and the new candidates, 128 entries of each at a time
    // with all their loads in flight
    for (int i0 = 0; i0 < max(L, c); i0 += 128) {
        unsigned long long lv[4];
        float cs[4];
        uint32_t ci[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = i0 + 32 * u + lane;
            lv[u] = i < L ? list[r * lcap + i] : 0ull;
            cs[u] = i < c ? cand_s[r * cap + i] : 0.0f;
            ci[u] = i < c ? (uint32_t)cand_id[r * cap + i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = i0 + 32 * u + lane;
            if (i < L) keys[i] = lv[u];
            if (i < c) keys[L + i] = dkey(cs[u], ci[u]);
        }
    }
    const int T = L + c;
    __syncwarp();
    float t_new = __int_as_float(0x7f800000);
    if (T >= kr) {
        const unsigned long long K = warp_radix_nth_u64(keys, T, kr, hist);
        const float tk = key_float((uint32_t)(K >> 32));
        t_new = tk + e2[r] + 2e-5f * (fabsf(tk) + asl[r]);
    }
    int m = 0;
    for (int i0 = 0; i0 < T; i0 += 32) {
        const int i = i0 + lane;
        const unsigned long long key = i < T ? keys[i] : 0ull;
        const bool keep = i < T && key_float((uint32_t)(key >> 32)) <= t_new;
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if (keep) list[r * lcap + m + __popc(b & ((1u << lane) - 1u))] = key;
        m += __popc(b);
    }
    if (lane == 0) {
        lcount[r] = m;  // m <= T <= CAPK <= lcap
        thr[r] = t_new;
        cnt[r] = 0;
    }
}

// Exact rescoring of each query's band and the final top k, written as
// (id, distance). Queries flagged need_exact are appended to exact_list.
template <int METRIC>
__global__ void __launch_bounds__(KM_THREADS) knn_final_band_kernel(
    int k, int lcap, int dim, const float* __restrict__ queries, const float* __restrict__ base,
    const float* __restrict__ qnorm, const float* __restrict__ bnorm, const unsigned long long* __restrict__ list,
    const int32_t* __restrict__ lcount, const int32_t* __restrict__ need_exact, int32_t* __restrict__ exact_list,
    int* __restrict__ exact_count, int64_t* __restrict__ out_ids, double* __restrict__ out_dist) {
    extern __shared__ __align__(16) unsigned long long keys[];
    __shared__ unsigned int hist[256];
    __shared__ unsigned long long s_and, s_or, s_prefix;
    __shared__ unsigned int s_rem;
    __shared__ int s_pos;
    __shared__ float qv[KNN_TC_DMAX];
    const int64_t r = blockIdx.x;
    if (need_exact[r]) {
        if (threadIdx.x == 0) exact_list[atomicAdd(exact_count, 1)] = (int32_t)r;
        return;
    }
    for (int i = threadIdx.x; i < dim; i += KM_THREADS) qv[i] = queries[r * dim + i];
    const int L = lcount[r];
    const float qn = METRIC == 3 ? qnorm[r] : 0.0f;
    __syncthreads();
    for (int i = threadIdx.x; i < L; i += KM_THREADS) {
        const uint32_t row = (uint32_t)(list[r * lcap + i] & 0xffffffffull);
        const float d = metric_ref<METRIC>(qv, base + (int64_t)row * dim, dim, qn, METRIC == 3 ? bnorm[row] : 0.0f);
        keys[i] = dkey(d, row);
    }
    __syncthreads();
    const int m = min(L, k);
    int P = 1;
    while (P < m) P <<= 1;
    unsigned long long* out = keys + L;
    if (L > k) {
        const unsigned long long K = radix_nth_u64(keys, L, k, hist, &s_and, &s_or, &s_prefix, &s_rem);
        if (threadIdx.x == 0) s_pos = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < L; i += KM_THREADS)
            if (keys[i] <= K) out[atomicAdd(&s_pos, 1)] = keys[i];
    } else {
        for (int i = threadIdx.x; i < L; i += KM_THREADS) out[i] = keys[i];
    }
    for (int i = m + threadIdx.x; i < P; i += KM_THREADS) out[i] = ~0ull;
    __syncthreads();
    if (P > 1) sort_u64(out, P);
    for (int i = threadIdx.x; i < k; i += KM_THREADS) {
        if (i < m) {
            out_ids[r * k + i] = (int64_t)(out[i] & 0xffffffffull);
            out_dist[r * k + i] = (double)key_float((uint32_t)(out[i] >> 32));
        } else {
            out_ids[r * k + i] = -1;
            out_dist[r * k + i] = (double)__int_as_float(0x7f800000);
        }
    }
}

// Sorted exact lists to (id, distance) for rows qlist[p] (or every row).
__global__ void knn_emit_kernel(int nrows, int k, const unsigned long long* __restrict__ list,
                                const int32_t* __restrict__ lcount, const int32_t* __restrict__ qlist,
                                int64_t* __restrict__ out_ids, double* __restrict__ out_dist) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)nrows * k) return;
    const int p = (int)(e / k), i = (int)(e - (int64_t)p * k);
    const int64_t r = qlist ? (int64_t)qlist[p] : p;
    const int64_t o = r * k + i;
    if (i < lcount[r]) {
        const unsigned long long key = list[r * k + i];
        out_ids[o] = (int64_t)(key & 0xffffffffull);
        out_dist[o] = (double)key_float((uint32_t)(key >> 32));
    } else {
        out_ids[o] = -1;
        out_dist[o] = (double)__int_as_float(0x7f800000);
    }
}

// Reference-order squared norms dot_ref(x, x) (the cosine kernel's norm
// accumulations), one warp-free thread per row.
__global__ void ref_sqnorm_kernel(const float* __restrict__ x, int64_t n, int dim, float* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float* p = x + r * dim;
    out[r] = dot_ref(p, p, dim);
}

// Per-column epilogue terms of the screen score s~ = t.x + t.y * <q~, b~>:
// squared Euclidean (and Euclidean) t = (||b||^2, -2); cosine t = (0,
// -1/||b||), zero for a zero row (its cosine distance is 1 whatever the
// query). The maxima for the error bound: out[0] = max |b| (rounded up),
// out[1] = max |b - b~| (L2) or max |b - b~| / |b| (cosine).
__global__ void knn_col_terms_kernel(const float* __restrict__ sqnorm, const float* __restrict__ resid, int64_t n,
                                     int cosine, float2* __restrict__ terms, unsigned int* __restrict__ maxes) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float m0 = 0.0f, m1 = 0.0f;
    if (r < n) {
        const float nb = sqrtf(fmaxf(sqnorm[r], 0.0f));
        if (cosine) {
            terms[r] = nb > 0.0f ? make_float2(0.0f, -1.0f / nb) : make_float2(0.0f, 0.0f);
            m1 = nb > 0.0f ? resid[r] / nb * 1.0001f : 0.0f;
        } else {
            terms[r] = make_float2(sqnorm[r], -2.0f);
            m1 = resid[r];
        }
        m0 = nb * 1.0001f;
    }
    // non-negative floats order like their bit patterns
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 16));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 16));
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 8));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 8));
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 4));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 4));
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 2));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 2));
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 1));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 1));
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&maxes[0], __float_as_uint(m0));
        atomicMax(&maxes[1], __float_as_uint(m1));
    }
}

// Per-query band constants: e2 = 2 eps and the slack scale a (||q||^2 for
// the squared score, ||q|| for cosine). For cosine eps bounds
// |s~ - s| with s = -<q, b>/|b|:
//   operand rounding  ar + |q~| rho           (rho = max |b - b~| / |b|)
//   accumulation      kp 2^-22 |q~| (1 + rho)
//   the 1/|b| factor and the final product: 16 ulps of |q~| (1 + rho)
__global__ void knn_query_band_kernel(const float* __restrict__ qsq, const float* __restrict__ qres, int64_t nq,
                                      int kp, int cosine, const unsigned int* __restrict__ maxes,
                                      float* __restrict__ e2, float* __restrict__ asl) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nq) return;
    const float an = sqrtf(fmaxf(qsq[r], 0.0f)), ar = qres[r];
    const float m0 = __uint_as_float(maxes[0]), m1 = __uint_as_float(maxes[1]);
    if (cosine) {
        const float at = an + ar;
        const float u22 = 2.384185791015625e-7f, u24 = 5.9604644775390625e-8f;
        const float eps = ar + at * m1 + (float)kp * u22 * at * (1.0f + m1) + 16.0f * u24 * at * (1.0f + m1);
        e2[r] = 2.0f * eps;
        asl[r] = an;
    } else {
        e2[r] = 2.0f * bf16_score_eps(an, ar, m0, m1, kp);
        asl[r] = qsq[r];
    }
}

template <int METRIC, bool MATRIX>
cudaError_t launch_filter_t(const float* q, const int32_t* qlist, int nrows, int dim, const float* base,
                            int64_t c_begin, int64_t c_end, const float* qnorm, const float* bnorm,
                            const unsigned long long* thr, int cap, int32_t* cnt, int32_t* cand_id, float* cand_d,
                            double* out_mat, int64_t ld, cudaStream_t s) {
    if (nrows <= 0 || c_end <= c_begin) return cudaSuccess;
    if (dim <= KNN_SIMT_DMAX) {
        const size_t smem = (size_t)dim * (KF_TP + KF_TC) * sizeof(float);
        cudaError_t e = cudaFuncSetAttribute(knn_filter_kernel<METRIC, MATRIX>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)((size_t)KNN_SIMT_DMAX * (KF_TP + KF_TC) * sizeof(float)));
        if (e != cudaSuccess) return e;
        const int64_t qtiles = ceil_div(nrows, KF_TP);
        const int64_t tiles = ceil_div(c_end - c_begin, KF_TC);
        // about four waves of one block per SM
        int64_t splits = std::min<int64_t>(tiles, std::max<int64_t>(1, ceil_div(4 * 152, qtiles)));
        const int64_t per = ceil_div(tiles, splits);
        splits = ceil_div(tiles, per);
        knn_filter_kernel<METRIC, MATRIX><<<dim3((unsigned)qtiles, (unsigned)splits), KF_THREADS, smem, s>>>(
            q, qlist, nrows, dim, base, c_begin, c_end, (int)per, qnorm, bnorm, thr, cap, cnt, cand_id, cand_d,
            out_mat, ld);
    } else {
        const int64_t total = (int64_t)nrows * (c_end - c_begin);
        knn_filter_generic_kernel<METRIC, MATRIX><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(
            q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt, cand_id, cand_d, out_mat, ld);
    }
    return cudaGetLastError();
}

template <bool MATRIX>
cudaError_t launch_filter_m(int metric, const float* q, const int32_t* qlist, int nrows, int dim, const float* base,
                            int64_t c_begin, int64_t c_end, const float* qnorm, const float* bnorm,
                            const unsigned long long* thr, int cap, int32_t* cnt, int32_t* cand_id, float* cand_d,
                            double* out_mat, int64_t ld, cudaStream_t s) {
    switch (metric) {
    case 0:
        return launch_filter_t<0, MATRIX>(q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt,
                                          cand_id, cand_d, out_mat, ld, s);
    case 1:
        return launch_filter_t<1, MATRIX>(q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt,
                                          cand_id, cand_d, out_mat, ld, s);
    case 2:
        return launch_filter_t<2, MATRIX>(q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt,
                                          cand_id, cand_d, out_mat, ld, s);
    case 3:
        return launch_filter_t<3, MATRIX>(q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt,
                                          cand_id, cand_d, out_mat, ld, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t set_smem_attr(const void* fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

cudaError_t launch_knn_filter(int metric, const float* q, const int32_t* qlist, int nrows, int dim, const float* base,
                              int64_t c_begin, int64_t c_end, const float* qnorm, const float* bnorm,
                              const unsigned long long* thr, int cap, int32_t* cnt, int32_t* cand_id, float* cand_d,
                              cudaStream_t s) {
    return launch_filter_m<false>(metric, q, qlist, nrows, dim, base, c_begin, c_end, qnorm, bnorm, thr, cap, cnt,
                                  cand_id, cand_d, nullptr, 0, s);
}

cudaError_t launch_knn_matrix(int metric, const float* q, int nrows, int dim, const float* base, int64_t c_begin,
                              int64_t c_end, const float* qnorm, const float* bnorm, double* out, int64_t ld,
                              cudaStream_t s) {
    return launch_filter_m<true>(metric, q, nullptr, nrows, dim, base, c_begin, c_end, qnorm, bnorm, nullptr, 0,
                                 nullptr, nullptr, nullptr, out, ld, s);
}

size_t knn_merge_exact_smem(int k, int cap) {
    int P = 1;
    while (P < k) P <<= 1;
    return (size_t)(k + cap + P) * sizeof(unsigned long long);
}

cudaError_t launch_knn_merge_exact(int nrows, const int32_t* qlist, int k, int cap, int32_t* cnt,
                                   const int32_t* cand_id,
                                   const float* cand_d, unsigned long long* list, int32_t* lcount,
                                   unsigned long long* thr, int32_t* redo, int* redo_count, cudaStream_t s) {
    if (nrows <= 0) return cudaSuccess;
    const size_t smem = knn_merge_exact_smem(k, cap);
    cudaError_t e = set_smem_attr((const void*)knn_merge_exact_kernel, smem);
    if (e != cudaSuccess) return e;
    knn_merge_exact_kernel<<<(unsigned)nrows, KM_THREADS, smem, s>>>(qlist, k, cap, cnt, cand_id, cand_d, list,
                                                                     lcount, thr, redo, redo_count);
    return cudaGetLastError();
}

size_t knn_merge_band_smem(int lcap, int cap) { return (size_t)(lcap + cap) * sizeof(unsigned long long); }

cudaError_t launch_knn_merge_band(int nrows, int k, const int32_t* krow, int cap, int lcap, int32_t* cnt,
                                  const int32_t* cand_id, const float* cand_s, const float* e2, const float* asl,
                                  unsigned long long* list, int32_t* lcount, float* thr, int32_t* need_exact,
                                  int32_t* todo, cudaStream_t s) {
    if (nrows <= 0) return cudaSuccess;
    const size_t smem = knn_merge_band_smem(lcap, cap);
    cudaError_t e = set_smem_attr((const void*)knn_merge_band_kernel, smem);
    if (e != cudaSuccess) return e;
    int32_t* todo_count = todo + nrows;
    const bool warp_form = lcap >= MW_MAX;
    if (warp_form) {
        e = cudaMemsetAsync(todo_count, 0, sizeof(int32_t), s);
        if (e != cudaSuccess) return e;
    }
    if (k > 32 && lcap >= MW_MAX_L) {
        constexpr size_t ws = merge_warp_smem<MW_MAX_L, MW_WARPS_L>();
        e = set_smem_attr((const void*)knn_merge_band_warp_kernel<MW_MAX_L, MW_WARPS_L>, ws);
        if (e != cudaSuccess) return e;
        knn_merge_band_warp_kernel<MW_MAX_L, MW_WARPS_L><<<(unsigned)ceil_div(nrows, MW_WARPS_L), MW_WARPS_L * 32, ws, s>>>(
            nrows, k, krow, cap, lcap, cnt, cand_id, cand_s, e2, asl, list, lcount, thr, need_exact, todo, todo_count);
    } else if (warp_form) {
        constexpr size_t ws = merge_warp_smem<MW_MAX, MW_WARPS>();
        e = set_smem_attr((const void*)knn_merge_band_warp_kernel<MW_MAX, MW_WARPS>, ws);
        if (e != cudaSuccess) return e;
        knn_merge_band_warp_kernel<MW_MAX, MW_WARPS><<<(unsigned)ceil_div(nrows, MW_WARPS), MW_WARPS * 32, ws, s>>>(
            nrows, k, krow, cap, lcap, cnt, cand_id, cand_s, e2, asl, list, lcount, thr, need_exact, todo, todo_count);
    }
    // the rows the warp form left: a grid of a few blocks per SM walks the list
    const unsigned grid = warp_form ? (unsigned)std::min<int64_t>(nrows, 4 * 152) : (unsigned)nrows;
    knn_merge_band_kernel<<<grid, KM_THREADS, smem, s>>>(k, krow, cap, lcap, cnt, cand_id, cand_s, e2, asl, list,
                                                         lcount, thr, need_exact, warp_form ? todo : nullptr,
                                                         todo_count);
    return cudaGetLastError();
}

cudaError_t launch_knn_final_band(int metric, int nrows, int k, int lcap, int dim, const float* queries,
                                  const float* base, const float* qnorm, const float* bnorm,
                                  const unsigned long long* list, const int32_t* lcount, const int32_t* need_exact,
                                  int32_t* exact_list, int* exact_count, int64_t* out_ids, double* out_dist,
                                  cudaStream_t s) {
    if (nrows <= 0) return cudaSuccess;
    if (dim > KNN_TC_DMAX) return cudaErrorInvalidValue;
    int P = 1;
    while (P < k) P <<= 1;
    const size_t smem = (size_t)(lcap + std::max(P, 1)) * sizeof(unsigned long long);
    const void* fn = nullptr;
    switch (metric) {
    case 0: fn = (const void*)knn_final_band_kernel<0>; break;
    case 1: fn = (const void*)knn_final_band_kernel<1>; break;
    case 3: fn = (const void*)knn_final_band_kernel<3>; break;
    default: return cudaErrorInvalidValue;
    }
    cudaError_t e = set_smem_attr(fn, smem);
    if (e != cudaSuccess) return e;
    switch (metric) {
    case 0:
        knn_final_band_kernel<0><<<(unsigned)nrows, KM_THREADS, smem, s>>>(
            k, lcap, dim, queries, base, qnorm, bnorm, list, lcount, need_exact, exact_list, exact_count, out_ids,
            out_dist);
        break;
    case 1:
        knn_final_band_kernel<1><<<(unsigned)nrows, KM_THREADS, smem, s>>>(
            k, lcap, dim, queries, base, qnorm, bnorm, list, lcount, need_exact, exact_list, exact_count, out_ids,
            out_dist);
        break;
    default:
        knn_final_band_kernel<3><<<(unsigned)nrows, KM_THREADS, smem, s>>>(
            k, lcap, dim, queries, base, qnorm, bnorm, list, lcount, need_exact, exact_list, exact_count, out_ids,
            out_dist);
        break;
    }
    return cudaGetLastError();
}

cudaError_t launch_knn_emit(int nrows, int k, const unsigned long long* list, const int32_t* lcount,
                            const int32_t* qlist, int64_t* out_ids, double* out_dist, cudaStream_t s) {
    if (nrows <= 0 || k <= 0) return cudaSuccess;
    const int64_t total = (int64_t)nrows * k;
    knn_emit_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(nrows, k, list, lcount, qlist, out_ids, out_dist);
    return cudaGetLastError();
}

cudaError_t launch_ref_sqnorm(const float* x, int64_t n, int dim, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    ref_sqnorm_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(x, n, dim, out);
    return cudaGetLastError();
}

cudaError_t launch_knn_col_terms(const float* sqnorm, const float* resid, int64_t n, int cosine, float2* terms,
                                 unsigned int* maxes, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    knn_col_terms_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(sqnorm, resid, n, cosine, terms, maxes);
    return cudaGetLastError();
}

namespace {
__global__ void fill_f32_kernel(float* __restrict__ p, int64_t n, float v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void fill_i32_kernel(int32_t* __restrict__ p, int64_t n, int32_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void sq_terms_kernel(const float* __restrict__ sqnorm, int64_t n, float2* __restrict__ terms) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) terms[i] = make_float2(sqnorm[i], -2.0f);
}
}  // namespace

cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    fill_f32_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_fill_i32(int32_t* p, int64_t n, int32_t v, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    fill_i32_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_sq_terms(const float* sqnorm, int64_t n, float2* terms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    sq_terms_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(sqnorm, n, terms);
    return cudaGetLastError();
}

cudaError_t launch_knn_query_band(const float* qsq, const float* qres, int64_t nq, int kp, int cosine,
                                  const unsigned int* maxes, float* e2, float* asl, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    knn_query_band_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(qsq, qres, nq, kp, cosine, maxes, e2, asl);
    return cudaGetLastError();
}

}  // namespace hann
