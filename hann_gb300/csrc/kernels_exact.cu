// kernels_exact.cu -- the distance layer beneath the index: exact FP32
// distances in the reference's NEON summation order (core/simd_kernels.inc.h),
// batch form of simd_<metric>_batch (core/simd_kernels.inc.h:235-264).
#include "common.cuh"
#include "kernels.h"

namespace hann {

__global__ void distance_rows_kernel(int metric, const float* __restrict__ q, const float* __restrict__ flat, int dim,
                                     int64_t n, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* x = flat + i * dim;
    float r;
    switch (metric) {
    case 0: r = sqeuclid_ref(q, x, dim); break;
    case 1: r = __fsqrt_rn(sqeuclid_ref(q, x, dim)); break;
    case 2: r = manhattan_ref(q, x, dim); break;
    default: r = cosine_from_parts(dot_ref(q, x, dim), dot_ref(q, q, dim), dot_ref(x, x, dim)); break;
    }
    out[i] = (double)r;
}

cudaError_t launch_distance_rows(int metric, const float* q, const float* flat, int dim, int64_t n, double* out,
                                 cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    distance_rows_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(metric, q, flat, dim, n, out);
    return cudaGetLastError();
}

// Gathered distances for graph and tree indexes: for query q and each j in
// [offsets[q], offsets[q + 1]), out[j] = distance(queries[q], base[ids[j]]),
// one thread per pair (each distance is one thread's reference-order sum);
// the thread finds its query by binary search over offsets. An id outside
// [0, n) sets *bad and writes NaN.
__global__ void distance_gather_kernel(int metric, const float* __restrict__ queries, int64_t nq,
                                       const int64_t* __restrict__ offsets, const int32_t* __restrict__ ids,
                                       const float* __restrict__ base, int64_t n, int dim, double* __restrict__ out,
                                       int* __restrict__ bad) {
    const int64_t total = offsets[nq];
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= total) return;
    int64_t lo = 0, hi = nq - 1;  // the last query whose range starts at or before j
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= j) lo = mid;
        else hi = mid - 1;
    }
    const int32_t id = ids[j];
    if (id < 0 || (int64_t)id >= n) {
        out[j] = __longlong_as_double(0x7ff8000000000000ll);
        atomicExch(bad, 1);
        return;
    }
    const float* q = queries + lo * dim;
    const float* x = base + (int64_t)id * dim;
    float r;
    switch (metric) {
    case 0: r = sqeuclid_ref(q, x, dim); break;
    case 1: r = __fsqrt_rn(sqeuclid_ref(q, x, dim)); break;
    case 2: r = manhattan_ref(q, x, dim); break;
    default: r = cosine_from_parts(dot_ref(q, x, dim), dot_ref(q, q, dim), dot_ref(x, x, dim)); break;
    }
    out[j] = (double)r;
}

cudaError_t launch_distance_gather(int metric, const float* queries, int64_t nq, const int64_t* offsets,
                                   const int32_t* ids, int64_t total, const float* base, int64_t n, int dim,
                                   double* out, int* bad, cudaStream_t s) {
    if (nq <= 0 || total <= 0) return cudaSuccess;
    distance_gather_kernel<<<(unsigned)ceil_div(total, 128), 128, 0, s>>>(metric, queries, nq, offsets, ids, base, n,
                                                                        dim, out, bad);
    return cudaGetLastError();
}

}  // namespace hann
