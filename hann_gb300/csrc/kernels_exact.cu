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

}  // namespace hann
