// knn.cu -- the batched exact k-NN handle and its C ABI (include/hann_gb300.h).
//
// A hann_knn holds one flat base in device memory and answers batches of
// queries with the k nearest rows under squared Euclidean, Euclidean,
// Manhattan or cosine distance, ordered by (distance, row) -- the order of
// testutil.BruteForceKNN (internal/testutil/data.go:66-93) -- with each
// distance the reference's FP32 value (core/simd_kernels.inc.h:235-264).
//
// Queries run in blocks of at most KNN_QB rows. The base is walked in chunks
// that grow geometrically: the first chunk (at most CAP rows) fills every
// query's candidate buffer, later chunks only pass rows that can still enter
// the query's top k, so per query only about k * growth candidates move per
// chunk. Exact path and tensor-core screen: kernels_knn.cu.
#include <cuda_bf16.h>

#include "index_internal.h"

namespace hann {
namespace {

constexpr int KNN_QB = 8192;       // queries per block of work
constexpr int KNN_CAP = 8192;      // candidate buffer per query and chunk
constexpr int KNN_KMAX = 4096;     // largest k
constexpr int64_t KNN_GROW = 4;    // chunk growth factor (3-4 measured best on 1M x 128, k 100: 5.50 ms against 5.64 at 8, 5.87 at 16)

__global__ void knn_init_rows_kernel(const int32_t* __restrict__ qlist, int nsel, int32_t* __restrict__ lcount,
                                     unsigned long long* __restrict__ thr, int32_t* __restrict__ cnt) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsel) return;
    const int r = qlist ? qlist[p] : p;
    lcount[r] = 0;
    thr[r] = ~0ull;
    cnt[r] = 0;
}

__global__ void knn_fill_f32_kernel(float* __restrict__ p, int n, float v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void knn_fill_kernel(int64_t nq, int k, int64_t n, int64_t* __restrict__ ids, double* __restrict__ dist) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nq * k) return;
    const int i = (int)(e % k);
    ids[e] = i < n ? i : -1;
    dist[e] = i < n ? 0.0 : (double)__int_as_float(0x7f800000);
}

}  // namespace
}  // namespace hann

using namespace hann;

// Message of the calling thread's last failed hann_knn_* call.
static thread_local std::string t_knn_error;

struct hann_knn {
    int64_t n = 0;
    int dim = 0, kp = 0;
    DBuf<float> base;                 // [n][dim]
    DBuf<float> bnorm;                // dot_ref(b, b), cosine only
    DBuf<__nv_bfloat16> base_bf;      // [n][kp]
    DBuf<float> bsq, bres;            // FP32 squared norm and BF16 residual norm per row
    DBuf<float2> cterm[2];            // screen terms: [0] squared Euclidean, [1] cosine
    DBuf<unsigned int> maxes[2];
    bool have_bf = false, have_bnorm = false, have_terms[2] = {false, false};

    // per query block
    DBuf<__nv_bfloat16> q_bf;
    DBuf<float> qsq, qres, qnorm, e2, asl, thr_f, cand_v;
    DBuf<int32_t> cnt, cand_id, lcount, need_exact, exact_list, redo, qlist2, todo;
    DBuf<unsigned long long> list, thr_k;
    DBuf<int> counters;               // [0] exact_count, [1] GEMM error, [2..] redo counts per chunk
    DBuf<float> q_in;
    DBuf<int64_t> ids_out;
    DBuf<double> dist_out;
    DBuf<int> gather_bad;             // set by the gathered-distance kernel for an id outside the base

    cudaStream_t stream = nullptr;
    std::mutex mu;
    hann_knn_stats stats{};

    int fail(int code, const char* msg) {
        t_knn_error = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        t_knn_error = std::string(what) + ": " + cudaGetErrorString(e);
        return HANN_E_CUDA;
    }
};

namespace {

// Chunk boundaries of the base walk: a first chunk of `first` rows (at most
// CAP: every row of it enters the candidate buffer), then chunks that make
// the walked prefix grow KNN_GROW-fold, so about k * (KNN_GROW - 1) rows per
// query pass each later chunk.
std::vector<int64_t> chunk_bounds(int64_t n, int k) {
    std::vector<int64_t> b{0};
    int64_t c = std::min<int64_t>(n, std::min<int64_t>(KNN_CAP, std::max<int64_t>(1024, round_up(8 * (int64_t)k, 256))));
    while (b.back() < n) {
        b.push_back(std::min<int64_t>(n, b.back() + c));
        c = b.back() * (KNN_GROW - 1);
    }
    return b;
}

int prepare_bnorm(hann_knn* h, cudaStream_t s) {
    if (h->have_bnorm) return HANN_OK;
    CK(h->bnorm.reserve(h->n));
    CK(launch_ref_sqnorm(h->base.p, h->n, h->dim, h->bnorm.p, s));
    h->have_bnorm = true;
    return HANN_OK;
}

int prepare_screen(hann_knn* h, int cos, cudaStream_t s) {
    if (!h->have_bf) {
        CK(h->base_bf.reserve((size_t)h->n * h->kp));
        CK(h->bsq.reserve(h->n));
        CK(h->bres.reserve(h->n));
        CK(launch_to_bf16(h->base.p, h->n, h->dim, h->kp, h->base_bf.p, h->bsq.p, h->bres.p, s));
        h->have_bf = true;
    }
    if (!h->have_terms[cos]) {
        CK(h->cterm[cos].reserve(h->n));
        CK(h->maxes[cos].reserve(2));
        CK(cudaMemsetAsync(h->maxes[cos].p, 0, 2 * sizeof(unsigned int), s));
        CK(launch_knn_col_terms(h->bsq.p, h->bres.p, h->n, cos, h->cterm[cos].p, h->maxes[cos].p, s));
        h->have_terms[cos] = true;
    }
    return HANN_OK;
}

int reserve_block(hann_knn* h, int64_t qb, int k, int nchunks) {
    const int lcap = std::max(4096, 2 * k);
    CK(h->cnt.reserve(qb));
    CK(h->cand_id.reserve((size_t)qb * KNN_CAP));
    CK(h->cand_v.reserve((size_t)qb * KNN_CAP));
    CK(h->lcount.reserve(qb));
    CK(h->thr_k.reserve(qb));
    CK(h->thr_f.reserve(qb));
    CK(h->need_exact.reserve(qb));
    CK(h->todo.reserve(qb + 1));
    CK(h->exact_list.reserve(qb));
    CK(h->qlist2.reserve(qb));
    CK(h->redo.reserve((size_t)qb * nchunks));
    CK(h->counters.reserve(2 + nchunks));
    CK(h->list.reserve((size_t)qb * std::max(lcap, k)));
    CK(h->qnorm.reserve(qb));
    CK(h->qsq.reserve(qb));
    CK(h->qres.reserve(qb));
    CK(h->e2.reserve(qb));
    CK(h->asl.reserve(qb));
    CK(h->q_bf.reserve((size_t)qb * h->kp));
    return HANN_OK;
}

// Exact SIMT k-NN for rows qlist[0..nsel) of a query block (all nrows when
// qlist is null). Outputs go to rows of ids/dist (row-major, k per row).
int knn_exact(hann_knn* h, int metric, const float* q, int nrows, const int32_t* qlist, int nsel, int k,
              int64_t* ids, double* dist, cudaStream_t s) {
    if (nsel <= 0) return HANN_OK;
    const std::vector<int64_t> cb = chunk_bounds(h->n, k);
    const int nch = (int)cb.size() - 1;
    if (metric == HANN_METRIC_COSINE) {
        int rc = prepare_bnorm(h, s);
        if (rc != HANN_OK) return rc;
        CK(launch_ref_sqnorm(q, nrows, h->dim, h->qnorm.p, s));
    }
    unsigned long long* list = h->list.p;
    knn_init_rows_kernel<<<(unsigned)ceil_div(nsel, 256), 256, 0, s>>>(qlist, nsel, h->lcount.p, h->thr_k.p,
                                                                      h->cnt.p);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(h->redo.p, 0, sizeof(int32_t) * (size_t)nrows * nch, s));
    CK(cudaMemsetAsync(h->counters.p + 2, 0, sizeof(int) * nch, s));
    for (int c = 0; c < nch; c++) {
        CK(launch_knn_filter(metric, q, qlist, nsel, h->dim, h->base.p, cb[c], cb[c + 1], h->qnorm.p, h->bnorm.p,
                             h->thr_k.p, KNN_CAP, h->cnt.p, h->cand_id.p, h->cand_v.p, s));
        CK(launch_knn_merge_exact(nsel, qlist, k, KNN_CAP, h->cnt.p, h->cand_id.p, h->cand_v.p, list, h->lcount.p,
                                  h->thr_k.p, h->redo.p + (size_t)c * nrows, h->counters.p + 2 + c, s));
    }
    h->stats.chunks += nch;
    // Chunks whose candidates overflowed a query's buffer run again for those
    // queries in pieces of at most CAP rows, which cannot overflow.
    std::vector<int> redo_counts(nch);
    CK(cudaMemcpyAsync(redo_counts.data(), h->counters.p + 2, sizeof(int) * nch, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<int32_t> flags;
    std::vector<int32_t> rows;
    for (int c = 0; c < nch; c++) {
        if (redo_counts[c] == 0) continue;
        flags.resize(nrows);
        CK(cudaMemcpy(flags.data(), h->redo.p + (size_t)c * nrows, sizeof(int32_t) * nrows, cudaMemcpyDeviceToHost));
        rows.clear();
        for (int r = 0; r < nrows; r++)
            if (flags[r]) rows.push_back(r);
        CK(cudaMemcpyAsync(h->qlist2.p, rows.data(), sizeof(int32_t) * rows.size(), cudaMemcpyHostToDevice, s));
        for (int64_t c0 = cb[c]; c0 < cb[c + 1]; c0 += KNN_CAP) {
            const int64_t c1 = std::min<int64_t>(cb[c + 1], c0 + KNN_CAP);
            CK(launch_knn_filter(metric, q, h->qlist2.p, (int)rows.size(), h->dim, h->base.p, c0, c1, h->qnorm.p,
                                 h->bnorm.p, h->thr_k.p, KNN_CAP, h->cnt.p, h->cand_id.p, h->cand_v.p, s));
            CK(launch_knn_merge_exact((int)rows.size(), h->qlist2.p, k, KNN_CAP, h->cnt.p, h->cand_id.p,
                                      h->cand_v.p, list, h->lcount.p, h->thr_k.p, h->redo.p + (size_t)c * nrows,
                                      h->counters.p + 2 + c, s));
        }
        h->stats.redo_chunks++;
        CK(cudaStreamSynchronize(s));
    }
    CK(launch_knn_emit(nsel, k, list, h->lcount.p, qlist, ids, dist, s));
    return HANN_OK;
}

// Tensor-core screen for a whole query block; queries whose band overflowed
// finish on the exact path.
int knn_screen(hann_knn* h, int metric, const float* q, int nrows, int k, int64_t* ids, double* dist,
               cudaStream_t s) {
    const int cos = metric == HANN_METRIC_COSINE ? 1 : 0;
    int rc = prepare_screen(h, cos, s);
    if (rc != HANN_OK) return rc;
    if (cos) {
        rc = prepare_bnorm(h, s);
        if (rc != HANN_OK) return rc;
        CK(launch_ref_sqnorm(q, nrows, h->dim, h->qnorm.p, s));
    }
    const int lcap = std::max(4096, 2 * k);
    CK(launch_to_bf16(q, nrows, h->dim, h->kp, h->q_bf.p, h->qsq.p, h->qres.p, s));
    CK(launch_knn_query_band(h->qsq.p, h->qres.p, nrows, h->kp, cos, h->maxes[cos].p, h->e2.p, h->asl.p, s));
    CK(cudaMemsetAsync(h->lcount.p, 0, sizeof(int32_t) * nrows, s));
    CK(cudaMemsetAsync(h->cnt.p, 0, sizeof(int32_t) * nrows, s));
    CK(cudaMemsetAsync(h->need_exact.p, 0, sizeof(int32_t) * nrows, s));
    CK(cudaMemsetAsync(h->counters.p, 0, 2 * sizeof(int), s));
    knn_fill_f32_kernel<<<(unsigned)ceil_div(nrows, 256), 256, 0, s>>>(h->thr_f.p, nrows, INFINITY);
    CK(cudaGetLastError());
    const std::vector<int64_t> cb = chunk_bounds(h->n, k);
    const int nch = (int)cb.size() - 1;
    for (int c = 0; c < nch; c++) {
        CK(launch_gemm_filter(h->q_bf.p, nrows, h->base_bf.p, h->n, h->kp, (int)cb[c], (int)cb[c + 1],
                              h->cterm[cos].p, cos, h->thr_f.p, KNN_CAP, h->cnt.p, h->cand_id.p, h->cand_v.p,
                              h->counters.p + 1, s, c == 0));
        CK(launch_knn_merge_band(nrows, k, nullptr, KNN_CAP, lcap, h->cnt.p, h->cand_id.p, h->cand_v.p, h->e2.p, h->asl.p,
                                 h->list.p, h->lcount.p, h->thr_f.p, h->need_exact.p, h->todo.p, s));
    }
    h->stats.chunks += nch;
    CK(launch_knn_final_band(metric, nrows, k, lcap, h->dim, q, h->base.p, h->qnorm.p, h->bnorm.p, h->list.p,
                             h->lcount.p, h->need_exact.p, h->exact_list.p, h->counters.p, ids, dist, s));
    int hc[2];
    CK(cudaMemcpyAsync(hc, h->counters.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hc[1] != 0) return h->fail(HANN_E_CUDA, "tensor-core screen: a pipeline wait timed out");
    h->stats.tensor_queries += nrows - hc[0];
    if (hc[0] > 0) {
        h->stats.fallback_queries += hc[0];
        // the exact path reuses the list and candidate buffers
        rc = knn_exact(h, metric, q, nrows, h->exact_list.p, hc[0], k, ids, dist, s);
        if (rc != HANN_OK) return rc;
    }
    return HANN_OK;
}

int knn_run(hann_knn* h, int metric, const float* q, int64_t nq, int k, int method, int64_t* ids, double* dist,
            cudaStream_t s) {
    if (metric < 0 || metric > 3) return h->fail(HANN_E_INVALID, "unknown metric");
    if (k <= 0 || k > KNN_KMAX) return h->fail(HANN_E_INVALID, "k must be in [1, 4096]");
    if (nq < 0) return h->fail(HANN_E_INVALID, "negative query count");
    if (method < HANN_KNN_AUTO || method > HANN_KNN_TENSOR) return h->fail(HANN_E_INVALID, "unknown method");
    const bool screen_ok = metric != HANN_METRIC_MANHATTAN && h->dim <= KNN_TC_DMAX && h->dim > 0;
    if (method == HANN_KNN_TENSOR && !screen_ok)
        return h->fail(HANN_E_UNSUPPORTED, "the tensor-core screen covers squared Euclidean, Euclidean and cosine "
                                           "distance up to 128 dimensions");
    const bool screen = method == HANN_KNN_TENSOR || (method == HANN_KNN_AUTO && screen_ok);
    if (nq == 0) return HANN_OK;
    if (h->n == 0 || h->dim == 0) {
        // empty base: nothing found; empty vectors: every distance is 0
        const int64_t nn = h->dim == 0 ? h->n : 0;
        knn_fill_kernel<<<(unsigned)ceil_div(nq * k, 256), 256, 0, s>>>(nq, k, nn, ids, dist);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
        return HANN_OK;
    }
    const int nch = (int)chunk_bounds(h->n, k).size() - 1;
    for (int64_t q0 = 0; q0 < nq; q0 += KNN_QB) {
        const int nr = (int)std::min<int64_t>(KNN_QB, nq - q0);
        int rc = reserve_block(h, nr, k, nch);
        if (rc != HANN_OK) return rc;
        const float* qb = q + q0 * h->dim;
        if (screen) rc = knn_screen(h, metric, qb, nr, k, ids + q0 * k, dist + q0 * k, s);
        else {
            h->stats.exact_queries += nr;
            rc = knn_exact(h, metric, qb, nr, nullptr, nr, k, ids + q0 * k, dist + q0 * k, s);
        }
        if (rc != HANN_OK) return rc;
        h->stats.queries += nr;
    }
    CK(cudaStreamSynchronize(s));
    return HANN_OK;
}

}  // namespace

extern "C" {

hann_knn* hann_knn_new(const float* base, int64_t n, int32_t dim) {
    if (n < 0 || dim < 0 || (n > 0 && dim > 0 && !base)) return nullptr;
    if (n >= ((int64_t)1 << 31)) return nullptr;
    hann_knn* h = new (std::nothrow) hann_knn();
    if (!h) return nullptr;
    h->n = n;
    h->dim = dim;
    h->kp = gemm_kpad(dim > 0 ? dim : 1);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        h->base.reserve((size_t)n * dim) != cudaSuccess ||
        (n * dim > 0 && cudaMemcpy(h->base.p, base, sizeof(float) * n * dim, cudaMemcpyHostToDevice) != cudaSuccess)) {
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
        return nullptr;
    }
    return h;
}

}  // extern "C"

// A k-NN handle over a base already in device memory (copied, device to
// device, on stream s): the recall tuner's ground truth over an index's
// stored vectors.
hann_knn* knn_new_from_device(const float* d_base, int64_t n, int32_t dim, cudaStream_t s) {
    if (n < 0 || dim < 0 || n >= ((int64_t)1 << 31)) return nullptr;
    hann_knn* h = new (std::nothrow) hann_knn();
    if (!h) return nullptr;
    h->n = n;
    h->dim = dim;
    h->kp = gemm_kpad(dim > 0 ? dim : 1);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        h->base.reserve((size_t)n * dim) != cudaSuccess ||
        (n * dim > 0 && (cudaMemcpyAsync(h->base.p, d_base, sizeof(float) * n * dim, cudaMemcpyDeviceToDevice, s) !=
                             cudaSuccess ||
                         cudaStreamSynchronize(s) != cudaSuccess))) {
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
        return nullptr;
    }
    return h;
}

extern "C" {

void hann_knn_free(hann_knn* h) {
    if (!h) return;
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
    delete h;
}

const char* hann_knn_last_error(const hann_knn*) { return t_knn_error.c_str(); }

int hann_knn_search(hann_knn* h, int32_t metric, const float* queries, int64_t nq, int32_t k, int32_t method,
                    int64_t* ids, double* dist) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    if (nq > 0 && ((!queries && h->dim > 0) || !ids || !dist)) return h->fail(HANN_E_INVALID, "null buffer");
    if (nq <= 0 || k <= 0) return knn_run(h, metric, nullptr, nq < 0 ? nq : 0, k, method, nullptr, nullptr,
                                          h->stream);
    cudaStream_t s = h->stream;
    CK(upload(h->q_in, queries, (size_t)nq * h->dim, s));
    CK(h->ids_out.reserve((size_t)nq * k));
    CK(h->dist_out.reserve((size_t)nq * k));
    int rc = knn_run(h, metric, h->q_in.p, nq, k, method, h->ids_out.p, h->dist_out.p, s);
    if (rc != HANN_OK) return rc;
    CK(cudaMemcpyAsync(ids, h->ids_out.p, sizeof(int64_t) * nq * k, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(dist, h->dist_out.p, sizeof(double) * nq * k, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return HANN_OK;
}

int hann_knn_search_device(hann_knn* h, int32_t metric, const float* queries, int64_t nq, int32_t k, int32_t method,
                           int64_t* ids, double* dist, void* stream) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    if (nq > 0 && ((!queries && h->dim > 0) || !ids || !dist)) return h->fail(HANN_E_INVALID, "null buffer");
    return knn_run(h, metric, queries, nq, k, method, ids, dist, stream ? (cudaStream_t)stream : h->stream);
}

int hann_knn_append(hann_knn* h, const float* rows, int64_t n) {
    if (!h || n < 0 || (n > 0 && h->dim > 0 && !rows)) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    if (h->n + n >= ((int64_t)1 << 31)) return h->fail(HANN_E_UNSUPPORTED, "more than 2^31 base rows");
    if (n == 0) return HANN_OK;
    const size_t need = (size_t)(h->n + n) * h->dim;
    if (need > h->base.n) {
        // grow by half again, keeping the rows (device to device)
        DBuf<float> nb;
        if (nb.reserve(std::max(need, h->base.n + h->base.n / 2)) != cudaSuccess)
            return h->fail(HANN_E_NOMEM, "device allocation failed");
        if (h->n * h->dim > 0 &&
            cudaMemcpyAsync(nb.p, h->base.p, sizeof(float) * h->n * h->dim, cudaMemcpyDeviceToDevice, h->stream) !=
                cudaSuccess)
            return h->fail(HANN_E_CUDA, "copy failed");
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return h->fail(HANN_E_CUDA, "copy failed");
        h->base.swap(nb);
    }
    if (h->dim > 0 && cudaMemcpyAsync(h->base.p + (size_t)h->n * h->dim, rows, sizeof(float) * n * h->dim,
                                      cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
        return h->fail(HANN_E_CUDA, "copy failed");
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return h->fail(HANN_E_CUDA, "copy failed");
    h->n += n;
    // the screen's copies of the base are rebuilt on the next search
    h->have_bf = h->have_bnorm = false;
    h->have_terms[0] = h->have_terms[1] = false;
    return HANN_OK;
}

static int gather_run(hann_knn* h, int32_t metric, const float* d_q, int64_t nq, const int64_t* d_off,
                      const int32_t* d_ids, int64_t total, double* d_out, cudaStream_t s) {
    if (h->gather_bad.reserve(1) != cudaSuccess) return h->fail(HANN_E_NOMEM, "device allocation failed");
    if (cudaMemsetAsync(h->gather_bad.p, 0, sizeof(int), s) != cudaSuccess ||
        launch_distance_gather(metric, d_q, nq, d_off, d_ids, total, h->base.p, h->n, h->dim, d_out,
                               h->gather_bad.p, s) != cudaSuccess)
        return h->fail(HANN_E_CUDA, "gathered distances failed");
    int bad = 0;
    if (cudaMemcpyAsync(&bad, h->gather_bad.p, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return h->fail(HANN_E_CUDA, "gathered distances failed");
    if (bad) return h->fail(HANN_E_INVALID, "candidate id outside the base");
    return HANN_OK;
}

int hann_knn_distance_gather(hann_knn* h, int32_t metric, const float* queries, int64_t nq, const int64_t* offsets,
                             const int32_t* ids, double* out) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    if (metric < 0 || metric > 3) return h->fail(HANN_E_INVALID, "unknown metric");
    if (nq < 0 || (nq > 0 && !offsets)) return h->fail(HANN_E_INVALID, "null buffer");
    if (nq == 0) return HANN_OK;
    if (offsets[0] != 0) return h->fail(HANN_E_INVALID, "offsets must start at 0");
    for (int64_t q = 0; q < nq; q++)
        if (offsets[q + 1] < offsets[q]) return h->fail(HANN_E_INVALID, "offsets must not decrease");
    const int64_t total = offsets[nq];
    if (total == 0) return HANN_OK;
    if ((h->dim > 0 && !queries) || !ids || !out) return h->fail(HANN_E_INVALID, "null buffer");
    DBuf<float> dq;
    DBuf<int64_t> doff;
    DBuf<int32_t> dids;
    DBuf<double> dout;
    if (upload(dq, queries, (size_t)nq * h->dim, h->stream) != cudaSuccess ||
        upload(doff, offsets, (size_t)nq + 1, h->stream) != cudaSuccess ||
        upload(dids, ids, (size_t)total, h->stream) != cudaSuccess || dout.reserve((size_t)total) != cudaSuccess)
        return h->fail(HANN_E_CUDA, "device allocation or copy failed");
    const int rc = gather_run(h, metric, dq.p, nq, doff.p, dids.p, total, dout.p, h->stream);
    if (rc) return rc;
    if (cudaMemcpyAsync(out, dout.p, sizeof(double) * total, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return h->fail(HANN_E_CUDA, "copy failed");
    return HANN_OK;
}

int hann_knn_distance_gather_device(hann_knn* h, int32_t metric, const float* d_queries, int64_t nq,
                                    const int64_t* d_offsets, const int32_t* d_ids, int64_t total, double* d_out,
                                    void* stream) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    if (metric < 0 || metric > 3) return h->fail(HANN_E_INVALID, "unknown metric");
    if (nq < 0 || total < 0) return h->fail(HANN_E_INVALID, "negative size");
    if (nq == 0 || total == 0) return HANN_OK;
    if ((h->dim > 0 && !d_queries) || !d_offsets || !d_ids || !d_out) return h->fail(HANN_E_INVALID, "null buffer");
    return gather_run(h, metric, d_queries, nq, d_offsets, d_ids, total, d_out,
                      stream ? (cudaStream_t)stream : h->stream);
}

int hann_knn_get_stats(hann_knn* h, hann_knn_stats* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::lock_guard<std::mutex> g(h->mu);
    *out = h->stats;
    return HANN_OK;
}

int hann_gpu_knn(int32_t metric, const float* queries, int64_t nq, const float* base, int64_t n, int32_t dim,
                 int32_t k, int32_t method, int64_t* ids, double* dist) {
    hann_knn* h = hann_knn_new(base, n, dim);
    if (!h) return HANN_E_CUDA;
    const int rc = hann_knn_search(h, metric, queries, nq, k, method, ids, dist);
    hann_knn_free(h);
    return rc;
}

int hann_gpu_distance_matrix(int32_t metric, const float* queries, int64_t nq, const float* base, int64_t n,
                             int32_t dim, double* out) {
    if (metric < 0 || metric > 3 || nq < 0 || n < 0 || dim < 0) return HANN_E_INVALID;
    if (nq == 0 || n == 0) return HANN_OK;
    if (!queries || !base || !out) return HANN_E_INVALID;
    if (dim == 0) {
        for (int64_t i = 0; i < nq * n; i++) out[i] = 0.0;
        return HANN_OK;
    }
    DBuf<float> dq, dx, qn, bn;
    DBuf<double> dout;
    if (upload(dq, queries, (size_t)nq * dim, nullptr) != cudaSuccess ||
        upload(dx, base, (size_t)n * dim, nullptr) != cudaSuccess || qn.reserve(nq) != cudaSuccess ||
        bn.reserve(n) != cudaSuccess)
        return HANN_E_CUDA;
    if (metric == HANN_METRIC_COSINE &&
        (launch_ref_sqnorm(dq.p, nq, dim, qn.p, nullptr) != cudaSuccess ||
         launch_ref_sqnorm(dx.p, n, dim, bn.p, nullptr) != cudaSuccess))
        return HANN_E_CUDA;
    // rows of queries in slabs that keep the FP64 output under 1 GiB
    const int64_t slab = std::max<int64_t>(1, ((int64_t)1 << 27) / n);
    if (dout.reserve((size_t)std::min(slab, nq) * n) != cudaSuccess) return HANN_E_CUDA;
    for (int64_t q0 = 0; q0 < nq; q0 += slab) {
        const int64_t nr = std::min(slab, nq - q0);
        if (launch_knn_matrix(metric, dq.p + q0 * dim, (int)nr, dim, dx.p, 0, n, qn.p + q0, bn.p, dout.p, n,
                              nullptr) != cudaSuccess)
            return HANN_E_CUDA;
        if (cudaMemcpy(out + q0 * n, dout.p, sizeof(double) * nr * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            return HANN_E_CUDA;
    }
    return HANN_OK;
}

}  // extern "C"
