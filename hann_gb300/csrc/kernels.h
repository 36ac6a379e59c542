// kernels.h -- host-side launchers of the hann_gb300 CUDA kernels.
// Every launcher enqueues on the given stream and returns the launch status.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hann {

// ---- exact (reference-order) coarse distances --------------------------------

// For every point, the index of the nearest centroid under the reference-order
// FP32 squared Euclidean distance, the lowest index winning a tie
// (assignPoints, pqivf/index.go:738-789). out_dist may be null. key_scratch
// (n entries, may be null) lets small batches split the centroids over more
// blocks.
cudaError_t launch_assign_exact(const float* x, int64_t n, int dim, const float* cent, int k,
                                int32_t* out_idx, float* out_dist, unsigned long long* key_scratch,
                                cudaStream_t s);

// Full matrix D[q][c] of reference-order squared Euclidean distances.
cudaError_t launch_dist_matrix(const float* q, int64_t nq, int dim, const float* cent, int k,
                               float* out, cudaStream_t s);

// ---- k-means update (FP64 sums) ---------------------------------------------

cudaError_t launch_kmeans_accumulate(const float* x, int64_t n, int dim, const int32_t* assign,
                                     double* sums, int64_t* counts, cudaStream_t s);
// centroid = sum / count for non-empty clusters; empty clusters keep their row.
cudaError_t launch_kmeans_finalize(const double* sums, const int64_t* counts, int k, int dim,
                                   float* cent, cudaStream_t s);

// ---- product quantizer --------------------------------------------------------

// For sub-vector m of every point (residual layout [n][dim], dim = M*dsub),
// the nearest codeword of codebook m ([M][pqK][dsub]) by reference-order
// distance, lowest code winning a tie (encodeWithCodebooks,
// pqivf/index.go:641-666). out: [n][M] int32 (m_begin..m_end only).
cudaError_t launch_pq_assign(const float* res, int64_t n, int M, int dsub, const float* codebooks, int pqK,
                             int m_begin, int m_end, int32_t* out, cudaStream_t s);

// FP64 sums of sub-vectors per (m, code): sums[M][pqK][dsub], counts[M][pqK].
cudaError_t launch_pq_accumulate(const float* res, int64_t n, int M, int dsub, const int32_t* codes,
                                 int pqK, int m_begin, int m_end, double* sums, int64_t* counts,
                                 cudaStream_t s);

// residual[i] = x[i] - coarse[cluster[i]] (FP32), rows in the given order:
// out row i comes from x row src[i] (src may be null for identity).
cudaError_t launch_residuals(const float* x, const int64_t* src, const int32_t* cluster, int64_t n, int dim,
                             const float* coarse, float* out, cudaStream_t s);

// Encode rows: codes (uint8, row stride code_stride bytes) and the per-row
// scalar term = ||r||^2 + 2<c, r> of the reconstructed residual r, used by
// the ADC scan. Item i works on row r = rows ? rows[i] : i of x, cluster,
// codes and term.
cudaError_t launch_encode(const float* x, const int64_t* rows, const int32_t* cluster, int64_t n, int dim,
                          const float* coarse, const float* codebooks, int M, int pqK, uint8_t* codes,
                          int code_stride, float* term, cudaStream_t s);

// The per-row term from existing codes (rows as in launch_encode).
cudaError_t launch_term(const uint8_t* codes, const int64_t* rows, const int32_t* cluster, int64_t n, int dim,
                        const float* coarse, const float* codebooks, int M, int pqK, int code_stride, float* term,
                        cudaStream_t s);

// out[dst ? dst[i] : i] = in[src ? src[i] : i] for rows of `width` 32-bit words.
cudaError_t launch_copy_words(const void* in, const int64_t* src, void* out, const int64_t* dst, int64_t n,
                              int width, cudaStream_t s);

// out[i] = src[i] >= 0 ? a[src[i]] : b[-src[i] - 1], rows of dim floats.
cudaError_t launch_gather2(const float* a, const float* b, const int64_t* src, int64_t n, int dim, float* out,
                           cudaStream_t s);

// out[(dst ? dst[i] : i) * ldo + j] = in[src[i] * ld + off + j], j < w.
cudaError_t launch_gather_cols(const float* in, int64_t ld, int off, const int64_t* src, const int32_t* dst,
                               int64_t n, int w, float* out, int64_t ldo, cudaStream_t s);

// Reference-order batch distances of one query to n rows (simd_*_batch).
cudaError_t launch_distance_rows(int metric, const float* q, const float* flat, int dim, int64_t n, double* out,
                                 cudaStream_t s);

// ---- search ---------------------------------------------------------------------

struct ScanParams {
    int dim, M, dsub, pqK, nlist, code_stride;
    const float* coarse;      // [nlist][dim]
    const float* codebooks;   // [M][pqK][dsub]
    const int64_t* list_start;  // [nlist] first row of each list
    const int32_t* list_len;    // [nlist]
    const uint8_t* codes;     // [rows][code_stride]
    const float* term;        // [rows]
    const int32_t* row_cluster;  // [rows]
    const float* vectors;     // [rows][dim]
    const int64_t* row_id;    // [rows]
};

// Per query: the nprobe nearest coarse lists in ascending (distance, index)
// order and their distances, from a distance matrix D[nq][nlist]. Also sets
// fallback[q] when the probed lists hold fewer than k[q] rows.
cudaError_t launch_probe_select(const float* D, int64_t nq, int nlist, const int32_t* nprobe, int np_max,
                                const int32_t* k, const int32_t* list_len, int allow_fallback,
                                int32_t* probe_ids, float* probe_d, int32_t* fallback,
                                unsigned long long* fallback_count, cudaStream_t s);

// ADC scan: per query, the R best rows by the decomposed PQ distance over the
// probed lists (all lists for a fallback query). D is the coarse distance
// matrix [nq][nlist]. Outputs rows (-1 padded), approximate distances and
// candidate sequence keys; adds the rows it scanned to *rows_scanned (may be
// null).
cudaError_t launch_scan(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                        const float* D, const int32_t* nprobe, int np_max, const int32_t* fallback,
                        int R, int32_t* cand_row, float* cand_d, uint32_t* cand_seq,
                        unsigned long long* rows_scanned, cudaStream_t s);

// Rerank the R candidates of each query with an exact FP32 distance and emit
// the k best: mode 0 = the reference's reconstructed-vector distance
// (decodePQCode + vectorAdd, pqivf/index.go:909-923), mode 1 = the raw
// vector. ids [nq][kmax] (-1 padded), dist [nq][kmax] = sqrt(rank) in FP64,
// nout [nq].
cudaError_t launch_rerank(const ScanParams& p, const float* queries, int64_t nq, const int32_t* cand_row,
                          const uint32_t* cand_seq, int R, const int32_t* k, int kmax, int mode,
                          int64_t* ids, double* dist, int32_t* nout, cudaStream_t s);

}  // namespace hann
