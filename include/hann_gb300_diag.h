/*
 * hann_gb300_diag.h -- diagnostic entry points of libhann_gb300.so. They have
 * no counterpart in the reference; tests use them to check single kernels
 * against a host computation. Host buffers; 0 or a negative HANN_E_* status.
 */
#ifndef HANN_GB300_DIAG_H
#define HANN_GB300_DIAG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The BF16 tensor-core distance GEMM (tcgen05, TMA-fed): for rows a [n][dim]
 * and columns b [m][dim] (dim <= 128), scores s[i][j] = ||b_j||^2 - 2 <a_i, b_j>
 * with a and b rounded to BF16, FP32 accumulation and ||b_j||^2 from the FP32
 * rows; and per row the 8 smallest scores with their columns, ascending.
 * `scores` may be NULL. */
int hann_gpu_bf16_scores(const float* a, int64_t n, const float* b, int32_t m, int32_t dim, float* scores,
                         int32_t* top_idx, float* top_val);

/* The subquantizer assignment of training's k-means: for host residuals
 * res [n][M * dsub] and codebooks [M][pqK][dsub] (pqK <= 256), out [n][M] the
 * codeword nearest each row's sub-vector m, squared Euclidean distance in the
 * reference's summation order, ties to the lower index. With sums and counts
 * (both or neither), also the k-means update's FP64 sums of the rows of
 * every codeword, sums [M][pqK][dsub], and their counts [M][pqK], computed by
 * the kernels training runs (the fused assignment + accumulation for dsub 4,
 * 8 and 16). */
int hann_gpu_pq_assign(const float* res, int64_t n, int32_t M, int32_t dsub, const float* codebooks, int32_t pqK,
                       int32_t* out, double* sums, int64_t* counts);

/* The index's row arena: out[0] rows allocated, out[1] rows up to the end
 * of the last list (the rest is free slack), out[2] rows left as holes by
 * lists that moved, out[3] list moves and out[4] full relayouts since the
 * handle was made. h is a hann_pqivf*. */
int hann_pqivf_arena_stats(void* h, int64_t* out5);

/* Rows the list-major scan decoded (each list's rows once per work item),
 * counted while profiling was on, as of the last hann_pqivf_stage_times
 * (whose rows_scanned counts the scored (query, row) pairs). */
int hann_pqivf_rows_decoded(void* h, int64_t* out);

/* The list scan's choices. set8 (may be NULL) replaces them, get8 (may be
 * NULL) receives them: [0] list-major tensor-core scan on (1) or the table
 * scan for every batch (0); [1] smallest batch that takes the list-major
 * scan; [2] probe ranks in its first chunk; [3] growth of the later chunks'
 * ends; [4] rows of a list per work item; [5] blocks per SM (1 or 2); [6]
 * first thresholds from a table scan of each query's nearest list (1) or a
 * first chunk that keeps every score (0); [7] fewest probed lists of a
 * query that takes the list-major scan (the others take the table scan).
 * In mode 0 results do not depend on them. */
int hann_pqivf_scan_options(void* h, const int32_t* set8, int32_t* get8);

/* Coarse k-means assignments over the handle's life that took the warm
 * filter (every row's nearest centroid bounded from its previous one, the
 * filter GEMM keeping the centroids under the bound, an exact rescore among
 * them) instead of the top-8 screen: out2[0] the assignments, out2[1] the
 * rows they sent to the exact kernel. */
int hann_pqivf_train_stats(void* h, int64_t* out2);

/* Wall milliseconds of the last Train or Retrain, by phase, each ending at a
 * stream synchronisation: out4[0] gathering the vectors in id order onto the
 * device, [1] the coarse k-means with the final assignment and its copy to
 * the host, [2] the subquantizer k-means, [3] the inverted lists, the device
 * layout, the encoding and the host copies of the quantizers. */
int hann_pqivf_train_phases(void* h, double* out4);

/* Queries, over the handle's life, whose parity-mode top k the FP16
 * lookup-table screen could not prove and that were scanned again with FP32
 * tables (waits for the handle's searches). */
int hann_pqivf_adc_redos(void* h, int64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* HANN_GB300_DIAG_H */
