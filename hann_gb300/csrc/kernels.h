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
// Assignment and FP64 accumulation of one subquantizer's k-means iteration
// in one kernel (sub-dimensions 4, 8 and 16, pqK <= 256; otherwise
// cudaErrorNotSupported and nothing runs): out[p * M + m] the codeword of
// row p, sums_m [pqK][dsub] and counts_m [pqK] (zeroed by the caller)
// accumulated over the rows.
bool pq_assign_accumulate_supported(int dsub, int pqK);
cudaError_t launch_pq_assign_accumulate(const float* res, int64_t n, int M, int dsub, const float* codebooks,
                                        int pqK, int m, int32_t* out, double* sums_m, int64_t* counts_m,
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

// Marks rows deleted: term = +inf (never selected by a scan), row_id = -1.
cudaError_t launch_tombstone(const int64_t* rows, int64_t n, float* term, int64_t* row_id, cudaStream_t s);

// Reference-order batch distances of one query to n rows (simd_*_batch).
// out[j] = distance(queries[q], base[ids[j]]) for j in [offsets[q],
// offsets[q + 1]), total = offsets[nq] pairs; *bad is set for an id outside
// [0, n) (its distance is NaN).
cudaError_t launch_distance_gather(int metric, const float* queries, int64_t nq, const int64_t* offsets,
                                   const int32_t* ids, int64_t total, const float* base, int64_t n, int dim,
                                   double* out, int* bad, cudaStream_t s);
cudaError_t launch_distance_rows(int metric, const float* q, const float* flat, int dim, int64_t n, double* out,
                                 cudaStream_t s);

// ---- BF16 tensor-core distance GEMM (kernels_gemm.cu) ----------------------------

// K padded for the GEMM (multiple of 8 BF16 = 16 bytes); candidates per row of
// the argmin mode.
int gemm_kpad(int dim);
int gemm_topc();
// FP32 rows to BF16 [n][kp] (zero padded) and, when not null, the FP32
// squared norm of each row and the norm of its BF16 rounding error.
cudaError_t launch_to_bf16(const float* x, int64_t n, int dim, int kp, void* out_bf16, float* sqnorm, float* resid,
                           cudaStream_t s);
// S[i][j] = bias[j] - 2 <a_i, b_j> for every pair (a: nrows x kp, b: ncols x kp).
cudaError_t launch_gemm_scores(const void* a_bf16, int64_t nrows, const void* b_bf16, int ncols, int kp,
                               const float* bias, float* out, int* err, cudaStream_t s);
// Per row the gemm_topc() smallest scores and their columns, ascending.
cudaError_t launch_gemm_top8(const void* a_bf16, int64_t nrows, const void* b_bf16, int ncols, int kp,
                             const float* bias, int32_t* cand_idx, float* cand_val, int* err, cudaStream_t s);

// ---- exact answers from the BF16 scores (kernels_rescore.cu) --------------------

// Probe selection from BF16 scores S [nq][nlist] (rows may be overwritten):
// the nprobe nearest lists by exact reference-order distance, ascending
// (distance, index), with those distances; fallback flags as
// launch_probe_select. cmax points at max ||c||.
cudaError_t launch_probe_select_band(float* S, const float* Q, const float* qn2, const float* qres, int64_t nq,
                                     int dim, int kp, const float* coarse, const float* cmax, int nlist,
                                     const int32_t* nprobe,
                                     int np_max, const int32_t* k, const int32_t* list_len, int allow_fallback,
                                     int32_t* probe_ids, float* probe_d, int32_t* fallback,
                                     unsigned long long* fallback_count, cudaStream_t s);
// Exact argmin from the GEMM's 8 candidates per row; rows whose candidate
// band overflows are appended to overflow_rows (*n_overflow counts them) and
// left for the exact tiled kernel.
cudaError_t launch_rescore_top8(const float* x, const float* xn2, const float* xres, int64_t n, int dim, int kp,
                                const float* cent, int k, const float* cmax, const int32_t* cand_idx,
                                const float* cand_val, int32_t* out_idx, float* out_d2, int64_t* overflow_rows,
                                int* n_overflow, cudaStream_t s);
// Warm k-means assignment (after the first iteration): how far each centroid
// moved, each row's bound on its best screened score from its previous
// centroid's distance and shift, and the exact nearest among the centroids
// the filter GEMM kept under that bound (rows over cap, or with none, to
// overflow_rows for the exact kernel). out_d2: the reference-order squared
// distance to the chosen centroid.
cudaError_t launch_centroid_shift(const float* cnew, const float* cold, int k, int dim, float* shift,
                                  cudaStream_t s);
cudaError_t launch_warm_bound(const float* d2, const int32_t* prev, const float* shift, const float* xn2,
                              const float* xres, const float* cmax, int kp, int64_t n, float* rthr, cudaStream_t s);
cudaError_t launch_rescore_filtered(const float* x, int64_t n, int dim, const float* cent, const int32_t* cnt,
                                    const int32_t* cand_id, int cap, int32_t* out_idx, float* out_d2,
                                    int64_t* overflow_rows, int* n_overflow, cudaStream_t s);
// Final step of the screened probe (kernels_rescore.cu): exact rescoring of
// each query's band list, the np nearest lists ascending, fallback flags.
// Queries flagged need_exact select on their whole exact row (Drow scratch,
// nlist floats per query).
cudaError_t launch_probe_final(const float* Q, int64_t nq, int dim, const float* coarse, int nlist,
                               const int32_t* nprobe, int np_max, const int32_t* k, const int32_t* list_len,
                               int allow_fallback, int lcap, const unsigned long long* band, const int32_t* lcount,
                               const int32_t* need_exact, float* Drow, int32_t* probe_ids, float* probe_d,
                               int32_t* fallback, unsigned long long* fallback_count, int32_t* todo,
                               cudaStream_t s);

// out[0] = max_i sqrt(sqnorm[i]), out[1] = max_i resid[i].
cudaError_t launch_norm_maxes(const float* sqnorm, const float* resid, int n, float* out, cudaStream_t s);

// ---- search ---------------------------------------------------------------------

struct ScanParams {
    int dim, M, dsub, pqK, nlist, code_stride;
    const float* coarse;      // [nlist][dim]
    const float* codebooks;   // [M][pqK][dsub]
    const float* codebooks_t; // [pqK][M][dsub]: codeword j of every subquantizer in one row
    const int64_t* list_start;  // [nlist] first row of each list
    const int32_t* list_len;    // [nlist]
    const uint8_t* codes;     // [rows][code_stride]
    const uint8_t* scanc;     // scan codes (kernels_scan.cu): permuted per lane, blocked by groups of rows
    const int64_t* sw_start;  // [nlist] first scan-code slot of each list
    // FP16 lookup tables (kernels_scan.cu)
    const float* adc_cb;      // [pqK][M][dsub] codewords minus their subquantizer's mean
    const float* adc_mu;      // [dim] the subquantizers' mean codewords, concatenated
    const float* adc_rm;      // [M] largest ||codeword - mean|| per subquantizer
    float adc_rfull;          // bound on ||r|| over every residual the codebooks reconstruct
    float adc_tbound;         // bound on |term| = | ||r||^2 + 2 <c, r> |
    int adc_table;            // lookup tables: 0 FP32, 1 FP16, 2 16-bit fixed point
    float* scan_cut;          // [nq] parity mode, 16-bit tables: no row left out screened below it
    float* scan_eps;          // [nq] bound on the screen's error
    int32_t* redo;            // rerank: queries whose top k the 16-bit screen cannot prove ...
    int32_t* redo_count;      // ... and their count
    unsigned long long* redo_total;  // optional: running count of those queries
    const float* term;        // [rows]
    const int32_t* row_cluster;  // [rows]
    const float* vectors;     // [rows][dim]
    const int64_t* row_id;    // [rows]
    const int32_t* kq;        // [nq] per-query k (sets each query's rerank depth)
    const int32_t* qorder;    // optional: block b works on query qorder[b] (L2-friendly order)
    const int32_t* qcount;    // optional with qorder: blocks at or past *qcount have no query
    int mode, rerank_fixed;
    // optional (table scan): scan_dump_bytes(R) bytes per query slot where
    // the scan's warps leave their candidates for a separate selection
    // kernel, so that a scan block ends with its walk; null: the scan block
    // selects its query's candidates itself
    void* dump;
};

// Bytes of the table scan's candidate dump per query slot at rerank depth R.
size_t scan_dump_bytes(int R);

// Per query: the nprobe nearest coarse lists in ascending (distance, index)
// order and their distances, from a distance matrix D[nq][nlist]. Also sets
// fallback[q] when the probed lists hold fewer than k[q] rows.
cudaError_t launch_probe_select(const float* D, int64_t nq, int nlist, const int32_t* nprobe, int np_max,
                                const int32_t* k, const int32_t* list_len, int allow_fallback,
                                int32_t* probe_ids, float* probe_d, int32_t* fallback,
                                unsigned long long* fallback_count, cudaStream_t s);

// ADC scan: per query, the R best rows by the decomposed PQ distance over the
// probed lists (all lists for a fallback query). probe_d [nq][np_max] holds
// the exact coarse distance of each probed list. Outputs rows (-1 padded),
// approximate distances and candidate sequence keys; adds the rows it
// scanned to *rows_scanned (may be null).
cudaError_t launch_scan(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                        const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback,
                        int R, int32_t* cand_row, float* cand_d, uint32_t* cand_seq,
                        unsigned long long* rows_scanned, cudaStream_t s);

// The bank-conflict-free scan (kernels_scan.cu) for M up to 32, with FP16
// or FP32 lookup tables; launch_scan dispatches to it when it applies. Its
// candidates leave unsorted.
bool scan_adc_supported(int M);
int scan_codes_per_row(int M);
int scan_group_rows(int M);
size_t scan_adc_smem(int R, int M, int fp16);
// Scan codes (kernels_scan.cu) of every slot of every list, or of the rows at
// positions rows[i] in lists cluster[i].
cudaError_t launch_scan_codes_lists(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                    const int32_t* list_len, const int64_t* sw_start, int nlist, uint8_t* scanc,
                                    cudaStream_t s);
cudaError_t launch_scan_codes_rows(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                   const int64_t* sw_start, const int64_t* rows, const int32_t* cluster, int64_t n,
                                   uint8_t* scanc, cudaStream_t s);
// Codebooks [M][pqK][dsub] -> [pqK][M][dsub] (the scan's table-build layout).
cudaError_t launch_transpose_codebooks(const float* cb, int M, int pqK, int dsub, float* out, cudaStream_t s);
cudaError_t launch_scan_adc(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                            const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback, int R,
                            int32_t* cand_row, float* cand_d, uint32_t* cand_seq, unsigned long long* rows_scanned,
                            cudaStream_t s);

// Rerank the R candidates of each query with an exact FP32 distance and emit
// the k best: mode 0 = the reference's reconstructed-vector distance
// (decodePQCode + vectorAdd, pqivf/index.go:909-923), mode 1 = the raw
// vector. ids [nq][kmax] (-1 padded), dist [nq][kmax] = sqrt(rank) in FP64,
// nout [nq].
cudaError_t launch_rerank(const ScanParams& p, const float* queries, int64_t nq, const int32_t* cand_row,
                          const uint32_t* cand_seq, int R, const int32_t* k, int kmax, int mode,
                          int64_t* ids, double* dist, int32_t* nout, cudaStream_t s);

// Query order for the scan and rerank: queries grouped by their first
// probed list (a counting sort), so blocks that run at the same time read
// overlapping lists and more of the list reads hit L2. scratch: nlist ints.
cudaError_t launch_probe_order(const int32_t* probe_ids, int64_t nq, int np_max, int nlist, int32_t* scratch,
                               int32_t* order, cudaStream_t s);

// Moves every list's slots to a new layout (one block per list), dropping
// tombstones (row id -1) in the lists flagged compact.
cudaError_t launch_relayout_lists(int nlist, const int64_t* src_start, const int32_t* src_len,
                                  const int64_t* dst_start, const int32_t* compact, int dim, int cwords,
                                  const float* vin, float* vout, const void* cin, void* cout, const float* tin,
                                  float* tout, const int64_t* rin, int64_t* rout, const int32_t* clin, int32_t* clout,
                                  cudaStream_t s);

// ---- list-major batched scan on the tensor cores (kernels_lms.cu) --------------

constexpr int LMS_NQ = 64;        // queries per work item (the MMA's largest N here)
constexpr int LMS_MAX_CHUNKS = 8;  // probe-rank chunks of one search

// One work item: rows [row_begin, row_begin + n_rows) of list `list` against
// the n_pairs queries whose pairs start at pair_begin in the pair arrays.
struct LmsItem {
    int32_t list, pair_begin, n_pairs, row_begin, n_rows, pad;
    int64_t row0;  // global row of row_begin
};

// Probe-rank chunks: chunk c holds ranks [bound[c], bound[c + 1]), the last
// one up to each query's nprobe.
struct LmsChunks {
    int n;
    int bound[LMS_MAX_CHUNKS + 1];
};

// Index-wide constants of the FP16 error bound: max ||r|| and max ||r - r~||
// over every reconstructable residual (from the codebooks), max |term|, the
// padded K of the dot products.
struct LmsBound {
    float rmax, rd, tmax;
    int kpad;
};

struct LmsParams {
    const uint8_t* codes;
    int code_stride;
    const float* term;
    const int64_t* list_start;
    const void* cb16;  // __half [M][pqK][dsub]
    int M, dsub, pqK, dim;
    const void* q16;   // __half [nq][128]
    const LmsItem* items;
    const int32_t* n_items;
    int32_t* item_counter;
    int item_cap;       // items of one chunk's region
    const int32_t* pair_q;
    const float* pair_base;
    const int32_t* pair_off;
    const float* thr;
    int32_t* cnt;
    int32_t* cand_id;
    float* cand_s;
    int cap, dense;
    unsigned long long* stats;  // optional: [0] (query, row) pairs scored, [1] rows decoded
    int* err;
};

bool lms_supported(int dim, int M, int pqK);
int lms_smem_bytes();
cudaError_t launch_lms_prep(const float* Q, int64_t nq, int dim, const int32_t* probe_ids, const float* probe_d,
                            const int32_t* nprobe, int np_max, const int32_t* fallback, const int32_t* list_len,
                            int first_w, int min_nprobe, const LmsBound& bd, int mode, const int32_t* kq, int rfixed,
                            int32_t* bandk, float* eps, void* q16, float* e2, float* asl, int32_t* cnt,
                            int32_t* lcount, float* thr, int32_t* need, cudaStream_t s);
// First thresholds from a table scan of each query's nearest list (its R
// best scores in cand_d [nq][R]).
cudaError_t launch_lms_seed(int64_t nq, int R, const float* cand_d, const int32_t* bandk, const float* eps,
                            const float* e2, const float* asl, float* thr, cudaStream_t s);
// Work queue of every chunk (queries flagged in `skip` -- the prep's
// table-scan flags -- take no part): counts [n * nlist], cursor [n * nlist],
// totals [2] ([1]: set when a chunk's items overflow item_cap, which sends
// every query to the table scan), items [n * item_cap], n_items [n], pair
// arrays [nq * np_max].
cudaError_t launch_lms_queue(const int32_t* probe_ids, const float* probe_d, const int32_t* nprobe, int64_t nq,
                             int np_max, const int32_t* fallback, const LmsChunks& ch, int nlist,
                             const int32_t* list_len, const int64_t* list_start, int rows_max, int item_cap,
                             int32_t* counts, int32_t* cursor,
                             int32_t* totals, LmsItem* items, int32_t* n_items, int32_t* pair_q, float* pair_base,
                             int32_t* pair_off, cudaStream_t s);
cudaError_t launch_lms_scan(const LmsParams& p, int grid, cudaStream_t s);
// Band lists to rerank candidates; queries for the table scan to redo
// (count at redo[nq]).
cudaError_t launch_lms_finish(int64_t nq, int mode, int R, int lcap, const int32_t* kq, int rfixed,
                              const unsigned long long* list, const int32_t* lcount, const int32_t* need,
                              const int32_t* probe_ids, const int32_t* nprobe, int np_max, const int32_t* row_cluster,
                              const int32_t* overflow, int32_t* cand_row, uint32_t* cand_seq, int32_t* redo,
                              cudaStream_t s);

// ---- batched exact k-NN over a flat base (kernels_knn.cu) ------------------------

constexpr int KNN_SIMT_DMAX = 256;  // register-tiled SIMT distances up to this dimension
constexpr int KNN_TC_DMAX = 128;    // tensor-core screen up to this dimension (GEMM K)

// Exact SIMT filter over base rows [c_begin, c_end) for metric 0..3: every
// (distance, row) key below thr[qi] is appended to the candidate buffer of
// query qi (cap entries per query; cnt keeps counting past cap). Row r of the
// launch is query qlist[r] (all nrows queries when qlist is null).
cudaError_t launch_knn_filter(int metric, const float* q, const int32_t* qlist, int nrows, int dim, const float* base,
                              int64_t c_begin, int64_t c_end, const float* qnorm, const float* bnorm,
                              const unsigned long long* thr, int cap, int32_t* cnt, int32_t* cand_id, float* cand_d,
                              cudaStream_t s);
// Reference-order distances of nrows queries to base rows [c_begin, c_end)
// as FP64, out[r * ld + col - c_begin].
cudaError_t launch_knn_matrix(int metric, const float* q, int nrows, int dim, const float* base, int64_t c_begin,
                              int64_t c_end, const float* qnorm, const float* bnorm, double* out, int64_t ld,
                              cudaStream_t s);
// Folds each query's candidates into its sorted top-k list; a query whose
// candidates overflowed is flagged in redo (and counted) and keeps its list.
cudaError_t launch_knn_merge_exact(int nrows, const int32_t* qlist, int k, int cap, int32_t* cnt,
                                   const int32_t* cand_id, const float* cand_d, unsigned long long* list,
                                   int32_t* lcount, unsigned long long* thr, int32_t* redo, int* redo_count,
                                   cudaStream_t s);
size_t knn_merge_exact_smem(int k, int cap);
// Tensor-core screen: filter GEMM (kernels_gemm.cu), band merge, exact final.
// cmode 0: cterm = (bias, -2) (squared scores); cmode 1: cterm = (0, scale).
// first: every row's threshold is +inf (the first chunk, counts zero), so
// every column is kept: they are written in column order without atomics
// (when the chunk fits cap).
cudaError_t launch_gemm_filter(const void* a_bf16, int64_t nrows, const void* b_bf16, int64_t nb, int kp,
                               int col_begin, int col_end, const float2* cterm, int cmode, const float* rthr, int cap,
                               int32_t* cnt, int32_t* cand_id, float* cand_s, int* err, cudaStream_t s,
                               bool first = false);
// todo: nrows + 1 ints of scratch (the rows left to the block kernel and
// their count).
cudaError_t launch_knn_merge_band(int nrows, int k, const int32_t* krow, int cap, int lcap, int32_t* cnt,
                                  const int32_t* cand_id, const float* cand_s, const float* e2, const float* asl,
                                  unsigned long long* list, int32_t* lcount, float* thr, int32_t* need_exact,
                                  int32_t* todo, cudaStream_t s);
size_t knn_merge_band_smem(int lcap, int cap);
cudaError_t launch_knn_final_band(int metric, int nrows, int k, int lcap, int dim, const float* queries,
                                  const float* base, const float* qnorm, const float* bnorm,
                                  const unsigned long long* list, const int32_t* lcount, const int32_t* need_exact,
                                  int32_t* exact_list, int* exact_count, int64_t* out_ids, double* out_dist,
                                  cudaStream_t s);
// Sorted exact lists of rows qlist[p] (or all nrows) to ids / FP64 distances.
cudaError_t launch_knn_emit(int nrows, int k, const unsigned long long* list, const int32_t* lcount,
                            const int32_t* qlist, int64_t* out_ids, double* out_dist, cudaStream_t s);
// dot_ref(x, x) of every row (the cosine kernel's norm accumulation).
cudaError_t launch_ref_sqnorm(const float* x, int64_t n, int dim, float* out, cudaStream_t s);
// Screen epilogue terms per base row and the maxima the error bound needs
// (maxes: two floats as bits, zeroed by the caller).
cudaError_t launch_knn_col_terms(const float* sqnorm, const float* resid, int64_t n, int cosine, float2* terms,
                                 unsigned int* maxes, cudaStream_t s);
cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s);
cudaError_t launch_fill_i32(int32_t* p, int64_t n, int32_t v, cudaStream_t s);
// (sqnorm[i], -2): squared-Euclidean screen terms.
cudaError_t launch_sq_terms(const float* sqnorm, int64_t n, float2* terms, cudaStream_t s);
// Per-query band constants e2 (= 2 eps) and slack scale.
cudaError_t launch_knn_query_band(const float* qsq, const float* qres, int64_t nq, int kp, int cosine,
                                  const unsigned int* maxes, float* e2, float* asl, cudaStream_t s);

}  // namespace hann
