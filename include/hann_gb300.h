/*
 * hann_gb300.h -- C ABI of the GB300 PQIVF index and the GPU distance layer.
 *
 * This is the boundary a host binding (the cgo package of a Go drop-in
 * beside hann's pqivf, or the ctypes mirror in hann_gb300/__init__.py)
 * calls. Plain pointers and sizes only. Every function returns 0 on success
 * or a negative HANN_E* status; hann_pqivf_last_error() then describes the
 * failure. Every host input is copied before the call returns, so a caller
 * may free or reuse its buffers at once (the cgo rule against retained Go
 * pointers). A handle is safe for concurrent use: mutations are exclusive and
 * searches are serialised on the handle's stream.
 *
 * Each entry point names the reference interface it replaces (file:line in
 * habedi/hann).
 */
#ifndef HANN_GB300_H
#define HANN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define HANN_OK 0
#define HANN_E_INVALID -1     /* invalid argument (dimension, k, parameter) */
#define HANN_E_NOT_FOUND -2   /* id not present */
#define HANN_E_EXISTS -3      /* id already present */
#define HANN_E_STATE -4       /* not trained / empty index / not enough vectors */
#define HANN_E_CUDA -5        /* CUDA runtime failure */
#define HANN_E_NOMEM -6       /* device or host allocation failed */
#define HANN_E_UNSUPPORTED -7 /* valid for the reference, outside this build's limits */
#define HANN_E_CHANGED -8     /* the index changed between a size query and the call sized from it: query again */

typedef struct hann_pqivf hann_pqivf;

/* Options of pqivf.New (pqivf/index.go:57-146). hann_pqivf_options_init
 * fills the reference's defaults: coarse_k 16, pq_k 16, kmeans_iters 10,
 * candidate_clusters 3, fallback on, num_subquantizers = the largest of
 * 8/4/2/1 dividing the dimension (pqivf/index.go:106-157); the With*
 * options then overwrite single fields. */
typedef struct {
    int32_t dimension;
    int32_t coarse_k;           /* WithCoarseK */
    int32_t num_subquantizers;  /* WithNumSubquantizers */
    int32_t pq_k;               /* WithPQK; this build stores uint8 codes, so pq_k <= 256 */
    int32_t kmeans_iters;       /* WithKMeansIters */
    int32_t candidate_clusters; /* WithCandidateClusters (nprobe) */
    int32_t fallback;           /* WithBruteForceFallback: 1 on, 0 off */
    uint64_t seed;              /* plays HANN_SEED's role (core/utils.go:12-20) */
    int32_t device;             /* CUDA device ordinal */
    int32_t rerank;             /* candidates rescored exactly per query; 0 = automatic */
    int32_t plain_fp32;         /* 1: no tensor-core preselection; every assignment and probe runs the
                                   FP32 SIMT kernels (same results, for comparison); 0 = default */
} hann_pqivf_options;

/* Defaults of pqivf.New for the given dimension (pqivf/index.go:106-157). */
void hann_pqivf_options_init(hann_pqivf_options* opts, int32_t dimension);

/* core.IndexStats (core/index.go:131-140). */
typedef struct {
    int64_t count;
    int32_t dimension;
    int64_t fallback_searches;
    int32_t trained;
    int32_t nlist;
    int64_t rows_capacity;
} hann_pqivf_index_stats;

/* pqivf.New (pqivf/index.go:106-146). Validation errors as the reference. */
int hann_pqivf_new(const hann_pqivf_options* opts, hann_pqivf** out);
void hann_pqivf_free(hann_pqivf* h);
/* Message of the calling thread's last failed hann_pqivf_* call, on any
 * handle (h may be NULL, e.g. after a failed hann_pqivf_new). Kept per
 * thread, as errno is, so that threads sharing a handle each read their own
 * failure; valid until this thread's next failing call. */
const char* hann_pqivf_last_error(const hann_pqivf* h);

/* Index.Add (core/index.go:25; pqivf/index.go:212-237). */
int hann_pqivf_add(hann_pqivf* h, int64_t id, const float* vector);
/* BulkIndex.BulkAdd (core/index.go:57; pqivf/index.go:266-297): applied in
 * ascending id order; stops at the first failing id, keeping earlier ones. */
int hann_pqivf_bulk_add(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n);
/* Index.Delete (core/index.go:29; pqivf/index.go:300-345). */
int hann_pqivf_delete(hann_pqivf* h, int64_t id);
/* BulkIndex.BulkDelete (core/index.go:60; pqivf/index.go:350-384): unknown
 * ids are skipped. */
int hann_pqivf_bulk_delete(hann_pqivf* h, const int64_t* ids, int64_t n);
/* Index.Update (core/index.go:34; pqivf/index.go:402-413). */
int hann_pqivf_update(hann_pqivf* h, int64_t id, const float* vector);
/* BulkIndex.BulkUpdate (core/index.go:63; pqivf/index.go:419-444). */
int hann_pqivf_bulk_update(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n);

/* Trainer.Train (core/index.go:68; pqivf/index.go:451-605). */
int hann_pqivf_train(hann_pqivf* h);
/* Train with explicit k-means seeding, replacing the reference's draws from
 * its package RNG (pqivf/index.go:804-810, 830-837): coarse_init holds
 * coarse_k row indices into the id-sorted data (its Perm(n)[:k]); pq_init
 * holds num_subquantizers x pq_k row indices into each subquantizer's
 * residual data; reseed is the stream of row indices used in order for
 * every empty cluster (coarse run first, then subquantizer 0, 1, ...).
 * Any pointer may be NULL to draw from the handle's seeded generator. */
int hann_pqivf_train_seeded(hann_pqivf* h, const int64_t* coarse_init, const int64_t* pq_init,
                            const int64_t* reseed, int64_t n_reseed);
/* Incremental re-Train after many mutations (no counterpart: the
 * reference's Train reseeds from scratch, pqivf/index.go:451-605, and keeps
 * the centroids fixed between Train calls, 306-312). `iters` Lloyd
 * iterations over every stored vector starting from the index's own
 * centroids, then as many on the residuals starting from its own codebooks,
 * then every vector reassigned and re-encoded, as Train does; 0 iterations
 * only repacks the lists. Needs a trained index whose vector count still
 * gives the same list and codebook sizes. */
int hann_pqivf_retrain(hann_pqivf* h, int32_t iters);

/* Index.Search (core/index.go:38; pqivf/index.go:850-949) for one query:
 * ids/distances (true Euclidean distance as float64) of up to k neighbours
 * in non-decreasing order; *n_out receives the count. */
int hann_pqivf_search(hann_pqivf* h, const float* query, int32_t k, int64_t* ids, double* distances,
                      int32_t* n_out);

/* Batched Search: nq independent Search calls in one device pass. k and
 * nprobe are per query (nprobe NULL = the index's candidate clusters).
 * Row i of ids/distances starts at i * kmax. mode 0 returns the reference's
 * reconstructed-vector PQ distances (parity); mode 1 reranks the candidates
 * against the stored raw vectors (exact distances, higher recall). */
int hann_pqivf_search_batch(hann_pqivf* h, const float* queries, int64_t nq, const int32_t* k,
                            const int32_t* nprobe, int32_t kmax, int32_t mode, int64_t* ids, double* distances,
                            int32_t* n_out);

/* Same as hann_pqivf_search_batch with every buffer in device memory and
 * the work enqueued on `stream` (a cudaStream_t, NULL = the handle's own);
 * k and nprobe are uniform. Returns once enqueued, without waiting for the
 * device. Calls share the handle's scratch: calls on different streams must
 * be ordered by the caller. A mutation of the handle waits for the searches
 * enqueued before it; brute-force fallbacks are counted on the device and
 * appear in hann_pqivf_stats (which waits for those searches). */
int hann_pqivf_search_batch_device(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k, int32_t nprobe,
                                   int32_t mode, int64_t* d_ids, double* d_distances, int32_t* d_n_out,
                                   void* stream);

/* Autotuner of the list scan (no reference counterpart: the reference scans
 * each query's candidates one by one, pqivf/index.go:905-936). Times the
 * table scan and a few forms of the list-major tensor-core scan (chunking
 * of the probe ranks, rows of a list per work item) on the nq host queries
 * with k and mode, at nprobe 8, 16, 32, 64, 128 and 256 (capped at nlist),
 * keeps the fastest list-major form and routes every later query probing at
 * least the crossover nprobe (the smallest from which that form wins at
 * every larger value) to it, the others to the table scan. chosen8 (may be
 * NULL) receives the options in the layout of hann_pqivf_scan_options;
 * ms_table / ms_list (may be NULL, 6 entries) the measured milliseconds of
 * the table scan and of the chosen form per nprobe (-1 where not run). In
 * mode 0 results do not depend on the choice; in mode 1 a query's result
 * depends only on the query and the tuned state. */
int hann_pqivf_autotune_scan(hann_pqivf* h, const float* queries, int64_t nq, int32_t k, int32_t mode,
                             int32_t* chosen8, double* ms_table, double* ms_list);

/* Sets the default nprobe (WithCandidateClusters, pqivf/index.go:86-94) of a
 * live index, e.g. to the value a recall-target tuning picked. */
int hann_pqivf_set_candidate_clusters(hann_pqivf* h, int32_t n);

/* nprobe from a recall target: the caller side of Search, where the
 * reference's callers pick WithCandidateClusters by hand
 * (example/run_datasets.go:115-120, pqivf/index.go:86-94). Tries the nprobe
 * values of `ladder` (n_ladder entries, ascending; NULL = 1, 2, 4, ... up to
 * min(nlist, 4096), at most HANN_TUNE_LADDER_MAX values) in order, searching
 * the nq queries with k and mode, and stops at the first whose recall@k
 * reaches target_recall; *chosen = that nprobe, or the last one tried when
 * none does. Recall is measured against ground_truth ids [nq][k] (-1 = no
 * neighbour), or, when NULL, against an exact k-NN of the stored vectors
 * computed on the GPU. tried_out / recall_out (may be NULL; room for every
 * ladder entry) receive each nprobe tried and its recall, *n_tried their
 * count. With apply != 0 the index's default nprobe becomes *chosen. */
#define HANN_TUNE_LADDER_MAX 14
int hann_pqivf_tune_candidate_clusters(hann_pqivf* h, const float* queries, int64_t nq, int32_t k,
                                       double target_recall, const int32_t* ladder, int32_t n_ladder, int32_t mode,
                                       const int64_t* ground_truth, int32_t apply, int32_t* chosen,
                                       int32_t* tried_out, double* recall_out, int32_t* n_tried);

/* Lookup tables of the list scan: HANN_ADC_FP32, HANN_ADC_FP16 or
 * HANN_ADC_FIXED16 (16-bit fixed point, the default). The reference decodes
 * every candidate in FP32 (pqivf/index.go:909-923); here the scan screens
 * candidates with per-query tables and the rerank computes the reference's
 * distance. 16-bit tables take half the shared memory and read without bank
 * conflicts; fixed point sums a row exactly in integers (its only error is
 * each entry's rounding, a 65,534th of the largest entry bound, where FP16's
 * is a 2,048th of each entry). In parity mode (mode 0) each query's top k
 * is proven against the 16-bit screen's error bound, and the queries it
 * cannot prove are scanned again with FP32 tables, so parity-mode results do
 * not depend on this choice. In exact-rerank mode (mode 1) the screened
 * candidates can differ at the rerank depth. */
#define HANN_ADC_FP32 0
#define HANN_ADC_FP16 1
#define HANN_ADC_FIXED16 2
int hann_pqivf_set_adc_tables(hann_pqivf* h, int32_t kind);

/* Switches the plain-FP32 mode of hann_pqivf_options at run time (no
 * reference counterpart; results do not change). */
int hann_pqivf_set_plain_fp32(hann_pqivf* h, int32_t on);

/* Diagnostics (no reference counterpart). With profiling on, every search
 * stage is bracketed by CUDA events on the stream it runs on and the list
 * scan counts the rows it reads; hann_pqivf_stage_times waits for the events
 * and returns the accumulated device milliseconds of the stages [coarse
 * distances, probe select, list scan, rerank], the kernel launch count and
 * the rows scanned, then clears them. */
int hann_pqivf_set_profiling(hann_pqivf* h, int32_t on);
int hann_pqivf_stage_times(hann_pqivf* h, double* ms4, int64_t* launches, int64_t* rows_scanned);
/* Current length of every inverted list: *n_out = nlist, and out[0..nlist)
 * when nlist <= capacity, else HANN_E_CHANGED (a Train changed nlist). */
int hann_pqivf_list_lengths(hann_pqivf* h, int64_t* out, int32_t capacity, int32_t* n_out);

/* Allocation-free variant of hann_pqivf_search_batch_device. It has no
 * counterpart in the reference. It is for callers that cannot allocate
 * device memory while they search: a serving thread that must not stall on
 * the device-wide synchronisation cudaMalloc/cudaFree may cause, code that
 * records the search into a CUDA graph (no allocator calls while a stream is
 * captured), or a process whose device-memory budget is fixed at start-up.
 * All scratch comes from one fixed 16 MiB device array that every GPU which
 * loads this library holds until the process exits; a batch whose scratch
 * (about nq * (4 * nlist + 8 * nprobe + 12 * rerank depth + 24) bytes) does
 * not fit is rejected with HANN_E_UNSUPPORTED and a message that says so.
 * The coarse distances dominate: every query needs a full row of them, so
 * the number of queries per call is small when the index has many lists
 * (about 250 queries at 16,384 lists, about 65,000 at 64 lists).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call shares the array, so calls whose work overlaps on the GPU
 * (different streams, threads or handles) race; serialise them. Fallbacks
 * are counted as for hann_pqivf_search_batch_device. It scans the lists with
 * the table scan: in exact-rerank mode (1) its results are those of
 * hann_pqivf_search_batch_device with the list-major scan switched off,
 * which may differ from the list-major scan's where a row competes at the
 * rerank depth; in mode 0 both give the reference's results. */
int hann_pqivf_search_batch_device_noalloc(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k,
                                           int32_t nprobe, int32_t mode, int64_t* d_ids, double* d_distances,
                                           int32_t* d_n_out, void* stream);

/* Index.Stats (core/index.go:41; pqivf/index.go:953-966). */
int hann_pqivf_stats(hann_pqivf* h, hann_pqivf_index_stats* out);

/* ---- continuous-batching server -------------------------------------------
 * No single reference counterpart: the reference serves concurrent Search
 * calls under its RWMutex (pqivf/index.go:37, 850-853) from a goroutine pool
 * (example/run_datasets.go:84-120). Here requests from any host thread are
 * packed into device batches that run on `slots` CUDA streams at once;
 * requests arriving meanwhile join the next free slot; a batch is admitted
 * only while its device scratch fits the slot's share of memory_budget.
 * Add/Delete requests take effect before any batch queued after them starts;
 * when they move no row (appends into spare capacity, tombstone deletes)
 * they run beside the batches already in flight, which may or may not see
 * them. Each request's result equals a Search of its queries alone. */
typedef struct hann_server hann_server;
typedef struct {
    int32_t slots;             /* batches in flight (streams); default 4 */
    int32_t max_batch_queries; /* queries per device batch; default 4096 */
    int32_t max_k;             /* largest k a request may ask; default 100 */
    int32_t max_nprobe;        /* nprobe is clamped to this; default 256 */
    int32_t mode;              /* 0 PQ distances (parity), 1 exact rerank; default 1 */
    int64_t memory_budget;     /* device bytes for batch scratch; default 120 GiB */
    int64_t max_batch_probes;  /* sum over a batch's queries of nprobe, a bound on its scan work (and so on the
                                  latency of every request in it); 0 = no bound; default 0 */
} hann_serve_options;
typedef struct {
    int64_t requests, queries, batches, mutations, peak_admitted_bytes;
    double p50_ms, p99_ms, queries_per_s;
    int64_t relayouts;  /* mutations that had to wait for the batches in flight */
    double mutation_ms; /* host time spent applying mutations */
    double drain_ms;    /* of which waiting for the batches in flight before relayouts */
    double relayout_ms; /* of which applying relayouts (no batch starts meanwhile) */
    double relayout_max_ms; /* the longest single drain + relayout */
} hann_serve_statistics;

void hann_serve_options_init(hann_serve_options* opts);
int hann_serve_start(hann_pqivf* h, const hann_serve_options* opts, hann_server** out);
/* Queues nq queries (copied) with one k and nprobe; returns a ticket. */
int hann_serve_submit(hann_server* s, const float* queries, int32_t nq, int32_t k, int32_t nprobe, uint64_t* ticket);
/* hann_serve_submit with a priority: 1 puts the request ahead of every
 * normal-priority search still queued (no reference counterpart). */
int hann_serve_submit_priority(hann_server* s, const float* queries, int32_t nq, int32_t k, int32_t nprobe,
                               int32_t priority, uint64_t* ticket);
/* Withdraws a search that has not started: HANN_OK and the ticket's wait
 * returns HANN_E_STATE ("request cancelled"); HANN_E_STATE when it already
 * runs or finished (its wait returns the results); HANN_E_NOT_FOUND for an
 * unknown ticket. Mutations are not cancelled (no reference counterpart). */
int hann_serve_cancel(hann_server* s, uint64_t ticket);
/* Queues a BulkAdd / BulkDelete, applied in order beside the running
 * batches; a search submitted after the mutation's ticket was waited for
 * sees it. */
int hann_serve_submit_add(hann_server* s, const int64_t* ids, const float* vectors, int64_t n, uint64_t* ticket);
int hann_serve_submit_delete(hann_server* s, const int64_t* ids, int64_t n, uint64_t* ticket);
/* Waits for a ticket (timeout_ms < 0: no limit) and copies its results:
 * ids/distances [nq*k], n_out [nq]; latency_ms = submit to completion. */
int hann_serve_wait(hann_server* s, uint64_t ticket, int64_t* ids, double* distances, int32_t* n_out,
                    int32_t timeout_ms, double* latency_ms);
int hann_serve_stats(hann_server* s, hann_serve_statistics* out);
/* Message of the calling thread's last failed hann_serve_* call (per
 * thread, as hann_pqivf_last_error). */
const char* hann_serve_last_error(const hann_server* s);
/* Finishes the queued work, then releases the server. */
int hann_serve_stop(hann_server* s);
/* A load generator for the server (no reference counterpart: the caller
 * side of example/run_datasets.go:84-120 driven by an arrival schedule).
 * The calling thread submits the n requests at their arrival times (sleeping
 * to within 0.2 ms, then spinning) while a native thread waits for each in
 * submission order, so neither the submission schedule nor the latency
 * depends on the caller's language runtime. Search requests take rows
 * query_rows[first .. first + count) of queries [n_queries][dim]; BulkAdd
 * requests add_ids / add_vectors rows [first, first + count) of n_add;
 * BulkDelete requests del_ids [first, first + count) of n_del. A search with
 * out_offset >= 0 copies its ids ([count][k]) to out_ids + out_offset (of
 * n_out_ids). A request naming a range outside its array is refused
 * (HANN_E_INVALID) before anything is submitted. Per request: latency_ms[i]
 * (submit to completion, the server's clock) and late_ms[i] (how long after
 * its arrival time it was submitted). */
typedef struct {
    double at_ms;        /* arrival time after the start, milliseconds */
    int32_t kind;        /* 0 search, 1 BulkAdd, 2 BulkDelete */
    int32_t k, nprobe;   /* search */
    int32_t pad;
    int64_t first, count;
    int64_t out_offset;  /* search: where its ids go in out_ids, -1 = not kept */
} hann_serve_request;
int hann_serve_replay(hann_server* s, const hann_serve_request* reqs, int64_t n, const float* queries,
                      int64_t n_queries, const int64_t* query_rows, int64_t n_query_rows, const int64_t* add_ids,
                      const float* add_vectors, int64_t n_add, const int64_t* del_ids, int64_t n_del,
                      int64_t* out_ids, int64_t n_out_ids, double* latency_ms, double* late_ms);

/* ---- persisted state (Save/Load, pqivf/index.go:969-1101) ----------------
 * The binding encodes/decodes the reference's gob stream itself and moves
 * the arrays through these calls. */
typedef struct {
    int32_t dimension, coarse_k, num_subquantizers, pq_k, kmeans_iters, candidate_clusters, fallback, trained;
    int32_t nlist;          /* rows of coarse centroids */
    int32_t pq_k_eff;       /* codewords per subquantizer actually trained */
    int64_t n_rows;         /* entries held in inverted lists */
    int64_t n_pending;      /* vectors waiting for Train */
} hann_pqivf_layout;

int hann_pqivf_export_layout(hann_pqivf* h, hann_pqivf_layout* out);
/* Arrays sized from `layout` (what hann_pqivf_export_layout returned):
 * coarse [nlist*dim], codebooks [M*pq_k_eff*(dim/M)], list_len [nlist],
 * list_key [nlist] (1 when the reference's list map holds the cluster),
 * cluster_counts [nlist], ids [n_rows] (list by list, in storage order),
 * vectors [n_rows*dim], codes [n_rows*M] (int32), pending_ids [n_pending],
 * pending_vectors [n_pending*dim]. The arrays are one consistent state
 * (GobEncode holds the read lock the same way, pqivf/index.go:992-1017);
 * when a mutation changed those sizes after the layout was read, nothing is
 * written and HANN_E_CHANGED is returned: read the layout again. */
int hann_pqivf_export(hann_pqivf* h, const hann_pqivf_layout* layout, float* coarse, float* codebooks,
                      int64_t* list_len, uint8_t* list_key, int64_t* cluster_counts, int64_t* ids, float* vectors,
                      int32_t* codes, int64_t* pending_ids, float* pending_vectors);
/* Replaces the handle's state (GobDecode, pqivf/index.go:1020-1084). Codes
 * of an entry with has_codes[i] == 0 are recomputed on the device. */
int hann_pqivf_import(hann_pqivf* h, const hann_pqivf_layout* layout, const float* coarse, const float* codebooks,
                      const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                      const int64_t* ids, const float* vectors, const int32_t* codes, const uint8_t* has_codes,
                      const int64_t* pending_ids, const float* pending_vectors);

/* ---- gob stream of Save/Load (pqivf/index.go:969-1101), host only -------
 * Save is hann_pqivf_export + hann_gob_encode; Load is hann_gob_decode +
 * hann_gob_state_layout + hann_gob_state_arrays + hann_pqivf_import. None of
 * these calls touches the GPU. The gob bytes are those the reference's Save
 * writes: the *pqivf.Index GobEncoder around a serializedPQIVF stream. */
typedef struct hann_gob_state hann_gob_state;
/* Encodes exported arrays (hann_pqivf_export's layout and arrays). With
 * out == NULL only *out_len is set (the exact size); otherwise capacity
 * must be at least that size. */
int hann_gob_encode(const hann_pqivf_layout* layout, const float* coarse, const float* codebooks,
                    const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                    const int64_t* ids, const float* vectors, const int32_t* codes, const int64_t* pending_ids,
                    const float* pending_vectors, uint8_t* out, int64_t capacity, int64_t* out_len);
/* GobEncode's bytes (pqivf/index.go:992-1017): the serializedPQIVF stream
 * alone, without Save's GobEncoder wrapper. Same size query and capacity
 * rules as hann_gob_encode. */
int hann_gob_encode_payload(const hann_pqivf_layout* layout, const float* coarse, const float* codebooks,
                            const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                            const int64_t* ids, const float* vectors, const int32_t* codes,
                            const int64_t* pending_ids, const float* pending_vectors, uint8_t* out, int64_t capacity,
                            int64_t* out_len);
/* Parses a gob stream: Save's (the *pqivf.Index GobEncoder value) or
 * GobEncode's (a struct value, its fields matched by name). */
int hann_gob_decode(const uint8_t* data, int64_t len, hann_gob_state** out);
/* GobDecode's checks and defaults (pqivf/index.go:1020-1084): the layout
 * of the decoded index; default_candidate_clusters is the configured
 * nprobe kept when the file carries none. */
int hann_gob_state_layout(const hann_gob_state* st, int32_t default_candidate_clusters, hann_pqivf_layout* out);
/* The decoded arrays, sized from the layout, as hann_pqivf_import takes
 * them; has_codes[i] is 0 where entry i's codes are missing or out of
 * range. */
int hann_gob_state_arrays(const hann_gob_state* st, float* coarse, float* codebooks, int64_t* list_len,
                          uint8_t* list_key, int64_t* cluster_counts, int64_t* ids, float* vectors, int32_t* codes,
                          uint8_t* has_codes, int64_t* pending_ids, float* pending_vectors);
void hann_gob_state_free(hann_gob_state* st);
/* Message of the calling thread's last failed hann_gob_* call. */
const char* hann_gob_last_error(void);

/* Binary snapshot of the whole index (the content of Save/Load's gob
 * stream, pqivf/index.go:969-1101, as flat arrays with byte codes and a
 * checksum; layout in hann_gb300/csrc/snapshot.cu). Save lets searches run
 * and holds mutations; Load replaces the handle's state after checking the
 * file's sizes and checksum, and leaves the index unchanged when they fail. */
int hann_pqivf_save_snapshot(hann_pqivf* h, const char* path);
int hann_pqivf_load_snapshot(hann_pqivf* h, const char* path);

/* ---- distance layer (core/simd_distance.h:30-33, core/metric.go:64-99) ----
 * metric: 0 squared Euclidean, 1 Euclidean, 2 Manhattan, 3 cosine. */
#define HANN_METRIC_SQEUCLID 0
#define HANN_METRIC_EUCLID 1
#define HANN_METRIC_MANHATTAN 2
#define HANN_METRIC_COSINE 3

/* simd_<metric>_batch (core/simd_kernels.inc.h:235-264): distance from one
 * query to n rows of flat, FP32 in the reference's NEON summation order,
 * widened to double. Host buffers. */
int hann_gpu_distance_batch(int32_t metric, const float* query, const float* flat, size_t dim, size_t n,
                            double* out);

/* Many queries at once: out[q * n + i] = distance(queries[q], base[i]), the
 * same values as hann_gpu_distance_batch row by row. Host buffers. */
int hann_gpu_distance_matrix(int32_t metric, const float* queries, int64_t nq, const float* base, int64_t n,
                             int32_t dim, double* out);

/* ---- batched exact k-NN over a flat base ---------------------------------
 * testutil.BruteForceKNN (internal/testutil/data.go:66-93) for a batch of
 * queries: per query the k rows of base with the smallest distance under the
 * metric, ascending by (distance, row), each distance the value
 * hann_gpu_distance_batch returns for that pair. Row numbers stand for the
 * reference's ids (0..n-1); slots past n are id -1, distance +inf. k is in
 * [1, 4096], n below 2^31.
 * method: HANN_KNN_EXACT computes every distance in FP32 in the reference's
 * summation order; HANN_KNN_TENSOR (squared Euclidean, Euclidean, cosine; dim
 * <= 128) screens with a BF16 tensor-core GEMM, then rescores exactly every
 * row whose screened score lies within the GEMM's error bound of the k-th --
 * the results are identical to HANN_KNN_EXACT; HANN_KNN_AUTO picks the tensor
 * screen where it applies. */
#define HANN_KNN_AUTO 0
#define HANN_KNN_EXACT 1
#define HANN_KNN_TENSOR 2

typedef struct hann_knn hann_knn;
typedef struct hann_knn_stats {
    int64_t queries;          /* queries answered */
    int64_t exact_queries;    /* answered by the exact path as requested */
    int64_t tensor_queries;   /* answered through the tensor-core screen */
    int64_t fallback_queries; /* screened queries whose band overflowed and ran exactly */
    int64_t chunks;           /* base chunks walked */
    int64_t redo_chunks;      /* chunks rerun in pieces after a candidate overflow */
} hann_knn_stats;

/* Copies the flat base [n][dim] (host) to the device. NULL on failure. */
hann_knn* hann_knn_new(const float* base, int64_t n, int32_t dim);
void hann_knn_free(hann_knn* h);
/* Message of the calling thread's last failed hann_knn_* call, also after
 * a hann_knn_new that returned NULL (per thread, as hann_pqivf_last_error). */
const char* hann_knn_last_error(const hann_knn* h);
/* Host buffers: queries [nq][dim], ids [nq][k], dist [nq][k]. */
int hann_knn_search(hann_knn* h, int32_t metric, const float* queries, int64_t nq, int32_t k, int32_t method,
                    int64_t* ids, double* dist);
/* Device buffers, work enqueued on `stream` (a cudaStream_t; NULL = the
 * handle's own); returns once the results are complete. */
int hann_knn_search_device(hann_knn* h, int32_t metric, const float* queries, int64_t nq, int32_t k, int32_t method,
                           int64_t* ids, double* dist, void* stream);
int hann_knn_get_stats(hann_knn* h, hann_knn_stats* out);
/* Appends n rows [n][dim] (host) to the handle's base; they get the next
 * row numbers. For indexes whose points arrive over time (hnsw Add,
 * rpt Add). */
int hann_knn_append(hann_knn* h, const float* rows, int64_t n);
/* Gathered distances for graph and tree indexes: Metric.RankBatch over many
 * (query, candidate list) pairs at once. The reference ranks candidates one
 * Rank call at a time (hnsw/index.go:1178 in the greedy descent and
 * searchLayer, rpt/index.go:461 over a leaf's ids). For query q (queries
 * [nq][dim]) and every j in [offsets[q], offsets[q + 1]) (offsets [nq + 1],
 * starting at 0, never decreasing): out[j] = distance(queries[q],
 * base[ids[j]]), the value hann_gpu_distance_batch gives for that pair (FP32
 * in the reference's NEON order, widened to double). A Metric's Rank maps
 * to the metric whose distance equals it (Euclidean's Rank: squared
 * Euclidean). An id outside [0, n) fails with HANN_E_INVALID. Host buffers. */
int hann_knn_distance_gather(hann_knn* h, int32_t metric, const float* queries, int64_t nq, const int64_t* offsets,
                             const int32_t* ids, double* out);
/* The same with device buffers (total = offsets[nq] pairs), work enqueued on
 * `stream` (NULL = the handle's own); returns once the results are
 * complete. */
int hann_knn_distance_gather_device(hann_knn* h, int32_t metric, const float* d_queries, int64_t nq,
                                    const int64_t* d_offsets, const int32_t* d_ids, int64_t total, double* d_out,
                                    void* stream);
/* One-shot form: copies base, searches, frees. */
int hann_gpu_knn(int32_t metric, const float* queries, int64_t nq, const float* base, int64_t n, int32_t dim,
                 int32_t k, int32_t method, int64_t* ids, double* dist);

#ifdef __cplusplus
}
#endif

#endif /* HANN_GB300_H */
