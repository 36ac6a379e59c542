// index_internal.h -- the PQIVF handle shared by the library's host files
// (index.cu: the index and its C ABI; serve.cu: the batching server).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <shared_mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "hann_gb300.h"
#include "host_maps.h"
#include "common.cuh"
#include "kernels.h"

namespace hann {

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // Grows to at least cnt elements; contents are not kept.
    cudaError_t reserve(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        reset();
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(cnt, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(cnt, 1);
        else p = nullptr;
        return e;
    }
    void swap(DBuf& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
    }
};

// xoshiro256** seeded through splitmix64: the index's own seeded source for
// k-means seeding and empty-cluster reseeds (the reference's seededRand,
// pqivf/index.go:20-23).
struct Rng {
    uint64_t s[4];
    void seed(uint64_t x) {
        for (int i = 0; i < 4; i++) {
            x += 0x9e3779b97f4a7c15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            s[i] = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    int64_t intn(int64_t n) {
        const uint64_t un = (uint64_t)n;
        const uint64_t lim = UINT64_MAX - UINT64_MAX % un;
        uint64_t v;
        do v = next();
        while (v >= lim);
        return (int64_t)(v % un);
    }
    // First k entries of a uniform random permutation of [0, n).
    std::vector<int64_t> perm_prefix(int64_t n, int64_t k) {
        std::unordered_map<int64_t, int64_t> sw;
        std::vector<int64_t> out((size_t)k);
        for (int64_t i = 0; i < k; i++) {
            const int64_t j = i + intn(n - i);
            auto get = [&](int64_t a) {
                auto it = sw.find(a);
                return it == sw.end() ? a : it->second;
            };
            const int64_t vi = get(i), vj = get(j);
            out[(size_t)i] = vj;
            sw[j] = vi;
        }
        return out;
    }
};

}  // namespace hann

using namespace hann;

// Scratch of the exact nearest-centroid search, reused across k-means
// iterations.
struct AssignScratch {
    DBuf<uint16_t> xbf, cbf;
    DBuf<float> xn2, xres, cn2, cres, cmax, cand_val;
    DBuf<int32_t> cand_idx, ovf_idx;
    DBuf<int64_t> ovf_rows;
    DBuf<int> counters;  // [0] overflow rows, [1] GEMM wait errors
    DBuf<float> ovf_x, ovf_d2;
    bool x_ready = false;
    // Warm assignments (k-means after its first iteration): each row's
    // squared distance to its centroid, the centroids they were measured
    // against, and the filter's buffers (assign_rows)
    DBuf<float> d2, cent_old, shift, rthr, fcand_s;
    DBuf<float2> cterm;
    DBuf<int32_t> fcnt, fcand;
    bool warm_ok = false;     // set by k-means for the iterations of one run
    bool warm = false;        // d2 and cent_old hold the previous assignment's
    bool warm_skip = false;   // the last warm assignment overflowed: take the top-8 screen once
    int warm_k = 0;
    int64_t warm_n = 0;
    const float* warm_cent = nullptr;
};

// Scratch of Add/Delete, kept on the handle so mutations allocate nothing
// once warm (an allocator call could synchronise with searches in flight).
struct MutationScratch {
    DBuf<float> x, term;
    DBuf<int32_t> asg;
    DBuf<uint8_t> codes;
    DBuf<int64_t> dst, ids, rows;
    DBuf<int64_t> mv_src, mv_dst, mv_sw;  // list moves: old and new starts, new scan-word starts
    DBuf<int32_t> mv_len, mv_cmp;
    AssignScratch asc;
    std::vector<int32_t> hasg;
    std::vector<int64_t> add;
    int64_t n = 0;
    bool grow = false;
    bool held = false;               // prepared rows waiting for a relayout
    std::vector<int64_t> held_ids;   // their ids
};

// Device scratch of one search stream: query staging, coarse scores, probe
// lists, candidates and results. One per stream that searches concurrently.
struct SearchScratch {
    DBuf<float> q, D, probe_d, cand_d, qn2, qres;
    DBuf<uint16_t> qbf;
    DBuf<int32_t> probe_ids, fb, cand_row, k, np, nout;
    DBuf<uint32_t> cand_seq;
    DBuf<int64_t> ids;
    DBuf<double> dist;
    DBuf<unsigned long long> fbcount;
    // screened probe (band lists per query)
    DBuf<float> pe2, pasl, pthr, pcand_s;
    DBuf<int32_t> pcnt, pcand_id, plcount, pneed, ptodo;  // ptodo: rows left to the block kernels (+ count)
    DBuf<unsigned long long> pband;
    DBuf<int32_t> qorder, order_scratch;  // L2-friendly query order for scan and rerank
    // parity mode with FP16 tables: per query the scan's cut and error bound,
    // and the queries the rerank could not prove (count at credo[nq])
    DBuf<float> scut, seps;
    DBuf<int32_t> credo;
    // the table scan's candidate dump (scan_dump_bytes per query); dump_off:
    // never reserve one (a server slot sized without it must not allocate
    // one while batches run)
    DBuf<unsigned char> dump;
    bool dump_off = false;
    // list-major tensor-core scan (kernels_lms.cu)
    DBuf<uint16_t> q16;
    DBuf<float> le2, lasl, lthr, lcand_s, lpair_base, leps;
    DBuf<int32_t> lones, lzeros;  // per-query nprobe 1 and no fallback: the seeding table scan
    DBuf<int32_t> lcnt, lcand_id, llcount, lneed, ltodo, lredo, lbandk, lcounts, lcursor, ltotal, lpair_q,
        lpair_off, ln_items, litem_counter;
    DBuf<unsigned long long> lband, lstats;
    DBuf<LmsItem> litems;
};

// The list-major scan's choices: chunks of probe ranks, rows per work item,
// blocks per SM, and the smallest batch worth it. Defaults until the
// autotuner (hann_pqivf_autotune) measures better ones for the index.
struct LmsConfig {
    int enabled = 1;       // 0: every batch takes the table scan
    // Smaller batches take the table scan. 1 by default: in exact-rerank
    // mode the two scans may pass different candidates to the rerank (FP16
    // against FP32 screening at the rerank depth), so a query's result would
    // depend on the size of the batch it runs in.
    int min_queries = 1;
    // 1: each query's first threshold comes from a table scan of its nearest
    // list and every chunk appends below it; 0: the first chunk writes every
    // score of its lists (densely, no threshold yet)
    int seed = 0;
    int first = 1;         // probe ranks in the first chunk
    int growth = 32;       // each later chunk ends at growth x the previous end
    int rows_max = 1024;   // rows of one list per work item (the list-split threshold; the autotuner picked it on a 10M x 96 index)
    // Queries probing fewer lists take the table scan: below about this many
    // probes per query the table scan is faster (the autotuner measures it).
    int min_nprobe = 64;
    int ctas_per_sm = 1;   // persistent blocks per SM (one fits: the codebooks sit in shared memory)
};

// Message of the calling thread's last failed call on any handle. Kept per
// thread (as errno is) so that concurrent callers of one handle each read
// their own failure, and no thread rewrites a string another one reads.
std::string& hann_thread_error();

struct hann_pqivf {
    hann_pqivf_options o{};
    int dsub = 0, code_stride = 0;
    std::shared_mutex mu;   // searches shared, mutations exclusive
    std::mutex wmu;         // every writer; taken before mu
    std::mutex run_mu;
    MutationScratch mut;
    cudaStream_t stream = nullptr;
    Rng rng;
    bool trained = false;
    std::atomic<int64_t> fallback_searches{0};

    PendingStore pending;

    int nlist = 0, pqk_eff = 0;
    std::vector<float> h_coarse, h_codebooks;
    std::vector<std::vector<int64_t>> list_ids;     // per list, the id of every slot
    std::vector<std::vector<uint8_t>> list_alive;   // 0 for a deleted (tombstoned) slot
    std::vector<int64_t> live_count;
    int64_t dead_rows = 0;
    std::vector<uint8_t> list_key;
    std::vector<int64_t> cluster_counts;
    IdMap<int32_t> id_cluster;
    std::vector<int64_t> h_start, h_cap;
    // Row arena: lists packed from 0 up to arena_end, then free slack up to
    // rows_cap; a list that outgrows its capacity moves to the slack and
    // leaves hole_rows behind until the next full relayout. Scan-word
    // regions follow the same plan (sw_end, sw_cap).
    int64_t rows_cap = 0, arena_end = 0, hole_rows = 0, sw_end = 0, sw_cap = 0;
    int64_t list_moves = 0, full_relayouts = 0;

    DBuf<float> d_coarse, d_codebooks, d_vectors, d_term;
    DBuf<float> d_codebooks_t;  // [pqK][M][dsub], the scan's table-build layout
    // 16-bit lookup tables: centred codebooks in the table-build layout, the
    // means, each subquantizer's largest centred codeword norm and the
    // bounds on ||r|| and |term| (prepare_adc)
    DBuf<float> d_adc_cb, d_adc_mu, d_adc_rm;
    float adc_rfull = 0.0f, adc_tbound = 0.0f;
    int adc_table = 2;          // table scan's lookup tables: 0 FP32, 1 FP16, 2 fixed point (hann_pqivf_set_adc_tables)
    DBuf<unsigned long long> d_adc_redo;  // queries scanned again with FP32 tables (diagnostic)
    // BF16 copy of the coarse centroids for the tensor-core preselection
    int kp = 0;
    bool tc = false;
    DBuf<uint16_t> d_coarse_bf16;
    DBuf<float> d_coarse_norm, d_cmax;
    DBuf<float2> d_coarse_terms;  // (||c||^2, -2) per centroid, the screen's epilogue terms
    DBuf<int> d_err;
    DBuf<int64_t> d_start, d_row_id;
    DBuf<int32_t> d_len, d_live, d_row_cluster;
    DBuf<uint8_t> d_codes;
    DBuf<uint8_t> d_scanc;    // scan codes, rebuilt from the codes when rows are placed
    DBuf<int64_t> d_swstart;  // first scan-code slot of each list
    std::vector<int64_t> h_swstart;
    bool scanc_dirty = false;
    // the previous row arrays, kept for the next relayout to reuse
    DBuf<float> s_vectors, s_term;
    DBuf<int64_t> s_row_id;
    DBuf<int32_t> s_row_cluster;
    DBuf<uint8_t> s_codes;
    DBuf<uint8_t> s_scanc;

    // list-major tensor-core scan: FP16 codebooks [M][pqK][dsub], the error
    // bound's constants, the longest list (slots) and the scan's choices
    DBuf<uint16_t> d_cb16;
    LmsBound lms_bound{};
    bool lms_ok = false;
    int64_t max_list_slots = 0;
    LmsConfig lms;
    int64_t rows_decoded = 0;  // rows the list-major scan decoded, as of the last hann_pqivf_stage_times

    // search scratch of the handle's own stream
    SearchScratch main;
    DBuf<unsigned long long> s_rows;
    // Device-buffer searches (hann_pqivf_search_batch_device and its
    // allocation-free variant) return before their kernels run, on the
    // caller's stream. dev_ev is recorded after the last one's kernels; every
    // mutation waits for it before it touches a device array, so a relayout
    // cannot move rows under a scan still reading them. d_fb_dev counts their
    // brute-force fallbacks on the device; Stats adds it once the searches
    // behind dev_ev are done.
    cudaEvent_t dev_ev = nullptr;
    bool dev_pending = false;
    DBuf<unsigned long long> d_fb_dev;

    // stage profiling: pairs of events per stage (a diagnostic of the
    // handle's own calls; not meant while a server drives the handle)
    std::atomic<bool> profile{false};
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[4];
    std::atomic<int64_t> launches{0};  // kernels launched by searches (servers' threads included)
    // k-means assignments that took the warm filter, and the rows they sent
    // to the exact kernel (hann_pqivf_train_stats)
    int64_t warm_assignments = 0, warm_overflow_rows = 0;
    // wall milliseconds of the last training's phases (hann_pqivf_train_phases)
    double train_phase_ms[4] = {0, 0, 0, 0};

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        hann_thread_error() = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(e == cudaErrorMemoryAllocation ? HANN_E_NOMEM : HANN_E_CUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    int64_t total_rows() const {
        int64_t t = 0;
        for (int64_t c : live_count) t += c;
        return t;
    }
    ScanParams scan_params() const {
        ScanParams p;
        p.dim = o.dimension;
        p.M = o.num_subquantizers;
        p.dsub = dsub;
        p.pqK = pqk_eff;
        p.nlist = nlist;
        p.code_stride = code_stride;
        p.coarse = d_coarse.p;
        p.codebooks = d_codebooks.p;
        p.codebooks_t = d_codebooks_t.p;
        p.list_start = d_start.p;
        p.list_len = d_len.p;
        p.codes = d_codes.p;
        p.scanc = scan_adc_supported(o.num_subquantizers) ? d_scanc.p : nullptr;
        p.adc_cb = d_adc_cb.p;
        p.adc_mu = d_adc_mu.p;
        p.adc_rm = d_adc_rm.p;
        p.adc_rfull = adc_rfull;
        p.adc_tbound = adc_tbound;
        p.adc_table = d_adc_cb.p ? adc_table : 0;
        p.scan_cut = nullptr;
        p.scan_eps = nullptr;
        p.redo = nullptr;
        p.redo_count = nullptr;
        p.redo_total = d_adc_redo.p;
        p.qorder = nullptr;
        p.qcount = nullptr;
        p.sw_start = d_swstart.p;
        p.term = d_term.p;
        p.row_cluster = d_row_cluster.p;
        p.vectors = d_vectors.p;
        p.row_id = d_row_id.p;
        p.kq = nullptr;
        p.dump = nullptr;
        p.mode = 0;
        p.rerank_fixed = o.rerank;
        return p;
    }
};


#define CK(expr)                                          \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return h->cuda_fail(_e, #expr); \
    } while (0)

// Marks the end of a device-buffer search enqueued on stream s (shared lock
// and run_mu held).
inline cudaError_t note_device_search(hann_pqivf* h, cudaStream_t s) {
    cudaError_t e = cudaEventRecord(h->dev_ev, s);
    if (e == cudaSuccess) h->dev_pending = true;
    return e;
}

// Waits until every device-buffer search enqueued so far has finished. Called
// by mutations (exclusive lock held, so no new search is enqueued meanwhile)
// before they write or move device arrays: those searches run on callers'
// streams, which neither the handle's stream nor a synchronous copy orders.
inline cudaError_t wait_device_searches(hann_pqivf* h) {
    if (!h->dev_pending) return cudaSuccess;
    cudaError_t e = cudaEventSynchronize(h->dev_ev);
    if (e == cudaSuccess) h->dev_pending = false;
    return e;
}

template <typename T>
inline cudaError_t upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s) {
    cudaError_t e = b.reserve(n);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    return cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Search pipeline of index.cu, usable from any stream with its own scratch.
int run_search(hann_pqivf* h, SearchScratch& sc, const float* d_q, int64_t nq, const int32_t* d_k, const int32_t* d_np,
               int np_max, int kmax, int mode, int64_t* d_ids, double* d_dist, int32_t* d_nout, cudaStream_t s,
               unsigned long long* fb_counter = nullptr);
int check_searchable(hann_pqivf* h);
int reserve_search_scratch(hann_pqivf* h, SearchScratch& sc, int64_t nq, int np_max, int kmax, int mode);
int rerank_depth(const hann_pqivf* h, int kmax, int mode);
// Mutations with the writer lock held. Without allow_relayout a mutation
// that would move rows (a list overflowing, or tombstone compaction) changes
// nothing and sets *needs_relayout; the rest is safe beside running searches.
int bulk_add_locked(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n,
                    bool allow_relayout = true, bool* needs_relayout = nullptr);
int bulk_delete_locked(hann_pqivf* h, const int64_t* ids, int64_t n, bool allow_relayout = true,
                       bool* needs_relayout = nullptr);
int add_prepare(hann_pqivf* h, const int64_t* ids, const float* vecs, int64_t n);
int add_commit(hann_pqivf* h, const int64_t* ids);
bool compaction_due(const hann_pqivf* h, int64_t extra);
// k-NN handle (knn.cu) over n rows of dim floats already on the device.
struct hann_knn* knn_new_from_device(const float* d_base, int64_t n, int32_t dim, cudaStream_t s);
// Replaces the handle's state (every lock held); codes as ints (codes32) or
// bytes (codes8), M per row.
int import_locked(hann_pqivf* h, const hann_pqivf_layout* L, const float* coarse, const float* codebooks,
                  const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                  const int64_t* ids, const float* vectors, const int32_t* codes32, const uint8_t* codes8,
                  const uint8_t* has_codes, const int64_t* pending_ids, const float* pending_vectors);
