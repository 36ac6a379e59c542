// index.cu -- the PQIVF index behind the C ABI (include/hann_gb300.h).
//
// Host-side state mirrors the reference's pqivf.Index (pqivf/index.go:36-54):
// pending vectors before Train, the id -> cluster map, per-list id order, the
// ClusterCounts map and the list-map key set. Everything the kernels read
// lives in HBM in structure-of-arrays form, one row per stored vector:
//   codes  [rows][code_stride] uint8   PQ codes (M bytes, padded to 4)
//   term   [rows] f32                  ||r||^2 + 2<c, r> of the decoded residual
//   vectors[rows][dim] f32             raw vectors (exact rerank, re-Train)
//   row_id [rows] i64, row_cluster [rows] i32
// Rows of one inverted list are contiguous; every list starts on a multiple
// of 32 rows and keeps spare capacity so Adds append in place.
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

struct hann_pqivf {
    hann_pqivf_options o{};
    int dsub = 0, code_stride = 0;
    std::shared_mutex mu;
    std::mutex run_mu;
    std::string err;
    cudaStream_t stream = nullptr;
    Rng rng;
    bool trained = false;
    std::atomic<int64_t> fallback_searches{0};

    std::unordered_map<int64_t, std::vector<float>> pending;

    int nlist = 0, pqk_eff = 0;
    std::vector<float> h_coarse, h_codebooks;
    std::vector<std::vector<int64_t>> list_ids;
    std::vector<uint8_t> list_key;
    std::vector<int64_t> cluster_counts;
    std::unordered_map<int64_t, int32_t> id_cluster;
    std::vector<int64_t> h_start, h_cap;
    int64_t rows_cap = 0;

    DBuf<float> d_coarse, d_codebooks, d_vectors, d_term;
    DBuf<int64_t> d_start, d_row_id;
    DBuf<int32_t> d_len, d_row_cluster;
    DBuf<uint8_t> d_codes;

    // search scratch
    DBuf<float> s_q, s_D, s_probe_d, s_cand_d;
    DBuf<int32_t> s_probe_ids, s_fb, s_cand_row, s_k, s_np, s_nout;
    DBuf<uint32_t> s_cand_seq;
    DBuf<int64_t> s_ids;
    DBuf<double> s_dist;
    DBuf<unsigned long long> s_fbcount, s_rows;

    // stage profiling: pairs of events per stage
    bool profile = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[4];
    int64_t launches = 0;

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(e == cudaErrorMemoryAllocation ? HANN_E_NOMEM : HANN_E_CUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    int64_t total_rows() const {
        int64_t t = 0;
        for (const auto& l : list_ids) t += (int64_t)l.size();
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
        p.list_start = d_start.p;
        p.list_len = d_len.p;
        p.codes = d_codes.p;
        p.term = d_term.p;
        p.row_cluster = d_row_cluster.p;
        p.vectors = d_vectors.p;
        p.row_id = d_row_id.p;
        return p;
    }
};

static thread_local std::string g_new_error;

#define CK(expr)                                          \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return h->cuda_fail(_e, #expr); \
    } while (0)

template <typename T>
static cudaError_t upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s) {
    cudaError_t e = b.reserve(n);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    return cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

static int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Capacity for a list that must hold `len` rows.
static int64_t list_capacity(int64_t len) { return round_up(len + len / 8 + 32, 32); }

// ---------------------------------------------------------------------------
// Device layout management.

// Lays the lists out afresh with capacities caps[], moving the live rows.
static int relayout(hann_pqivf* h, const std::vector<int64_t>& caps) {
    const int dim = h->o.dimension;
    std::vector<int64_t> start(h->nlist);
    int64_t total = 0;
    for (int l = 0; l < h->nlist; l++) {
        start[l] = total;
        total += round_up(caps[l], 32);
    }
    if (total >= (int64_t)1 << 31) return h->fail(HANN_E_UNSUPPORTED, "more than 2^31 stored rows");
    DBuf<float> vec, term;
    DBuf<int64_t> rid;
    DBuf<int32_t> rcl;
    DBuf<uint8_t> codes;
    CK(vec.reserve((size_t)total * dim));
    CK(term.reserve((size_t)total));
    CK(rid.reserve((size_t)total));
    CK(rcl.reserve((size_t)total));
    CK(codes.reserve((size_t)total * h->code_stride));
    if (h->rows_cap > 0) {
        std::vector<int64_t> src, dst;
        for (int l = 0; l < h->nlist; l++) {
            const int64_t len = (int64_t)h->list_ids[l].size();
            for (int64_t j = 0; j < len; j++) {
                src.push_back(h->h_start[l] + j);
                dst.push_back(start[l] + j);
            }
        }
        DBuf<int64_t> dsrc, ddst;
        CK(upload(dsrc, src.data(), src.size(), h->stream));
        CK(upload(ddst, dst.data(), dst.size(), h->stream));
        const int64_t n = (int64_t)src.size();
        CK(launch_copy_words(h->d_vectors.p, dsrc.p, vec.p, ddst.p, n, dim, h->stream));
        CK(launch_copy_words(h->d_term.p, dsrc.p, term.p, ddst.p, n, 1, h->stream));
        CK(launch_copy_words(h->d_row_id.p, dsrc.p, rid.p, ddst.p, n, 2, h->stream));
        CK(launch_copy_words(h->d_row_cluster.p, dsrc.p, rcl.p, ddst.p, n, 1, h->stream));
        CK(launch_copy_words(h->d_codes.p, dsrc.p, codes.p, ddst.p, n, h->code_stride / 4, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    h->d_vectors.swap(vec);
    h->d_term.swap(term);
    h->d_row_id.swap(rid);
    h->d_row_cluster.swap(rcl);
    h->d_codes.swap(codes);
    h->h_start = start;
    h->h_cap.assign(h->nlist, 0);
    for (int l = 0; l < h->nlist; l++) h->h_cap[l] = round_up(caps[l], 32);
    h->rows_cap = total;
    CK(upload(h->d_start, h->h_start.data(), h->h_start.size(), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

static int upload_lens(hann_pqivf* h) {
    std::vector<int32_t> len(h->nlist);
    for (int l = 0; l < h->nlist; l++) len[l] = (int32_t)h->list_ids[l].size();
    CK(upload(h->d_len, len.data(), len.size(), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

// Places n vectors (ids ascending, host memory) into a trained index:
// nearest coarse list, codes, append (assignLocked, pqivf/index.go:245-260).
static int assign_batch(hann_pqivf* h, const int64_t* ids, const float* vecs, int64_t n) {
    if (n <= 0) return HANN_OK;
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    DBuf<float> x, term;
    DBuf<int32_t> asg;
    DBuf<uint8_t> codes;
    CK(upload(x, vecs, (size_t)n * dim, h->stream));
    CK(asg.reserve((size_t)n));
    CK(term.reserve((size_t)n));
    CK(codes.reserve((size_t)n * h->code_stride));
    DBuf<unsigned long long> keys;
    CK(keys.reserve((size_t)n));
    CK(launch_assign_exact(x.p, n, dim, h->d_coarse.p, h->nlist, asg.p, nullptr, keys.p, h->stream));
    CK(launch_encode(x.p, nullptr, asg.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, h->pqk_eff, codes.p,
                     h->code_stride, term.p, h->stream));
    std::vector<int32_t> hasg((size_t)n);
    CK(cudaMemcpyAsync(hasg.data(), asg.p, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::vector<int64_t> need(h->nlist);
    bool grow = false;
    for (int l = 0; l < h->nlist; l++) need[l] = (int64_t)h->list_ids[l].size();
    for (int64_t i = 0; i < n; i++) need[hasg[i]]++;
    std::vector<int64_t> caps(h->nlist);
    for (int l = 0; l < h->nlist; l++) {
        caps[l] = h->h_cap[l];
        if (need[l] > h->h_cap[l]) {
            caps[l] = list_capacity(need[l] + need[l] / 2);
            grow = true;
        }
    }
    if (grow) {
        int rc = relayout(h, caps);
        if (rc) return rc;
    }
    std::vector<int64_t> dst((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const int c = hasg[i];
        dst[i] = h->h_start[c] + (int64_t)h->list_ids[c].size();
        h->list_ids[c].push_back(ids[i]);
        h->id_cluster[ids[i]] = c;
        h->cluster_counts[c]++;
        h->list_key[c] = 1;
    }
    DBuf<int64_t> ddst, did;
    CK(upload(ddst, dst.data(), dst.size(), h->stream));
    CK(upload(did, ids, (size_t)n, h->stream));
    CK(launch_copy_words(x.p, nullptr, h->d_vectors.p, ddst.p, n, dim, h->stream));
    CK(launch_copy_words(term.p, nullptr, h->d_term.p, ddst.p, n, 1, h->stream));
    CK(launch_copy_words(did.p, nullptr, h->d_row_id.p, ddst.p, n, 2, h->stream));
    CK(launch_copy_words(asg.p, nullptr, h->d_row_cluster.p, ddst.p, n, 1, h->stream));
    CK(launch_copy_words(codes.p, nullptr, h->d_codes.p, ddst.p, n, h->code_stride / 4, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return upload_lens(h);
}

// Removes the given (already validated, trained-side) ids from their lists,
// keeping every list's order (deleteLocked, pqivf/index.go:313-345).
static int remove_rows(hann_pqivf* h, const std::vector<int64_t>& ids) {
    if (ids.empty()) return HANN_OK;
    std::unordered_map<int, std::unordered_set<int64_t>> by_list;
    for (int64_t id : ids) {
        auto it = h->id_cluster.find(id);
        if (it == h->id_cluster.end()) continue;
        by_list[it->second].insert(id);
    }
    std::vector<int64_t> src, dst;
    for (auto& kv : by_list) {
        const int l = kv.first;
        auto& lst = h->list_ids[l];
        std::vector<int64_t> kept;
        kept.reserve(lst.size());
        int64_t w = 0;
        for (size_t j = 0; j < lst.size(); j++) {
            if (kv.second.count(lst[j])) {
                h->cluster_counts[l]--;
                h->id_cluster.erase(lst[j]);
                continue;
            }
            if ((int64_t)j != w) {
                src.push_back(h->h_start[l] + (int64_t)j);
                dst.push_back(h->h_start[l] + w);
            }
            kept.push_back(lst[j]);
            w++;
        }
        lst.swap(kept);
    }
    if (!src.empty()) {
        // Stage through a temporary so overlapping moves stay correct.
        const int dim = h->o.dimension;
        const int64_t n = (int64_t)src.size();
        DBuf<int64_t> dsrc, ddst;
        CK(upload(dsrc, src.data(), src.size(), h->stream));
        CK(upload(ddst, dst.data(), dst.size(), h->stream));
        DBuf<uint32_t> tmp;
        const int widths[5] = {dim, 1, 2, 1, h->code_stride / 4};
        void* arrs[5] = {h->d_vectors.p, h->d_term.p, h->d_row_id.p, h->d_row_cluster.p, h->d_codes.p};
        CK(tmp.reserve((size_t)n * std::max(dim, h->code_stride / 4 + 2)));
        for (int a = 0; a < 5; a++) {
            CK(launch_copy_words(arrs[a], dsrc.p, tmp.p, nullptr, n, widths[a], h->stream));
            CK(launch_copy_words(tmp.p, nullptr, arrs[a], ddst.p, n, widths[a], h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
    }
    return upload_lens(h);
}

// ---------------------------------------------------------------------------
// Train (pqivf/index.go:451-605) on the device.

struct SeedSource {
    const int64_t* coarse_init = nullptr;
    const int64_t* pq_init = nullptr;
    const int64_t* reseed = nullptr;
    int64_t n_reseed = 0;
    int64_t reseed_used = 0;
};

static int64_t draw_reseed(hann_pqivf* h, SeedSource& src, int64_t n, bool& ok) {
    ok = true;
    if (src.reseed) {
        if (src.reseed_used >= src.n_reseed) {
            ok = false;
            return 0;
        }
        const int64_t v = src.reseed[src.reseed_used++];
        if (v < 0 || v >= n) ok = false;
        return v;
    }
    return h->rng.intn(n);
}

// Lloyd iterations over rows of x (n x dim) into cent (k x dim), as runKMeans
// (pqivf/index.go:795-847): init rows given, FP64 sums, FP32 mean, empty
// clusters reseeded from `reseed` in cluster order.
static int kmeans_device(hann_pqivf* h, const float* x, int64_t ld, int off, int64_t n, int dim, int k, int iters,
                         const std::vector<int64_t>& init, SeedSource& seeds, float* cent, int32_t* asg_buf,
                         bool sub_mode, const float* sub_full, int M, int m) {
    // sub_mode: x is the full residual matrix [n][M*dim]; k-means runs on
    // columns [m*dim, (m+1)*dim) and cent is codebook m ([k][dim]).
    DBuf<int64_t> dsrc;
    DBuf<double> sums;
    DBuf<int64_t> counts;
    CK(upload(dsrc, init.data(), init.size(), h->stream));
    CK(launch_gather_cols(x, ld, off, dsrc.p, nullptr, k, dim, cent, dim, h->stream));
    CK(sums.reserve((size_t)k * dim * (sub_mode ? M : 1)));
    CK(counts.reserve((size_t)k * (sub_mode ? M : 1)));
    std::vector<int64_t> hcounts(k);
    for (int it = 0; it < iters; it++) {
        if (!sub_mode) {
            CK(launch_assign_exact(x, n, dim, cent, k, asg_buf, nullptr, nullptr, h->stream));
            CK(cudaMemsetAsync(sums.p, 0, (size_t)k * dim * sizeof(double), h->stream));
            CK(cudaMemsetAsync(counts.p, 0, (size_t)k * sizeof(int64_t), h->stream));
            CK(launch_kmeans_accumulate(x, n, dim, asg_buf, sums.p, counts.p, h->stream));
            CK(launch_kmeans_finalize(sums.p, counts.p, k, dim, cent, h->stream));
            CK(cudaMemcpyAsync(hcounts.data(), counts.p, (size_t)k * sizeof(int64_t), cudaMemcpyDeviceToHost,
                               h->stream));
        } else {
            // cent points at codebook m inside the [M][k][dim] codebook array.
            const float* cb_all = cent - (int64_t)m * k * dim;
            CK(launch_pq_assign(sub_full, n, M, dim, cb_all, k, m, m + 1, asg_buf, h->stream));
            CK(cudaMemsetAsync(sums.p + (size_t)m * k * dim, 0, (size_t)k * dim * sizeof(double), h->stream));
            CK(cudaMemsetAsync(counts.p + (size_t)m * k, 0, (size_t)k * sizeof(int64_t), h->stream));
            CK(launch_pq_accumulate(sub_full, n, M, dim, asg_buf, k, m, m + 1, sums.p, counts.p, h->stream));
            CK(launch_kmeans_finalize(sums.p + (size_t)m * k * dim, counts.p + (size_t)m * k, k, dim, cent,
                                      h->stream));
            CK(cudaMemcpyAsync(hcounts.data(), counts.p + (size_t)m * k, (size_t)k * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        std::vector<int64_t> rs;
        std::vector<int32_t> rd;
        for (int c = 0; c < k; c++) {
            if (hcounts[c] == 0) {
                bool ok;
                const int64_t r = draw_reseed(h, seeds, n, ok);
                if (!ok) return h->fail(HANN_E_INVALID, "reseed index stream exhausted or out of range");
                rs.push_back(r);
                rd.push_back(c);
            }
        }
        if (!rs.empty()) {
            DBuf<int64_t> drs;
            DBuf<int32_t> drd;
            CK(upload(drs, rs.data(), rs.size(), h->stream));
            CK(upload(drd, rd.data(), rd.size(), h->stream));
            CK(launch_gather_cols(x, ld, off, drs.p, drd.p, (int64_t)rs.size(), dim, cent, dim, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
    }
    return HANN_OK;
}

static int train_impl(hann_pqivf* h, SeedSource seeds) {
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    // Consolidate every vector, clustered and pending, in ascending id order.
    std::vector<std::pair<int64_t, int64_t>> all;  // (id, source)
    all.reserve(h->id_cluster.size() + h->pending.size());
    for (int l = 0; l < h->nlist; l++)
        for (size_t j = 0; j < h->list_ids[l].size(); j++)
            all.emplace_back(h->list_ids[l][j], h->h_start[l] + (int64_t)j);
    std::vector<const std::vector<float>*> pend;
    for (auto& kv : h->pending) {
        all.emplace_back(kv.first, -(int64_t)pend.size() - 1);
        pend.push_back(&kv.second);
    }
    const int64_t n = (int64_t)all.size();
    if (n < h->o.coarse_k)
        return h->fail(HANN_E_STATE, "not enough vectors (%lld) to train coarse quantizer with %d clusters",
                       (long long)n, h->o.coarse_k);
    if (n >= (int64_t)1 << 31) return h->fail(HANN_E_UNSUPPORTED, "more than 2^31 vectors");
    std::sort(all.begin(), all.end());
    std::vector<int64_t> ids(n), src(n);
    for (int64_t i = 0; i < n; i++) {
        ids[i] = all[i].first;
        src[i] = all[i].second;
    }
    std::vector<float> staging(pend.size() * (size_t)dim);
    for (size_t i = 0; i < pend.size(); i++) std::memcpy(&staging[i * dim], pend[i]->data(), sizeof(float) * dim);
    DBuf<float> X, dstage;
    DBuf<int64_t> dsrc;
    CK(X.reserve((size_t)n * dim));
    CK(upload(dstage, staging.data(), staging.size(), h->stream));
    CK(upload(dsrc, src.data(), src.size(), h->stream));
    CK(launch_gather2(h->d_vectors.p ? h->d_vectors.p : X.p, dstage.p, dsrc.p, n, dim, X.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    staging.clear();
    staging.shrink_to_fit();

    // Coarse k-means (runKMeans(allVectors, coarseK, iters)).
    const int k = (int)std::min<int64_t>(h->o.coarse_k, n);
    std::vector<int64_t> init;
    if (seeds.coarse_init) {
        init.assign(seeds.coarse_init, seeds.coarse_init + k);
        for (int64_t v : init)
            if (v < 0 || v >= n) return h->fail(HANN_E_INVALID, "coarse init index out of range");
    } else {
        init = h->rng.perm_prefix(n, k);
    }
    DBuf<float> C;
    DBuf<int32_t> asg;
    CK(C.reserve((size_t)k * dim));
    CK(asg.reserve((size_t)n));
    int rc = kmeans_device(h, X.p, dim, 0, n, dim, k, h->o.kmeans_iters, init, seeds, C.p, asg.p, false, nullptr, 0,
                           0);
    if (rc) return rc;
    // Final assignment and inverted lists in ascending (cluster, id) order.
    CK(launch_assign_exact(X.p, n, dim, C.p, k, asg.p, nullptr, nullptr, h->stream));
    std::vector<int32_t> hasg(n);
    CK(cudaMemcpyAsync(hasg.data(), asg.p, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::vector<int64_t> cnt(k, 0);
    for (int64_t i = 0; i < n; i++) cnt[hasg[i]]++;
    std::vector<int64_t> off(k + 1, 0);
    for (int c = 0; c < k; c++) off[c + 1] = off[c] + cnt[c];
    std::vector<int64_t> order(n);  // list-order position -> X row
    {
        std::vector<int64_t> fill(off.begin(), off.end() - 1);
        for (int64_t i = 0; i < n; i++) order[fill[hasg[i]]++] = i;
    }
    std::vector<int32_t> ord_cluster(n);
    for (int64_t j = 0; j < n; j++) ord_cluster[j] = hasg[order[j]];

    // Residuals in list order feed the subquantizer k-means.
    DBuf<int64_t> dorder;
    DBuf<int32_t> dordc;
    DBuf<float> Rm;
    CK(upload(dorder, order.data(), order.size(), h->stream));
    CK(upload(dordc, ord_cluster.data(), ord_cluster.size(), h->stream));
    CK(Rm.reserve((size_t)n * dim));
    CK(launch_residuals(X.p, dorder.p, dordc.p, n, dim, C.p, Rm.p, h->stream));
    const int kpq = (int)std::min<int64_t>(h->o.pq_k, n);
    const int ds = dim / M;
    DBuf<float> CB;
    CK(CB.reserve((size_t)M * kpq * ds));
    DBuf<int32_t> pqa;
    CK(pqa.reserve((size_t)n * M));
    for (int m = 0; m < M; m++) {
        std::vector<int64_t> pinit;
        if (seeds.pq_init) {
            pinit.assign(seeds.pq_init + (int64_t)m * h->o.pq_k, seeds.pq_init + (int64_t)m * h->o.pq_k + kpq);
            for (int64_t v : pinit)
                if (v < 0 || v >= n) return h->fail(HANN_E_INVALID, "subquantizer init index out of range");
        } else {
            pinit = h->rng.perm_prefix(n, kpq);
        }
        rc = kmeans_device(h, Rm.p, dim, m * ds, n, ds, kpq, h->o.kmeans_iters, pinit, seeds,
                           CB.p + (size_t)m * kpq * ds, pqa.p, true, Rm.p, M, m);
        if (rc) return rc;
    }
    Rm.reset();

    // New layout and state.
    h->nlist = k;
    h->pqk_eff = kpq;
    h->list_ids.assign(k, {});
    h->list_key.assign(k, 0);
    h->cluster_counts.assign(k, 0);
    h->id_cluster.clear();
    for (int64_t j = 0; j < n; j++) {
        const int c = ord_cluster[j];
        h->list_ids[c].push_back(ids[order[j]]);
        h->id_cluster[ids[order[j]]] = c;
    }
    for (int c = 0; c < k; c++) {
        h->cluster_counts[c] = cnt[c];
        h->list_key[c] = cnt[c] > 0;
    }
    h->d_coarse.swap(C);
    h->d_codebooks.swap(CB);
    h->d_vectors.reset();
    h->d_term.reset();
    h->d_row_id.reset();
    h->d_row_cluster.reset();
    h->d_codes.reset();
    h->rows_cap = 0;
    std::vector<int64_t> caps(k);
    for (int c = 0; c < k; c++) caps[c] = list_capacity(cnt[c]);
    // relayout() with rows_cap == 0 only allocates.
    std::vector<std::vector<int64_t>> saved;
    saved.swap(h->list_ids);
    h->list_ids.assign(k, {});
    rc = relayout(h, caps);
    h->list_ids.swap(saved);
    if (rc) return rc;
    std::vector<int64_t> dst(n), rid(n);
    std::vector<int32_t> rcl(n);
    {
        std::vector<int64_t> fill(k, 0);
        for (int64_t j = 0; j < n; j++) {
            const int c = ord_cluster[j];
            dst[j] = h->h_start[c] + fill[c]++;
            rid[j] = ids[order[j]];
            rcl[j] = c;
        }
    }
    DBuf<int64_t> ddst, drid;
    DBuf<int32_t> drcl;
    CK(upload(ddst, dst.data(), dst.size(), h->stream));
    CK(upload(drid, rid.data(), rid.size(), h->stream));
    CK(upload(drcl, rcl.data(), rcl.size(), h->stream));
    CK(launch_copy_words(X.p, dorder.p, h->d_vectors.p, ddst.p, n, dim, h->stream));
    CK(launch_copy_words(drid.p, nullptr, h->d_row_id.p, ddst.p, n, 2, h->stream));
    CK(launch_copy_words(drcl.p, nullptr, h->d_row_cluster.p, ddst.p, n, 1, h->stream));
    CK(launch_encode(h->d_vectors.p, ddst.p, h->d_row_cluster.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, kpq,
                     h->d_codes.p, h->code_stride, h->d_term.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->h_coarse.resize((size_t)k * dim);
    h->h_codebooks.resize((size_t)M * kpq * ds);
    CK(cudaMemcpy(h->h_coarse.data(), h->d_coarse.p, h->h_coarse.size() * sizeof(float), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->h_codebooks.data(), h->d_codebooks.p, h->h_codebooks.size() * sizeof(float),
                  cudaMemcpyDeviceToHost));
    h->pending.clear();
    h->trained = true;
    return upload_lens(h);
}

// ---------------------------------------------------------------------------
// Search.

static int rerank_depth(const hann_pqivf* h, int kmax, int mode) {
    if (h->o.rerank > 0) return std::max(h->o.rerank, kmax);
    const int r = mode == 0 ? kmax + 32 : std::max(4 * kmax, 64);
    return (int)round_up(r, 32);
}

// Runs the device search for nq queries already in d_q; k/nprobe per query
// in device arrays d_k/d_np. Outputs to device buffers.
static int run_search(hann_pqivf* h, const float* d_q, int64_t nq, const int32_t* d_k, const int32_t* d_np,
                      int np_max, int kmax, int mode, int64_t* d_ids, double* d_dist, int32_t* d_nout,
                      cudaStream_t s) {
    const int R = rerank_depth(h, kmax, mode);
    if (R > 480) return h->fail(HANN_E_UNSUPPORTED, "k (%d) above this build's limit of 448", kmax);
    np_max = std::min(np_max, h->nlist);
    if (np_max > 4096) return h->fail(HANN_E_UNSUPPORTED, "more than 4096 probed lists per query");
    const ScanParams p = h->scan_params();
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nq, ((int64_t)1 << 28) / std::max(1, h->nlist)));
    CK(h->s_D.reserve((size_t)chunk * h->nlist));
    CK(h->s_probe_ids.reserve((size_t)chunk * np_max));
    CK(h->s_probe_d.reserve((size_t)chunk * np_max));
    CK(h->s_fb.reserve((size_t)chunk));
    CK(h->s_cand_row.reserve((size_t)chunk * R));
    CK(h->s_cand_d.reserve((size_t)chunk * R));
    CK(h->s_cand_seq.reserve((size_t)chunk * R));
    auto mark = [&](int stage, bool begin) -> cudaError_t {
        if (!h->profile) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        if (begin) h->ev[stage].push_back({e, nullptr});
        else h->ev[stage].back().second = e;
        return cudaEventRecord(e, s);
    };
    for (int64_t q0 = 0; q0 < nq; q0 += chunk) {
        const int64_t nc = std::min(chunk, nq - q0);
        const float* qp = d_q + q0 * h->o.dimension;
        CK(mark(0, true));
        CK(launch_dist_matrix(qp, nc, h->o.dimension, h->d_coarse.p, h->nlist, h->s_D.p, s));
        CK(mark(0, false));
        CK(mark(1, true));
        CK(launch_probe_select(h->s_D.p, nc, h->nlist, d_np + q0, np_max, d_k + q0, h->d_len.p,
                               h->o.fallback ? 1 : 0, h->s_probe_ids.p, h->s_probe_d.p, h->s_fb.p,
                               h->s_fbcount.p, s));
        CK(mark(1, false));
        CK(mark(2, true));
        CK(launch_scan(p, qp, nc, h->s_probe_ids.p, h->s_D.p, d_np + q0, np_max, h->s_fb.p, R, h->s_cand_row.p,
                       h->s_cand_d.p, h->s_cand_seq.p, h->profile ? h->s_rows.p : nullptr, s));
        CK(mark(2, false));
        CK(mark(3, true));
        CK(launch_rerank(p, qp, nc, h->s_cand_row.p, h->s_cand_seq.p, R, d_k + q0, kmax, mode, d_ids + q0 * kmax,
                         d_dist + q0 * kmax, d_nout + q0, s));
        CK(mark(3, false));
        h->launches += 4;
    }
    return HANN_OK;
}

static int check_searchable(hann_pqivf* h) {
    if (!h->trained)
        return h->fail(HANN_E_STATE, "PQIVF index is not trained. Call Train() after adding data before searching");
    bool any = false;
    for (uint8_t b : h->list_key) any |= b != 0;
    if (!any) return h->fail(HANN_E_STATE, "index is empty");
    return HANN_OK;
}

static int read_fallbacks(hann_pqivf* h, cudaStream_t s) {
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, h->s_fbcount.p, sizeof(v), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->fallback_searches += (int64_t)v;
    return HANN_OK;
}

// ---------------------------------------------------------------------------
// C ABI.

extern "C" {

void hann_pqivf_options_init(hann_pqivf_options* o, int32_t dimension) {
    std::memset(o, 0, sizeof(*o));
    o->dimension = dimension;
    o->coarse_k = 16;
    o->pq_k = 16;
    o->kmeans_iters = 10;
    o->candidate_clusters = 3;
    o->fallback = 1;
    o->seed = 0x68616e6eull;
    o->device = 0;
    o->rerank = 0;
    int m = 1;
    for (int c : {8, 4, 2})
        if (dimension > 0 && dimension % c == 0) {
            m = c;
            break;
        }
    o->num_subquantizers = m;
}

int hann_pqivf_new(const hann_pqivf_options* opts, hann_pqivf** out) {
    char buf[256];
    auto bad = [&](int code) {
        g_new_error = buf;
        return code;
    };
    if (!opts || !out) {
        snprintf(buf, sizeof(buf), "null argument");
        return bad(HANN_E_INVALID);
    }
    const hann_pqivf_options& o = *opts;
    if (o.dimension <= 0) {
        snprintf(buf, sizeof(buf), "dimension (%d) must be positive", o.dimension);
        return bad(HANN_E_INVALID);
    }
    if (o.coarse_k <= 0) {
        snprintf(buf, sizeof(buf), "coarseK (%d) must be positive", o.coarse_k);
        return bad(HANN_E_INVALID);
    }
    if (o.pq_k <= 0) {
        snprintf(buf, sizeof(buf), "pqK (%d) must be positive", o.pq_k);
        return bad(HANN_E_INVALID);
    }
    if (o.kmeans_iters <= 0) {
        snprintf(buf, sizeof(buf), "kMeansIters (%d) must be positive", o.kmeans_iters);
        return bad(HANN_E_INVALID);
    }
    if (o.num_subquantizers <= 0) {
        snprintf(buf, sizeof(buf), "numSubquantizers (%d) must be positive", o.num_subquantizers);
        return bad(HANN_E_INVALID);
    }
    if (o.dimension % o.num_subquantizers != 0) {
        snprintf(buf, sizeof(buf), "dimension (%d) must be divisible by numSubquantizers (%d)", o.dimension,
                 o.num_subquantizers);
        return bad(HANN_E_INVALID);
    }
    if (o.pq_k > 256) {
        snprintf(buf, sizeof(buf), "pqK (%d) above 256: this build stores one-byte codes", o.pq_k);
        return bad(HANN_E_UNSUPPORTED);
    }
    hann_pqivf* h = new (std::nothrow) hann_pqivf();
    if (!h) {
        snprintf(buf, sizeof(buf), "out of host memory");
        return bad(HANN_E_NOMEM);
    }
    h->o = o;
    h->dsub = o.dimension / o.num_subquantizers;
    h->code_stride = (int)round_up(o.num_subquantizers, 4);
    h->rng.seed(o.seed);
    cudaError_t e = cudaSetDevice(o.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = h->s_fbcount.reserve(1);
    if (e == cudaSuccess) e = h->s_rows.reserve(1);
    if (e == cudaSuccess) e = cudaMemset(h->s_rows.p, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        snprintf(buf, sizeof(buf), "CUDA initialisation failed: %s", cudaGetErrorString(e));
        delete h;
        return bad(HANN_E_CUDA);
    }
    *out = h;
    return HANN_OK;
}

void hann_pqivf_free(hann_pqivf* h) {
    if (!h) return;
    cudaSetDevice(h->o.device);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    delete h;
}

const char* hann_pqivf_last_error(const hann_pqivf* h) { return h ? h->err.c_str() : g_new_error.c_str(); }

int hann_pqivf_bulk_add(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && (!ids || !vectors))) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    const int dim = h->o.dimension;
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
    // First failing position in ascending id order; everything before it is
    // applied, as the reference's loop does (pqivf/index.go:276-296).
    int64_t f = n;
    int code = HANN_OK;
    std::string msg;
    for (int64_t i = 0; i < n; i++) {
        const int64_t id = ids[order[i]];
        const bool dup_prev = i > 0 && ids[order[i - 1]] == id;
        if (h->id_cluster.count(id) || (dup_prev && h->trained)) {
            f = i;
            code = HANN_E_EXISTS;
            msg = "id " + std::to_string(id) + " already exists in a cluster";
            break;
        }
        if (h->pending.count(id) || dup_prev) {
            f = i;
            code = HANN_E_EXISTS;
            msg = "id " + std::to_string(id) + " already exists in pending vectors";
            break;
        }
    }
    if (!h->trained) {
        for (int64_t i = 0; i < f; i++) {
            const int64_t r = order[i];
            h->pending[ids[r]] = std::vector<float>(vectors + r * dim, vectors + (r + 1) * dim);
        }
    } else if (f > 0) {
        std::vector<int64_t> sid(f);
        std::vector<float> sv((size_t)f * dim);
        for (int64_t i = 0; i < f; i++) {
            sid[i] = ids[order[i]];
            std::memcpy(&sv[(size_t)i * dim], vectors + order[i] * dim, sizeof(float) * dim);
        }
        int rc = assign_batch(h, sid.data(), sv.data(), f);
        if (rc) return rc;
    }
    if (code) return h->fail(code, "%s", msg.c_str());
    return HANN_OK;
}

int hann_pqivf_add(hann_pqivf* h, int64_t id, const float* vector) { return hann_pqivf_bulk_add(h, &id, vector, 1); }

// Deletes in the given order; `strict` stops at the first unknown id.
static int delete_ids(hann_pqivf* h, std::vector<int64_t> ids, bool strict) {
    std::vector<int64_t> trained_side;
    std::unordered_set<int64_t> seen;
    for (int64_t id : ids) {
        auto pit = h->pending.find(id);
        if (pit != h->pending.end()) {
            h->pending.erase(pit);
            continue;
        }
        if (!h->id_cluster.count(id) || seen.count(id)) {
            if (strict) {
                int rc = remove_rows(h, trained_side);
                if (rc) return rc;
                return h->fail(HANN_E_NOT_FOUND, "id %lld not found", (long long)id);
            }
            continue;
        }
        seen.insert(id);
        trained_side.push_back(id);
    }
    return remove_rows(h, trained_side);
}

int hann_pqivf_delete(hann_pqivf* h, int64_t id) {
    if (!h) return HANN_E_INVALID;
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    return delete_ids(h, {id}, true);
}

int hann_pqivf_bulk_delete(hann_pqivf* h, const int64_t* ids, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && !ids)) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    std::vector<int64_t> v(ids, ids + n);
    std::sort(v.begin(), v.end());
    return delete_ids(h, v, false);
}

int hann_pqivf_bulk_update(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && (!ids || !vectors))) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    const int dim = h->o.dimension;
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
    // Delete-then-add per id in ascending order; the first id that is not
    // present stops the batch (pqivf/index.go:435-442).
    int64_t f = n;
    for (int64_t i = 0; i < n; i++) {
        const int64_t id = ids[order[i]];
        const bool present = h->pending.count(id) || h->id_cluster.count(id);
        const bool dup_prev = i > 0 && ids[order[i - 1]] == id;
        if (!present && !dup_prev) {
            f = i;
            break;
        }
    }
    // Apply the updates before f. A repeated id updates twice, the last wins.
    std::vector<int64_t> del;
    for (int64_t i = 0; i < f; i++) del.push_back(ids[order[i]]);
    std::vector<int64_t> last_pos;
    for (int64_t i = 0; i < f; i++)
        if (i + 1 == f || ids[order[i + 1]] != ids[order[i]]) last_pos.push_back(order[i]);
    int rc = delete_ids(h, del, false);
    if (rc) return rc;
    if (!h->trained) {
        for (int64_t r : last_pos) h->pending[ids[r]] = std::vector<float>(vectors + r * dim, vectors + (r + 1) * dim);
    } else if (!last_pos.empty()) {
        std::vector<int64_t> sid;
        std::vector<float> sv;
        for (int64_t r : last_pos) {
            sid.push_back(ids[r]);
            sv.insert(sv.end(), vectors + r * dim, vectors + (r + 1) * dim);
        }
        rc = assign_batch(h, sid.data(), sv.data(), (int64_t)sid.size());
        if (rc) return rc;
    }
    if (f < n) return h->fail(HANN_E_NOT_FOUND, "id %lld not found", (long long)ids[order[f]]);
    return HANN_OK;
}

int hann_pqivf_update(hann_pqivf* h, int64_t id, const float* vector) {
    return hann_pqivf_bulk_update(h, &id, vector, 1);
}

int hann_pqivf_train_seeded(hann_pqivf* h, const int64_t* coarse_init, const int64_t* pq_init, const int64_t* reseed,
                            int64_t n_reseed) {
    if (!h) return HANN_E_INVALID;
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    SeedSource s;
    s.coarse_init = coarse_init;
    s.pq_init = pq_init;
    s.reseed = reseed;
    s.n_reseed = n_reseed;
    return train_impl(h, s);
}

int hann_pqivf_train(hann_pqivf* h) { return hann_pqivf_train_seeded(h, nullptr, nullptr, nullptr, 0); }

int hann_pqivf_search_batch(hann_pqivf* h, const float* queries, int64_t nq, const int32_t* k, const int32_t* nprobe,
                            int32_t kmax, int32_t mode, int64_t* ids, double* distances, int32_t* n_out) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (nq < 0 || (nq > 0 && (!queries || !k || !ids || !distances || !n_out)))
        return h->fail(HANN_E_INVALID, "invalid arguments");
    for (int64_t i = 0; i < nq; i++)
        if (k[i] <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    for (int64_t i = 0; i < nq; i++)
        if (k[i] > kmax) return h->fail(HANN_E_INVALID, "k (%d) above kmax (%d)", k[i], kmax);
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq == 0) return HANN_OK;
    std::vector<int32_t> np(nq);
    int np_max = 1;
    for (int64_t i = 0; i < nq; i++) {
        np[i] = nprobe ? nprobe[i] : h->o.candidate_clusters;
        if (np[i] <= 0) return h->fail(HANN_E_INVALID, "nprobe must be positive");
        np[i] = std::min(np[i], h->nlist);
        np_max = std::max(np_max, np[i]);
    }
    cudaStream_t s = h->stream;
    CK(upload(h->s_q, queries, (size_t)nq * h->o.dimension, s));
    CK(upload(h->s_k, k, (size_t)nq, s));
    CK(upload(h->s_np, np.data(), (size_t)nq, s));
    CK(h->s_ids.reserve((size_t)nq * kmax));
    CK(h->s_dist.reserve((size_t)nq * kmax));
    CK(h->s_nout.reserve((size_t)nq));
    CK(cudaMemsetAsync(h->s_fbcount.p, 0, sizeof(unsigned long long), s));
    rc = run_search(h, h->s_q.p, nq, h->s_k.p, h->s_np.p, np_max, kmax, mode, h->s_ids.p, h->s_dist.p, h->s_nout.p,
                    s);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ids, h->s_ids.p, (size_t)nq * kmax * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(distances, h->s_dist.p, (size_t)nq * kmax * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(n_out, h->s_nout.p, (size_t)nq * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    return read_fallbacks(h, s);
}

int hann_pqivf_search(hann_pqivf* h, const float* query, int32_t k, int64_t* ids, double* distances,
                      int32_t* n_out) {
    if (!h) return HANN_E_INVALID;
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    return hann_pqivf_search_batch(h, query, 1, &k, nullptr, k, 0, ids, distances, n_out);
}

int hann_pqivf_search_batch_device(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k, int32_t nprobe,
                                   int32_t mode, int64_t* d_ids, double* d_distances, int32_t* d_n_out,
                                   void* stream) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (nprobe <= 0) nprobe = h->o.candidate_clusters;
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq <= 0) return HANN_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const int np = std::min<int>(nprobe, h->nlist);
    if ((int64_t)h->s_k.n < nq || h->s_k.p == nullptr) {
        std::vector<int32_t> kv(nq, k), nv(nq, np);
        CK(upload(h->s_k, kv.data(), kv.size(), s));
        CK(upload(h->s_np, nv.data(), nv.size(), s));
        CK(cudaStreamSynchronize(s));
    } else {
        std::vector<int32_t> kv(nq, k), nv(nq, np);
        CK(cudaMemcpyAsync(h->s_k.p, kv.data(), nq * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(h->s_np.p, nv.data(), nq * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    return run_search(h, d_queries, nq, h->s_k.p, h->s_np.p, np, k, mode, d_ids, d_distances, d_n_out, s);
}

int hann_pqivf_set_profiling(hann_pqivf* h, int32_t on) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> rl(h->run_mu);
    h->profile = on != 0;
    return HANN_OK;
}

int hann_pqivf_stage_times(hann_pqivf* h, double* ms4, int64_t* launches, int64_t* rows_scanned) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    for (int st = 0; st < 4; st++) {
        double tot = 0.0;
        for (auto& pr : h->ev[st]) {
            if (pr.second) {
                CK(cudaEventSynchronize(pr.second));
                float ms = 0.0f;
                CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
                tot += ms;
                cudaEventDestroy(pr.second);
            }
            cudaEventDestroy(pr.first);
        }
        h->ev[st].clear();
        if (ms4) ms4[st] = tot;
    }
    if (launches) *launches = h->launches;
    h->launches = 0;
    unsigned long long rows = 0;
    CK(cudaMemcpy(&rows, h->s_rows.p, sizeof(rows), cudaMemcpyDeviceToHost));
    CK(cudaMemset(h->s_rows.p, 0, sizeof(rows)));
    if (rows_scanned) *rows_scanned = (int64_t)rows;
    return HANN_OK;
}

int hann_pqivf_list_lengths(hann_pqivf* h, int64_t* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    for (int l = 0; l < h->nlist; l++) out[l] = (int64_t)h->list_ids[l].size();
    return HANN_OK;
}

int hann_pqivf_stats(hann_pqivf* h, hann_pqivf_index_stats* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    out->count = (int64_t)h->pending.size() + h->total_rows();
    out->dimension = h->o.dimension;
    out->fallback_searches = h->fallback_searches.load();
    out->trained = h->trained ? 1 : 0;
    out->nlist = h->nlist;
    out->rows_capacity = h->rows_cap;
    return HANN_OK;
}

int hann_pqivf_export_layout(hann_pqivf* h, hann_pqivf_layout* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    out->dimension = h->o.dimension;
    out->coarse_k = h->o.coarse_k;
    out->num_subquantizers = h->o.num_subquantizers;
    out->pq_k = h->o.pq_k;
    out->kmeans_iters = h->o.kmeans_iters;
    out->candidate_clusters = h->o.candidate_clusters;
    out->fallback = h->o.fallback;
    out->trained = h->trained;
    out->nlist = h->nlist;
    out->pq_k_eff = h->pqk_eff;
    out->n_rows = h->total_rows();
    out->n_pending = (int64_t)h->pending.size();
    return HANN_OK;
}

int hann_pqivf_export(hann_pqivf* h, float* coarse, float* codebooks, int64_t* list_len, uint8_t* list_key,
                      int64_t* cluster_counts, int64_t* ids, float* vectors, int32_t* codes, int64_t* pending_ids,
                      float* pending_vectors) {
    if (!h) return HANN_E_INVALID;
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    if (h->nlist > 0) {
        std::memcpy(coarse, h->h_coarse.data(), h->h_coarse.size() * sizeof(float));
        std::memcpy(codebooks, h->h_codebooks.data(), h->h_codebooks.size() * sizeof(float));
    }
    int64_t r = 0;
    std::vector<uint8_t> cbuf;
    for (int l = 0; l < h->nlist; l++) {
        const int64_t len = (int64_t)h->list_ids[l].size();
        list_len[l] = len;
        list_key[l] = h->list_key[l];
        cluster_counts[l] = h->cluster_counts[l];
        if (len == 0) continue;
        std::memcpy(ids + r, h->list_ids[l].data(), len * sizeof(int64_t));
        CK(cudaMemcpy(vectors + r * dim, h->d_vectors.p + h->h_start[l] * dim, (size_t)len * dim * sizeof(float),
                      cudaMemcpyDeviceToHost));
        cbuf.resize((size_t)len * h->code_stride);
        CK(cudaMemcpy(cbuf.data(), h->d_codes.p + h->h_start[l] * h->code_stride, cbuf.size(),
                      cudaMemcpyDeviceToHost));
        for (int64_t j = 0; j < len; j++)
            for (int m = 0; m < M; m++) codes[(r + j) * M + m] = cbuf[(size_t)j * h->code_stride + m];
        r += len;
    }
    // Pending vectors in ascending id order.
    std::vector<int64_t> pid;
    for (auto& kv : h->pending) pid.push_back(kv.first);
    std::sort(pid.begin(), pid.end());
    for (size_t i = 0; i < pid.size(); i++) {
        pending_ids[i] = pid[i];
        std::memcpy(pending_vectors + i * dim, h->pending[pid[i]].data(), sizeof(float) * dim);
    }
    return HANN_OK;
}

int hann_pqivf_import(hann_pqivf* h, const hann_pqivf_layout* L, const float* coarse, const float* codebooks,
                      const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                      const int64_t* ids, const float* vectors, const int32_t* codes, const uint8_t* has_codes,
                      const int64_t* pending_ids, const float* pending_vectors) {
    if (!h || !L) return HANN_E_INVALID;
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    // GobDecode's parameter checks (pqivf/index.go:1035-1045).
    if (L->dimension <= 0) return h->fail(HANN_E_INVALID, "serialized index has invalid dimension %d", L->dimension);
    if (L->num_subquantizers <= 0 || L->dimension % L->num_subquantizers != 0)
        return h->fail(HANN_E_INVALID, "serialized index has invalid subquantizer count %d for dimension %d",
                       L->num_subquantizers, L->dimension);
    if (L->coarse_k <= 0 || L->pq_k <= 0 || L->kmeans_iters <= 0)
        return h->fail(HANN_E_INVALID,
                       "serialized index has invalid training parameters: coarseK %d, pqK %d, kMeansIters %d",
                       L->coarse_k, L->pq_k, L->kmeans_iters);
    if (L->pq_k_eff > 256 || L->pq_k > 256)
        return h->fail(HANN_E_UNSUPPORTED, "pqK above 256: this build stores one-byte codes");
    if (L->n_rows > 0 && (L->nlist <= 0 || L->pq_k_eff <= 0))
        return h->fail(HANN_E_UNSUPPORTED, "entries without centroids or codebooks");
    h->o.dimension = L->dimension;
    h->o.coarse_k = L->coarse_k;
    h->o.num_subquantizers = L->num_subquantizers;
    h->o.pq_k = L->pq_k;
    h->o.kmeans_iters = L->kmeans_iters;
    if (L->candidate_clusters > 0) h->o.candidate_clusters = L->candidate_clusters;
    h->o.fallback = L->fallback;
    h->dsub = L->dimension / L->num_subquantizers;
    h->code_stride = (int)round_up(L->num_subquantizers, 4);
    const int dim = L->dimension, M = L->num_subquantizers;
    h->trained = L->trained != 0;
    h->pending.clear();
    for (int64_t i = 0; i < L->n_pending; i++)
        h->pending[pending_ids[i]] = std::vector<float>(pending_vectors + i * dim, pending_vectors + (i + 1) * dim);
    h->nlist = L->nlist;
    h->pqk_eff = L->pq_k_eff;
    h->h_coarse.assign(coarse, coarse + (size_t)L->nlist * dim);
    h->h_codebooks.assign(codebooks, codebooks + (size_t)M * L->pq_k_eff * h->dsub);
    h->list_ids.assign(h->nlist, {});
    h->list_key.assign(h->nlist, 0);
    h->cluster_counts.assign(h->nlist, 0);
    h->id_cluster.clear();
    int64_t r = 0;
    for (int l = 0; l < h->nlist; l++) {
        h->list_key[l] = list_key[l];
        h->cluster_counts[l] = cluster_counts[l];
        for (int64_t j = 0; j < list_len[l]; j++, r++) {
            h->list_ids[l].push_back(ids[r]);
            h->id_cluster[ids[r]] = l;
        }
    }
    h->d_vectors.reset();
    h->d_term.reset();
    h->d_row_id.reset();
    h->d_row_cluster.reset();
    h->d_codes.reset();
    h->d_coarse.reset();
    h->d_codebooks.reset();
    h->rows_cap = 0;
    h->h_start.assign(h->nlist, 0);
    h->h_cap.assign(h->nlist, 0);
    if (h->nlist == 0) return HANN_OK;
    CK(upload(h->d_coarse, h->h_coarse.data(), h->h_coarse.size(), h->stream));
    CK(upload(h->d_codebooks, h->h_codebooks.data(), h->h_codebooks.size(), h->stream));
    std::vector<int64_t> caps(h->nlist);
    for (int l = 0; l < h->nlist; l++) caps[l] = list_capacity(list_len[l]);
    std::vector<std::vector<int64_t>> saved;
    saved.swap(h->list_ids);
    h->list_ids.assign(h->nlist, {});
    int rc = relayout(h, caps);
    h->list_ids.swap(saved);
    if (rc) return rc;
    const int64_t n = L->n_rows;
    if (n == 0) return upload_lens(h);
    std::vector<int64_t> dst(n), recode;
    std::vector<int32_t> rcl(n);
    std::vector<uint8_t> cbytes((size_t)n * h->code_stride, 0);
    r = 0;
    for (int l = 0; l < h->nlist; l++)
        for (int64_t j = 0; j < list_len[l]; j++, r++) {
            dst[r] = h->h_start[l] + j;
            rcl[r] = l;
            bool ok = has_codes == nullptr || has_codes[r];
            for (int m = 0; ok && m < M; m++) {
                const int32_t c = codes[r * M + m];
                if (c < 0 || c >= h->pqk_eff) ok = false;
                else cbytes[(size_t)r * h->code_stride + m] = (uint8_t)c;
            }
            if (!ok) recode.push_back(dst[r]);
        }
    DBuf<int64_t> ddst, did;
    DBuf<int32_t> drcl;
    DBuf<float> dvec;
    DBuf<uint8_t> dcodes;
    CK(upload(ddst, dst.data(), dst.size(), h->stream));
    CK(upload(did, ids, (size_t)n, h->stream));
    CK(upload(drcl, rcl.data(), rcl.size(), h->stream));
    CK(upload(dvec, vectors, (size_t)n * dim, h->stream));
    CK(upload(dcodes, cbytes.data(), cbytes.size(), h->stream));
    CK(launch_copy_words(dvec.p, nullptr, h->d_vectors.p, ddst.p, n, dim, h->stream));
    CK(launch_copy_words(did.p, nullptr, h->d_row_id.p, ddst.p, n, 2, h->stream));
    CK(launch_copy_words(drcl.p, nullptr, h->d_row_cluster.p, ddst.p, n, 1, h->stream));
    CK(launch_copy_words(dcodes.p, nullptr, h->d_codes.p, ddst.p, n, h->code_stride / 4, h->stream));
    CK(launch_term(h->d_codes.p, ddst.p, h->d_row_cluster.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, h->pqk_eff,
                   h->code_stride, h->d_term.p, h->stream));
    if (!recode.empty()) {
        DBuf<int64_t> drec;
        CK(upload(drec, recode.data(), recode.size(), h->stream));
        CK(launch_encode(h->d_vectors.p, drec.p, h->d_row_cluster.p, (int64_t)recode.size(), dim, h->d_coarse.p,
                         h->d_codebooks.p, M, h->pqk_eff, h->d_codes.p, h->code_stride, h->d_term.p, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return upload_lens(h);
}

int hann_gpu_distance_batch(int32_t metric, const float* query, const float* flat, size_t dim, size_t n,
                            double* out) {
    if (metric < 0 || metric > 3) return HANN_E_INVALID;
    if (n == 0) return HANN_OK;
    if (dim == 0) {
        for (size_t i = 0; i < n; i++) out[i] = 0.0;
        return HANN_OK;
    }
    DBuf<float> dq, dx;
    DBuf<double> dout;
    if (upload(dq, query, dim, nullptr) != cudaSuccess || upload(dx, flat, dim * n, nullptr) != cudaSuccess ||
        dout.reserve(n) != cudaSuccess)
        return HANN_E_CUDA;
    if (launch_distance_rows(metric, dq.p, dx.p, (int)dim, (int64_t)n, dout.p, nullptr) != cudaSuccess)
        return HANN_E_CUDA;
    if (cudaMemcpy(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return HANN_E_CUDA;
    return HANN_OK;
}

}  // extern "C"
// ---------------------------------------------------------------------------
// Allocation-free batch search.
//
// Some callers cannot allocate device memory at the moment they search: a
// latency-bound serving thread must not stall on the device-wide
// synchronisation that cudaMalloc/cudaFree may imply; code that records its
// launches into a CUDA graph may not call the allocator while the stream is
// being captured; and a process that fixes its device-memory budget at start
// must not grow it per request. hann_pqivf_search_batch_device_noalloc serves
// them. It runs the same kernels as hann_pqivf_search_batch_device, but every
// scratch buffer of the search (coarse distance matrix, probe lists,
// fallback flags, candidates, per-query k and nprobe, the fallback counter)
// is carved out of one fixed device array of NOALLOC_ARENA_BYTES that every
// GPU which loads this library holds until the process exits. The index's
// own arrays were allocated when it was built; the call allocates nothing.

namespace {

constexpr size_t NOALLOC_ARENA_BYTES = (size_t)16 << 20;  // 16 MiB per device
constexpr int NOALLOC_MAX_DEVICES = 64;

// Host code must not take this symbol's address directly: on the host it is
// only a stand-in. The device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_arena[NOALLOC_ARENA_BYTES];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the arena on the current device `dev`, looked up once.
cudaError_t noalloc_arena(int dev, unsigned char** out) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
    return cudaSuccess;
}

__global__ void noalloc_fill_kernel(int32_t* a, int32_t va, int32_t* b, int32_t vb, int64_t n,
                                    unsigned long long* counter) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *counter = 0ull;
    if (i < n) {
        a[i] = va;
        b[i] = vb;
    }
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

extern "C" int hann_pqivf_search_batch_device_noalloc(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k,
                                                      int32_t nprobe, int32_t mode, int64_t* d_ids,
                                                      double* d_distances, int32_t* d_n_out, void* stream) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (nprobe <= 0) nprobe = h->o.candidate_clusters;
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq <= 0) return HANN_OK;
    const int np = std::min<int>(nprobe, h->nlist);
    const int R = rerank_depth(h, k, mode);
    if (R > 480) return h->fail(HANN_E_UNSUPPORTED, "k (%d) above this build's limit of 448", k);
    if (np > 4096) return h->fail(HANN_E_UNSUPPORTED, "more than 4096 probed lists per query");
    // Scratch layout inside the arena, every region 256-byte aligned.
    const size_t b_D = align256((size_t)nq * h->nlist * sizeof(float));
    const size_t b_pid = align256((size_t)nq * np * sizeof(int32_t));
    const size_t b_pd = align256((size_t)nq * np * sizeof(float));
    const size_t b_q32 = align256((size_t)nq * sizeof(int32_t));
    const size_t b_cr = align256((size_t)nq * R * sizeof(int32_t));
    const size_t b_cd = align256((size_t)nq * R * sizeof(float));
    const size_t b_cs = align256((size_t)nq * R * sizeof(uint32_t));
    const size_t need = b_D + b_pid + b_pd + 3 * b_q32 + b_cr + b_cd + b_cs + 256;
    if (need > NOALLOC_ARENA_BYTES)
        return h->fail(HANN_E_UNSUPPORTED,
                       "allocation-free search of %lld queries needs %zu bytes of scratch, above its fixed %zu-byte "
                       "arena; split the batch (at most about %lld queries at nlist %d, nprobe %d, k %d)",
                       (long long)nq, need, NOALLOC_ARENA_BYTES,
                       (long long)(NOALLOC_ARENA_BYTES / (need / nq + 1)), h->nlist, np, k);
    unsigned char* base = nullptr;
    CK(noalloc_arena(h->o.device, &base));
    float* D = reinterpret_cast<float*>(base);
    int32_t* pid = reinterpret_cast<int32_t*>(base + b_D);
    float* pd = reinterpret_cast<float*>(base + b_D + b_pid);
    int32_t* fb = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd);
    int32_t* dk = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + b_q32);
    int32_t* dnp = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + 2 * b_q32);
    int32_t* crow = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + 3 * b_q32);
    float* cd = reinterpret_cast<float*>(base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr);
    uint32_t* cs = reinterpret_cast<uint32_t*>(base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr + b_cd);
    unsigned long long* fbc =
        reinterpret_cast<unsigned long long*>(base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr + b_cd + b_cs);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    // The arena keeps the previous call's contents: the per-query k and
    // nprobe and the fallback counter are written first; every other region
    // is fully written by the kernel that produces it before it is read.
    noalloc_fill_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(dk, k, dnp, np, nq, fbc);
    CK(cudaGetLastError());
    const ScanParams p = h->scan_params();
    CK(launch_dist_matrix(d_queries, nq, h->o.dimension, h->d_coarse.p, h->nlist, D, s));
    CK(launch_probe_select(D, nq, h->nlist, dnp, np, dk, h->d_len.p, h->o.fallback ? 1 : 0, pid, pd, fb, fbc, s));
    CK(launch_scan(p, d_queries, nq, pid, D, dnp, np, fb, R, crow, cd, cs, nullptr, s));
    CK(launch_rerank(p, d_queries, nq, crow, cs, R, dk, k, mode, d_ids, d_distances, d_n_out, s));
    return HANN_OK;
}
