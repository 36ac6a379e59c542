// snapshot.cu -- binary snapshot of a PQIVF index: the live state written
// and read as flat arrays, for indexes (10M rows and more) where the gob
// stream of Save/Load (pqivf/index.go:969-1101) is slow to build.
//
// Layout (little-endian, no padding):
//   char[8]  "HANNGBS1"
//   u32      version (1), u32 0
//   i32 x 10 dimension, coarse_k, num_subquantizers, pq_k, kmeans_iters,
//            candidate_clusters, fallback, trained, nlist, pq_k_eff
//   i32 x 2  rerank, plain_fp32
//   u64      seed
//   i64 x 2  n_rows (entries in lists), n_pending
//   f32      coarse [nlist][dim]
//   f32      codebooks [M][pq_k_eff][dim / M]
//   i64      list_len [nlist] (live entries of each list)
//   u8       list_key [nlist]
//   i64      cluster_counts [nlist]
//   i64      ids [n_rows] (list by list, in storage order)
//   f32      vectors [n_rows][dim]
//   u8       codes [n_rows][M]
//   i64      pending_ids [n_pending] (ascending)
//   f32      pending_vectors [n_pending][dim]
//   u64      checksum of every byte before it
//   char[8]  "HANNGBSE"
// The same content as the gob stream (rows in the same order), with codes
// as bytes. Loading checks the sizes against the file length before it
// allocates anything and the checksum before it changes the index.
#include <cstdio>

#include "index_internal.h"

namespace {

constexpr char MAGIC[8] = {'H', 'A', 'N', 'N', 'G', 'B', 'S', '1'};
constexpr char MAGIC_END[8] = {'H', 'A', 'N', 'N', 'G', 'B', 'S', 'E'};
constexpr uint32_t VERSION = 1;

// Streaming 64-bit checksum: four multiply-rotate lanes over 8-byte words
// (32 bytes per round), a zero-padded tail and the length folded in at the
// end. Detects truncation and corruption; not a cryptographic hash.
struct Checksum {
    static constexpr uint64_t P1 = 0x9E3779B97F4A7C15ull, P2 = 0xC2B2AE3D27D4EB4Full;
    uint64_t h[4] = {0x243F6A8885A308D3ull, 0x13198A2E03707344ull, 0xA4093822299F31D0ull, 0x082EFA98EC4E6C89ull};
    unsigned char buf[32];
    size_t nb = 0;
    uint64_t total = 0;
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    void round(const unsigned char* b) {
        for (int i = 0; i < 4; i++) {
            uint64_t w;
            std::memcpy(&w, b + 8 * i, 8);
            h[i] = rotl(h[i] ^ (w * P2), 31) * P1;
        }
    }
    void add(const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        total += n;
        if (nb) {
            const size_t t = std::min(n, 32 - nb);
            std::memcpy(buf + nb, c, t);
            nb += t;
            c += t;
            n -= t;
            if (nb < 32) return;
            round(buf);
            nb = 0;
        }
        for (; n >= 32; c += 32, n -= 32) round(c);
        std::memcpy(buf, c, n);
        nb = n;
    }
    uint64_t value() const {
        uint64_t hh[4] = {h[0], h[1], h[2], h[3]};
        if (nb) {
            unsigned char b[32] = {};
            std::memcpy(b, buf, nb);
            for (int i = 0; i < 4; i++) {
                uint64_t w;
                std::memcpy(&w, b + 8 * i, 8);
                hh[i] = rotl(hh[i] ^ (w * P2), 31) * P1;
            }
        }
        uint64_t x = total * P1;
        for (int i = 0; i < 4; i++) {
            x = (x ^ rotl(hh[i], 7 * i + 11)) * P2;
            x ^= x >> 29;
        }
        return x;
    }
};

struct Header {
    int32_t dimension, coarse_k, num_subquantizers, pq_k, kmeans_iters, candidate_clusters, fallback, trained, nlist,
        pq_k_eff;
    int32_t rerank, plain_fp32;
    uint64_t seed;
    int64_t n_rows, n_pending;
};

struct Writer {
    FILE* f = nullptr;
    Checksum ck;
    bool ok = true;
    void put(const void* p, size_t n) {
        if (!ok || n == 0) return;
        ck.add(p, n);
        ok = std::fwrite(p, 1, n, f) == n;
    }
};

struct Reader {
    FILE* f = nullptr;
    Checksum ck;
    bool ok = true;
    void get(void* p, size_t n) {
        if (!ok || n == 0) return;
        ok = std::fread(p, 1, n, f) == n;
        if (ok) ck.add(p, n);
    }
};

// a * b when it stays below 2^62, else -1
int64_t mul_checked(int64_t a, int64_t b) {
    if (a < 0 || b < 0) return -1;
    if (a != 0 && b > ((int64_t)1 << 62) / a) return -1;
    return a * b;
}

}  // namespace

extern "C" {

int hann_pqivf_save_snapshot(hann_pqivf* h, const char* path) {
    if (!h || !path) return HANN_E_INVALID;
    // writers wait; searches go on (the snapshot only reads)
    std::lock_guard<std::mutex> wl(h->wmu);
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    Header hd{};
    hd.dimension = dim;
    hd.coarse_k = h->o.coarse_k;
    hd.num_subquantizers = M;
    hd.pq_k = h->o.pq_k;
    hd.kmeans_iters = h->o.kmeans_iters;
    hd.candidate_clusters = h->o.candidate_clusters;
    hd.fallback = h->o.fallback;
    hd.trained = h->trained ? 1 : 0;
    hd.nlist = h->nlist;
    hd.pq_k_eff = h->pqk_eff;
    hd.rerank = h->o.rerank;
    hd.plain_fp32 = h->o.plain_fp32;
    hd.seed = h->o.seed;
    hd.n_rows = h->total_rows();
    hd.n_pending = (int64_t)h->pending.size();

    // live rows in list order: their storage slots and ids
    std::vector<int64_t> src, ids, list_len(h->nlist);
    src.reserve((size_t)hd.n_rows);
    ids.reserve((size_t)hd.n_rows);
    for (int l = 0; l < h->nlist; l++) {
        list_len[l] = h->live_count[l];
        for (size_t j = 0; j < h->list_ids[l].size(); j++)
            if (h->list_alive[l][j]) {
                src.push_back(h->h_start[l] + (int64_t)j);
                ids.push_back(h->list_ids[l][j]);
            }
    }
    if ((int64_t)src.size() != hd.n_rows) return h->fail(HANN_E_STATE, "row bookkeeping out of step");

    Writer w;
    w.f = std::fopen(path, "wb");
    if (!w.f) return h->fail(HANN_E_INVALID, "cannot open %s for writing", path);
    const uint32_t ver[2] = {VERSION, 0};
    w.put(MAGIC, 8);
    w.put(ver, sizeof(ver));
    w.put(&hd, sizeof(hd));
    w.put(h->h_coarse.data(), sizeof(float) * (size_t)h->nlist * dim);
    w.put(h->h_codebooks.data(), sizeof(float) * h->h_codebooks.size());
    w.put(list_len.data(), sizeof(int64_t) * list_len.size());
    w.put(h->list_key.data(), h->list_key.size());
    w.put(h->cluster_counts.data(), sizeof(int64_t) * h->cluster_counts.size());
    w.put(ids.data(), sizeof(int64_t) * ids.size());

    // vectors, then codes: gathered on the device a chunk of rows at a time
    // into pinned memory and written out
    const int64_t n = hd.n_rows;
    const int64_t CH = (int64_t)1 << 18;
    const int cw = h->code_stride / 4;
    int rc = HANN_OK;
    if (n > 0) {
        DBuf<int64_t> dsrc;
        DBuf<float> dv;
        float* hv = nullptr;
        std::vector<uint8_t> packed;
        cudaError_t e = dsrc.reserve((size_t)std::min(n, CH));
        if (e == cudaSuccess) e = dv.reserve((size_t)std::min(n, CH) * std::max(dim, cw));
        if (e == cudaSuccess) e = cudaMallocHost(&hv, sizeof(float) * (size_t)std::min(n, CH) * std::max(dim, cw));
        for (int pass = 0; pass < 2 && e == cudaSuccess && w.ok; pass++) {
            for (int64_t r0 = 0; r0 < n && e == cudaSuccess && w.ok; r0 += CH) {
                const int64_t c = std::min(CH, n - r0);
                const int words = pass == 0 ? dim : cw;
                e = cudaMemcpyAsync(dsrc.p, src.data() + r0, sizeof(int64_t) * c, cudaMemcpyHostToDevice, h->stream);
                if (e == cudaSuccess)
                    e = launch_copy_words(pass == 0 ? (const void*)h->d_vectors.p : (const void*)h->d_codes.p,
                                          dsrc.p, dv.p, nullptr, c, words, h->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(hv, dv.p, sizeof(float) * c * words, cudaMemcpyDeviceToHost, h->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
                if (e != cudaSuccess) break;
                if (pass == 0) {
                    w.put(hv, sizeof(float) * c * dim);
                } else {
                    packed.resize((size_t)c * M);
                    const uint8_t* cb = reinterpret_cast<const uint8_t*>(hv);
                    for (int64_t i = 0; i < c; i++) std::memcpy(&packed[i * M], cb + i * h->code_stride, M);
                    w.put(packed.data(), packed.size());
                }
            }
        }
        if (hv) cudaFreeHost(hv);
        if (e != cudaSuccess) rc = h->cuda_fail(e, "snapshot gather");
    }
    if (rc == HANN_OK) {
        const std::vector<int64_t> pid = h->pending.sorted_ids();
        w.put(pid.data(), sizeof(int64_t) * pid.size());
        for (int64_t id : pid) w.put(h->pending.find(id), sizeof(float) * dim);
        const uint64_t sum = w.ck.value();
        if (w.ok) w.ok = std::fwrite(&sum, 8, 1, w.f) == 1 && std::fwrite(MAGIC_END, 1, 8, w.f) == 8;
        if (!w.ok) rc = h->fail(HANN_E_INVALID, "write to %s failed", path);
    }
    if (std::fclose(w.f) != 0 && rc == HANN_OK) rc = h->fail(HANN_E_INVALID, "write to %s failed", path);
    return rc;
}

int hann_pqivf_load_snapshot(hann_pqivf* h, const char* path) {
    if (!h || !path) return HANN_E_INVALID;
    Reader r;
    r.f = std::fopen(path, "rb");
    if (!r.f) return h->fail(HANN_E_INVALID, "cannot open %s", path);
    struct Closer {
        FILE* f;
        ~Closer() { std::fclose(f); }
    } closer{r.f};
    std::fseek(r.f, 0, SEEK_END);
    const int64_t fsize = (int64_t)std::ftell(r.f);
    std::fseek(r.f, 0, SEEK_SET);
    char magic[8];
    uint32_t ver[2];
    Header hd{};
    r.get(magic, 8);
    r.get(ver, sizeof(ver));
    r.get(&hd, sizeof(hd));
    if (!r.ok || std::memcmp(magic, MAGIC, 8) != 0) return h->fail(HANN_E_INVALID, "%s is not an index snapshot", path);
    if (ver[0] != VERSION) return h->fail(HANN_E_UNSUPPORTED, "snapshot version %u (this build reads %u)", ver[0], VERSION);
    const int64_t dim = hd.dimension, M = hd.num_subquantizers, nl = hd.nlist, kq = hd.pq_k_eff;
    if (dim <= 0 || M <= 0 || dim % M != 0 || nl < 0 || kq < 0 || kq > 256 || hd.n_rows < 0 || hd.n_pending < 0)
        return h->fail(HANN_E_INVALID, "snapshot header is inconsistent");
    // every section's size, checked against the file before allocating
    const int64_t parts[] = {mul_checked(nl, dim * 4), mul_checked(mul_checked(M, kq), (dim / M) * 4), nl * 8, nl,
                             nl * 8, mul_checked(hd.n_rows, 8), mul_checked(hd.n_rows, dim * 4),
                             mul_checked(hd.n_rows, M), mul_checked(hd.n_pending, 8),
                             mul_checked(hd.n_pending, dim * 4)};
    int64_t expect = 8 + (int64_t)sizeof(ver) + (int64_t)sizeof(hd) + 16;
    for (int64_t v : parts) {
        if (v < 0 || expect > ((int64_t)1 << 62) - v) return h->fail(HANN_E_INVALID, "snapshot header is inconsistent");
        expect += v;
    }
    if (expect != fsize)
        return h->fail(HANN_E_INVALID, "snapshot %s has %lld bytes, its header describes %lld", path, (long long)fsize,
                       (long long)expect);
    std::vector<float> coarse((size_t)(nl * dim)), codebooks((size_t)(M * kq * (dim / M)));
    std::vector<int64_t> list_len((size_t)nl), counts((size_t)nl), ids((size_t)hd.n_rows),
        pending_ids((size_t)hd.n_pending);
    std::vector<uint8_t> list_key((size_t)nl), codes((size_t)(hd.n_rows * M));
    std::vector<float> vectors((size_t)(hd.n_rows * dim)), pending((size_t)(hd.n_pending * dim));
    r.get(coarse.data(), coarse.size() * 4);
    r.get(codebooks.data(), codebooks.size() * 4);
    r.get(list_len.data(), list_len.size() * 8);
    r.get(list_key.data(), list_key.size());
    r.get(counts.data(), counts.size() * 8);
    r.get(ids.data(), ids.size() * 8);
    r.get(vectors.data(), vectors.size() * 4);
    r.get(codes.data(), codes.size());
    r.get(pending_ids.data(), pending_ids.size() * 8);
    r.get(pending.data(), pending.size() * 4);
    const uint64_t sum = r.ck.value();
    uint64_t stored = 0;
    char tail[8];
    if (!r.ok || std::fread(&stored, 8, 1, r.f) != 1 || std::fread(tail, 1, 8, r.f) != 8 ||
        std::memcmp(tail, MAGIC_END, 8) != 0)
        return h->fail(HANN_E_INVALID, "snapshot %s is truncated", path);
    if (stored != sum) return h->fail(HANN_E_INVALID, "snapshot %s fails its checksum", path);
    int64_t tot = 0;
    for (int64_t v : list_len) {
        if (v < 0) return h->fail(HANN_E_INVALID, "snapshot list lengths are inconsistent");
        tot += v;
    }
    if (tot != hd.n_rows) return h->fail(HANN_E_INVALID, "snapshot list lengths are inconsistent");

    hann_pqivf_layout L{};
    L.dimension = hd.dimension;
    L.coarse_k = hd.coarse_k;
    L.num_subquantizers = hd.num_subquantizers;
    L.pq_k = hd.pq_k;
    L.kmeans_iters = hd.kmeans_iters;
    L.candidate_clusters = hd.candidate_clusters;
    L.fallback = hd.fallback;
    L.trained = hd.trained;
    L.nlist = hd.nlist;
    L.pq_k_eff = hd.pq_k_eff;
    L.n_rows = hd.n_rows;
    L.n_pending = hd.n_pending;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    {
        cudaError_t e = wait_device_searches(h);
        if (e != cudaSuccess) return h->cuda_fail(e, "waiting for device searches");
    }
    h->o.seed = hd.seed;
    h->rng.seed(hd.seed);
    h->o.rerank = hd.rerank;
    h->o.plain_fp32 = hd.plain_fp32;
    return import_locked(h, &L, coarse.data(), codebooks.data(), list_len.data(), list_key.data(), counts.data(),
                         ids.data(), vectors.data(), nullptr, codes.data(), nullptr, pending_ids.data(),
                         pending.data());
}

}  // extern "C"
