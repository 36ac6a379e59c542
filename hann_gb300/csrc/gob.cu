// gob.cu -- native Go encoding/gob codec for the PQIVF index's persisted
// form (host code only, no device calls). The reference saves an index as a
// gob stream whose one value is the *pqivf.Index GobEncoder; its bytes are a
// second gob stream holding a serializedPQIVF struct (pqivf/index.go:
// 969-984, 992-1017, 1086-1101). The encoder writes the same bytes as the
// Python codec in hann_gb300/gob.py; the decoder reads any stream of that
// shape, Go's own included, resolving struct fields by name through the
// stream's type definitions as encoding/gob does.
//
// Wire format (the published encoding/gob specification): messages are
// (uint length)(int type id)(payload); a negative id introduces a wireType
// definition; an unsigned integer is one byte below 128, else a negated
// byte count and the big-endian bytes; a signed integer folds its sign into
// bit 0; a float is its IEEE-754 float64 bits byte-reversed, sent as an
// unsigned integer; a struct is (field delta, value) pairs ended by a zero
// delta and omits zero values; a top-level non-struct value is preceded by
// a zero byte.
//
// Layout of the work: an index of 10M rows x 96 dims is ~8 GB of gob, so
// the encoder first sizes every inverted list and every block of pending
// vectors in parallel, then writes each at its offset in parallel into the
// caller's buffer; the decoder is one pass that stores rows flat.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "hann_gb300.h"

namespace {

constexpr int T_BOOL = 1, T_INT = 2, T_UINT = 3, T_FLOAT = 4, T_BYTES = 5, T_STRING = 6, T_COMPLEX = 7;
constexpr int FIRST_USER_ID = 65;
constexpr int FORMAT_VERSION = 1;
constexpr int64_t PENDING_BLOCK = 8192;

thread_local std::string g_gob_error;

inline int uint_len(uint64_t v) { return v < 0x80 ? 1 : 1 + (64 - __builtin_clzll(v) + 7) / 8; }
inline uint64_t zigzag(int64_t v) { return v < 0 ? ((~(uint64_t)v) << 1) | 1u : ((uint64_t)v) << 1; }
inline uint64_t float_word(float f) {
    const double d = (double)f;
    uint64_t bits;
    std::memcpy(&bits, &d, 8);
    return __builtin_bswap64(bits);
}

// Byte sinks: Counter sizes a part, Writer writes it, Vec grows a small part.
struct Counter {
    size_t n = 0;
    void uint(uint64_t v) { n += uint_len(v); }
    void raw(const void*, size_t k) { n += k; }
};
struct Writer {
    uint8_t* p;
    void uint(uint64_t v) {
        if (v < 0x80) {
            *p++ = (uint8_t)v;
            return;
        }
        const int k = (64 - __builtin_clzll(v) + 7) / 8;
        *p++ = (uint8_t)(256 - k);
        for (int i = k - 1; i >= 0; i--) *p++ = (uint8_t)(v >> (8 * i));
    }
    void raw(const void* s, size_t k) {
        std::memcpy(p, s, k);
        p += k;
    }
};
struct Vec {
    std::vector<uint8_t> b;
    void uint(uint64_t v) {
        uint8_t tmp[9];
        Writer w{tmp};
        w.uint(v);
        b.insert(b.end(), tmp, w.p);
    }
    void raw(const void* s, size_t k) { b.insert(b.end(), (const uint8_t*)s, (const uint8_t*)s + k); }
};

template <class S> inline void put_int(S& s, int64_t v) { s.uint(zigzag(v)); }
template <class S> inline void put_floats(S& s, const float* v, int64_t n) {
    s.uint((uint64_t)n);
    for (int64_t i = 0; i < n; i++) s.uint(float_word(v[i]));
}
template <class S> inline void put_str(S& s, const std::string& t) {
    s.uint(t.size());
    s.raw(t.data(), t.size());
}

// Runs f(i) for i in [0, n) on up to the machine's cores.
template <class F> void parallel_for(int64_t n, F f) {
    if (n <= 0) return;
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>({hw, 64, n});
    if (nt <= 1) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    auto body = [&] {
        for (int64_t i; (i = next.fetch_add(1)) < n;) f(i);
    };
    std::vector<std::thread> ts;
    for (int64_t t = 1; t < nt; t++) ts.emplace_back(body);
    body();
    for (auto& t : ts) t.join();
}

// Type definitions of the inner stream, ids 65..74 in the order the value
// first needs them: []float32, [][]float32, map[int]int, []int,
// map[int][]pqEntry, []pqEntry, pqEntry, [][][]float32, map[int][]float32,
// serializedPQIVF.
enum { T_F32S = 65, T_F32SS, T_MAPII, T_INTS, T_MAPLIST, T_ENTRIES, T_ENTRY, T_F32SSS, T_MAPIVEC, T_SER };

void put_msg(Vec& out, int64_t tid, const Vec& payload) {
    out.uint(uint_len(zigzag(tid)) + payload.b.size());
    put_int(out, tid);
    out.raw(payload.b.data(), payload.b.size());
}
void put_common(Vec& w, const std::string& name, int tid) {
    if (!name.empty()) {
        w.uint(1);
        put_str(w, name);
        w.uint(1);
    } else {
        w.uint(2);
    }
    put_int(w, tid);
    w.uint(0);
}
void def_slice(Vec& out, int tid, int elem) {
    Vec w;
    w.uint(2);  // wireType field 1: SliceT
    w.uint(1);
    put_common(w, "", tid);
    w.uint(1);
    put_int(w, elem);
    w.uint(0);
    w.uint(0);
    put_msg(out, -tid, w);
}
void def_map(Vec& out, int tid, int key, int elem) {
    Vec w;
    w.uint(4);  // wireType field 3: MapT
    w.uint(1);
    put_common(w, "", tid);
    w.uint(1);
    put_int(w, key);
    w.uint(1);
    put_int(w, elem);
    w.uint(0);
    w.uint(0);
    put_msg(out, -tid, w);
}
void def_struct(Vec& out, int tid, const std::string& name, const std::vector<std::pair<std::string, int>>& fields) {
    Vec w;
    w.uint(3);  // wireType field 2: StructT
    w.uint(1);
    put_common(w, name, tid);
    w.uint(1);
    w.uint(fields.size());
    for (auto& f : fields) {
        w.uint(1);
        put_str(w, f.first);
        w.uint(1);
        put_int(w, f.second);
        w.uint(0);
    }
    w.uint(0);
    w.uint(0);
    put_msg(out, -tid, w);
}
void def_gobencoder(Vec& out, int tid, const std::string& name) {
    Vec w;
    w.uint(5);  // wireType field 4: GobEncoderT
    w.uint(1);
    put_common(w, name, tid);
    w.uint(0);
    w.uint(0);
    put_msg(out, -tid, w);
}

struct EncodeInput {
    const hann_pqivf_layout* L;
    const float *coarse, *codebooks, *vectors, *pending_vectors;
    const int64_t *list_len, *cluster_counts, *ids, *pending_ids;
    const uint8_t* list_key;
    const int32_t* codes;
    std::vector<int64_t> list_row;    // first row of each list
    std::vector<int64_t> pend_order;  // pending entries by ascending id
};

// One inverted-list map entry: key, length, then each pqEntry struct.
template <class S> void put_list(S& s, const EncodeInput& in, int64_t c) {
    const int64_t dim = in.L->dimension, M = in.L->num_subquantizers, n = in.list_len[c];
    put_int(s, c);
    s.uint((uint64_t)n);
    for (int64_t j = 0; j < n; j++) {
        const int64_t r = in.list_row[c] + j;
        int last = -1;
        auto field = [&](int i) {
            s.uint((uint64_t)(i - last));
            last = i;
        };
        if (in.ids[r] != 0) {
            field(0);
            put_int(s, in.ids[r]);
        }
        field(1);
        put_floats(s, in.vectors + r * dim, dim);
        field(2);
        s.uint((uint64_t)M);
        for (int64_t m = 0; m < M; m++) put_int(s, in.codes[r * M + m]);
        if (c != 0) {
            field(3);
            put_int(s, c);
        }
        s.uint(0);
    }
}

template <class S> void put_pending_block(S& s, const EncodeInput& in, int64_t b) {
    const int64_t dim = in.L->dimension;
    const int64_t e = std::min<int64_t>(in.L->n_pending, (b + 1) * PENDING_BLOCK);
    for (int64_t i = b * PENDING_BLOCK; i < e; i++) {
        const int64_t p = in.pend_order[i];
        put_int(s, in.pending_ids[p]);
        put_floats(s, in.pending_vectors + p * dim, dim);
    }
}

// ---------------------------------------------------------------- decoding

struct Err {};

struct In {
    const uint8_t* p;
    size_t n, i = 0;
    In(const uint8_t* d, size_t len) : p(d), n(len) {}
    bool eof() const { return i >= n; }
    size_t left() const { return n - i; }
    uint64_t uint() {
        if (i + 9 <= n) {  // fast path: no per-byte bounds checks
            const uint8_t c = p[i++];
            if (c < 0x80) return c;
            const int k = 256 - c;
            if (k > 8) throw Err();
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
            uint64_t w;  // the next 8 bytes as a big-endian word, of which the first k count
            std::memcpy(&w, p + i, 8);
            i += k;
            return __builtin_bswap64(w) >> (64 - 8 * k);
#else
            uint64_t v = 0;
            for (int j = 0; j < k; j++) v = (v << 8) | p[i++];
            return v;
#endif
        }
        if (i >= n) throw Err();
        const uint8_t c = p[i++];
        if (c < 0x80) return c;
        const int k = 256 - c;
        if (k > 8 || (size_t)k > n - i) throw Err();
        uint64_t v = 0;
        for (int j = 0; j < k; j++) v = (v << 8) | p[i++];
        return v;
    }
    void skip_uint() {
        if (i >= n) throw Err();
        const uint8_t c = p[i++];
        if (c >= 0x80) {
            const int k = 256 - c;
            if (k > 8 || (size_t)k > n - i) throw Err();
            i += k;
        }
    }
    int64_t sint() {
        const uint64_t u = uint();
        return (u & 1) ? (int64_t)~(u >> 1) : (int64_t)(u >> 1);
    }
    float flt() {
        const uint64_t bits = __builtin_bswap64(uint());
        double d;
        std::memcpy(&d, &bits, 8);
        return (float)d;
    }
    const uint8_t* take(uint64_t k) {
        if (k > n - i) throw Err();
        const uint8_t* q = p + i;
        i += k;
        return q;
    }
    std::string str() {
        const uint64_t k = uint();
        const uint8_t* q = take(k);
        return std::string((const char*)q, (size_t)k);
    }
    // a count of elements that each take at least one byte
    uint64_t count() {
        const uint64_t k = uint();
        if (k > left()) throw Err();
        return k;
    }
};

struct WireType {
    int kind = 0;  // 1 array, 2 slice, 3 struct, 4 map, 5 encoder (gob, binary or text)
    std::string name;
    int elem = 0, key = 0;
    std::vector<std::pair<std::string, int>> fields;
};

void decode_common(In& r, std::string& name) {
    int field = -1;
    for (;;) {
        const uint64_t d = r.uint();
        if (d == 0) return;
        if (d > 2) throw Err();
        field += (int)d;
        if (field == 0) name = r.str();
        else if (field == 1) (void)r.sint();
        else throw Err();
    }
}

WireType decode_wiretype(In& r) {
    WireType wt;
    int field = -1;
    for (;;) {
        const uint64_t d = r.uint();
        if (d == 0) break;
        if (d > 7) throw Err();
        field += (int)d;
        if (field < 0 || field > 6) throw Err();
        wt.kind = field < 4 ? field + 1 : 5;
        int f = -1;
        for (;;) {
            const uint64_t dd = r.uint();
            if (dd == 0) break;
            if (dd > 3) throw Err();
            f += (int)dd;
            if (f == 0) {
                decode_common(r, wt.name);
            } else if ((wt.kind == 1 || wt.kind == 2) && f == 1) {
                wt.elem = (int)r.sint();
            } else if (wt.kind == 1 && f == 2) {
                (void)r.sint();  // array length
            } else if (wt.kind == 3 && f == 1) {
                const uint64_t nf = r.count();
                for (uint64_t j = 0; j < nf; j++) {
                    std::string fname;
                    int fid = 0, g = -1;
                    for (;;) {
                        const uint64_t ddd = r.uint();
                        if (ddd == 0) break;
                        if (ddd > 2) throw Err();
                        g += (int)ddd;
                        if (g == 0) fname = r.str();
                        else if (g == 1) fid = (int)r.sint();
                        else throw Err();
                    }
                    wt.fields.emplace_back(fname, fid);
                }
            } else if (wt.kind == 4 && f == 1) {
                wt.key = (int)r.sint();
            } else if (wt.kind == 4 && f == 2) {
                wt.elem = (int)r.sint();
            } else {
                throw Err();
            }
        }
    }
    if (wt.kind == 0) throw Err();
    return wt;
}

}  // namespace

namespace {
// An array left uninitialised on allocation (decoding fills every element).
template <class T> struct Buf {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    void alloc(size_t k) {
        p.reset(k ? new T[k] : nullptr);
        n = k;
    }
    T* data() { return p.get(); }
    const T* data() const { return p.get(); }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
};
}  // namespace

// The decoded serializedPQIVF, held between the calls that read it. Rows
// are stored flat in stream order; segs records each list map entry.
struct hann_gob_state {
    int64_t dimension = 0, coarse_k = 0, num_subquantizers = 0, pq_k = 0, kmeans_iters = 0;
    int64_t format_version = 0, candidate_clusters = 0;
    bool fallback = false, trained = false;
    bool shape_error = false;  // a centroid or codeword of the wrong length, or ragged codebooks
    std::string shape_msg;
    std::vector<float> coarse;  // coarse_rows x dimension
    int64_t coarse_rows = 0;
    std::vector<float> codebooks;  // cb_tables x cb_words x (dimension / M)
    int64_t cb_tables = 0, cb_words = 0;
    std::vector<std::pair<int64_t, int64_t>> counts;
    // one inverted-list map entry: its rows and codes in the flat arrays,
    // its byte offset in the stream, the first row whose vector has the
    // wrong length
    struct Seg {
        int64_t cluster, row, n, code, ncodes;
        size_t at;
        int64_t bad_row, bad_len;
    };
    std::vector<Seg> segs;
    // Rows of all lists, stream order. Left uninitialised where an entry is
    // malformed; such an index is rejected before the rows are read.
    Buf<int64_t> ids;
    Buf<float> vecs;       // rows x dimension, when vecs_stored
    bool vecs_stored = false;
    Buf<int64_t> ncodes;   // codes per row
    Buf<int32_t> codes;    // row after row; -1 for a value outside int32
    std::vector<int64_t> pending_ids;
    std::vector<float> pending;  // one vector of dimension floats per pending id
    int64_t bad_pending = -1;
};

namespace {

enum EntryRole { R_SKIP, R_ID, R_VEC, R_CODES, R_CLUSTER };

// Ids below 9 are gob's basic types and interface; a stream numbers its own
// types from a first user id (64 in Go's encoder, 65 in the Python codec),
// one id per type it sends, so ids stay small: a larger one is malformed.
constexpr int FIRST_DEFINABLE_ID = 9;
constexpr int MAX_TYPE_ID = 1 << 16;

struct Dec {
    std::vector<WireType> types;
    std::vector<uint8_t> known;
    void define(int tid, WireType wt) {
        if (tid < FIRST_DEFINABLE_ID || tid > MAX_TYPE_ID) throw Err();
        if ((size_t)tid >= types.size()) {
            types.resize(tid + 1);
            known.resize(tid + 1, 0);
        }
        types[tid] = std::move(wt);
        known[tid] = 1;
    }
    const WireType& type(int tid) const {
        if (tid < FIRST_DEFINABLE_ID || (size_t)tid >= types.size() || !known[tid]) throw Err();
        return types[tid];
    }
    void skip(In& r, int tid, int depth = 0) const {
        if (depth > 64) throw Err();
        switch (tid) {
        case T_BOOL:
        case T_INT:
        case T_UINT:
        case T_FLOAT: (void)r.uint(); return;
        case T_BYTES:
        case T_STRING: (void)r.take(r.uint()); return;
        case T_COMPLEX: (void)r.uint(); (void)r.uint(); return;
        default: break;
        }
        const WireType& wt = type(tid);
        if (wt.kind == 3) {
            int field = -1;
            for (;;) {
                const uint64_t d = r.uint();
                if (d == 0) return;
                if (d > wt.fields.size()) throw Err();
                field += (int)d;
                if (field < 0 || (size_t)field >= wt.fields.size()) throw Err();
                skip(r, wt.fields[field].second, depth + 1);
            }
        }
        if (wt.kind == 1 || wt.kind == 2) {
            const uint64_t n = r.count();
            for (uint64_t j = 0; j < n; j++) skip(r, wt.elem, depth + 1);
            return;
        }
        if (wt.kind == 4) {
            const uint64_t n = r.count();
            for (uint64_t j = 0; j < n; j++) {
                skip(r, wt.key, depth + 1);
                skip(r, wt.elem, depth + 1);
            }
            return;
        }
        (void)r.take(r.uint());  // encoder bytes
    }
    static int64_t integer(In& r, int tid) {
        if (tid == T_INT) return r.sint();
        if (tid == T_UINT) return (int64_t)r.uint();
        throw Err();
    }
    void float_slice(int tid) const {
        const WireType& wt = type(tid);
        if ((wt.kind != 1 && wt.kind != 2) || wt.elem != T_FLOAT) throw Err();
    }
    // Reads a []float32 into dst when its length is want; returns the length.
    static uint64_t floats_into(In& r, float* dst, int64_t want) {
        const uint64_t n = r.count();
        if ((int64_t)n == want) {
            for (uint64_t j = 0; j < n; j++) dst[j] = r.flt();
        } else {
            for (uint64_t j = 0; j < n; j++) (void)r.uint();
        }
        return n;
    }
    // Appends the rows of a [][]float32 to out when each has length want; a
    // row of another length sets bad (the index is then rejected) and is not
    // stored. Storage grows only by floats the stream holds, so a small
    // malformed stream cannot make a large allocation. Returns the row count.
    int64_t float_rows(In& r, int tid, int64_t want, std::vector<float>& out, bool& bad) {
        const WireType& wt = type(tid);
        if (wt.kind != 1 && wt.kind != 2) throw Err();
        float_slice(wt.elem);
        const uint64_t n = r.count();
        for (uint64_t j = 0; j < n; j++) {
            const uint64_t k = r.count();
            if (want > 0 && (int64_t)k == want) {
                const size_t base = out.size();
                out.resize(base + (size_t)k);
                for (uint64_t i = 0; i < k; i++) out[base + i] = r.flt();
            } else {
                for (uint64_t i = 0; i < k; i++) r.skip_uint();
                bad = true;
            }
        }
        return (int64_t)n;
    }

    // Field roles of the pqEntry struct type, resolved once by name.
    struct EntryType {
        const WireType* et = nullptr;
        std::vector<int> role;
        int codes_elem = 0;
    };
    EntryType entry_type(int tid) const {
        EntryType e;
        e.et = &type(tid);
        if (e.et->kind != 3) throw Err();
        e.role.assign(e.et->fields.size(), R_SKIP);
        for (size_t f = 0; f < e.et->fields.size(); f++) {
            const std::string& nm = e.et->fields[f].first;
            const int ft = e.et->fields[f].second;
            if (nm == "ID" && (ft == T_INT || ft == T_UINT)) {
                e.role[f] = R_ID;
            } else if (nm == "Cluster" && (ft == T_INT || ft == T_UINT)) {
                e.role[f] = R_CLUSTER;
            } else if (nm == "Vector") {
                float_slice(ft);
                e.role[f] = R_VEC;
            } else if (nm == "Codes") {
                const WireType& ct = type(ft);
                if ((ct.kind != 1 && ct.kind != 2) || (ct.elem != T_INT && ct.elem != T_UINT)) throw Err();
                e.codes_elem = ct.elem;
                e.role[f] = R_CODES;
            }
        }
        return e;
    }
    // Walks one entry without storing it; returns its code count.
    int64_t skim_entry(In& r, const EntryType& e) const {
        const size_t nf = e.et->fields.size();
        int64_t nc = 0;
        int field = -1;
        for (;;) {
            const uint64_t d = r.uint();
            if (d == 0) return nc;
            if (d > nf) throw Err();
            field += (int)d;
            if ((size_t)field >= nf) throw Err();
            switch (e.role[field]) {
            case R_ID:
            case R_CLUSTER: r.skip_uint(); break;
            case R_VEC:
            case R_CODES: {
                const uint64_t n = r.count();
                for (uint64_t j = 0; j < n; j++) r.skip_uint();
                if (e.role[field] == R_CODES) nc += (int64_t)n;
                break;
            }
            default: skip(r, e.et->fields[field].second);
            }
        }
    }
    // Decodes one list's entries into the flat arrays at its rows.
    void decode_list(In& r, const EntryType& e, hann_gob_state& st, hann_gob_state::Seg& g) const {
        const size_t nf = e.et->fields.size();
        const int64_t dim = st.dimension;
        int64_t code_at = g.code;
        const int64_t code_end = g.code + g.ncodes;
        for (int64_t t = 0; t < g.n; t++) {
            const int64_t row = g.row + t;
            st.ids[row] = 0;
            st.ncodes[row] = 0;
            bool have_vec = false;
            int field = -1;
            for (;;) {
                const uint64_t d = r.uint();
                if (d == 0) break;
                if (d > nf) throw Err();
                field += (int)d;
                if ((size_t)field >= nf) throw Err();
                const int ft = e.et->fields[field].second;
                switch (e.role[field]) {
                case R_ID: st.ids[row] = integer(r, ft); break;
                case R_CLUSTER: (void)integer(r, ft); break;
                case R_VEC: {
                    const uint64_t got = floats_into(r, st.vecs_stored ? st.vecs.data() + row * dim : nullptr,
                                                     st.vecs_stored ? dim : -1);
                    have_vec = true;
                    if ((int64_t)got != dim && g.bad_row < 0) {
                        g.bad_row = row;
                        g.bad_len = (int64_t)got;
                    }
                    break;
                }
                case R_CODES: {
                    const uint64_t nc = r.count();
                    if ((int64_t)nc > code_end - code_at) throw Err();
                    st.ncodes[row] = (int64_t)nc;
                    for (uint64_t m = 0; m < nc; m++) {
                        const int64_t v = integer(r, e.codes_elem);
                        st.codes[code_at++] = v >= 0 && v <= INT32_MAX ? (int32_t)v : -1;
                    }
                    break;
                }
                default: skip(r, ft);
                }
            }
            if (!have_vec && dim != 0 && g.bad_row < 0) {  // a nil vector has length 0
                g.bad_row = row;
                g.bad_len = 0;
            }
        }
    }

    // The inverted-list map: a skim that finds each list's byte offset,
    // rows and codes, then the lists decoded in parallel into arrays sized
    // from the skim.
    void lists(In& r, int tid, hann_gob_state& st) {
        const WireType& mt = type(tid);
        if (mt.kind != 4) throw Err();
        const WireType& lt = type(mt.elem);
        if (lt.kind != 1 && lt.kind != 2) throw Err();
        const EntryType e = entry_type(lt.elem);
        if (!st.segs.empty()) throw Err();
        const uint64_t nmap = r.count();
        int64_t rows = 0, ncodes = 0;
        for (uint64_t j = 0; j < nmap; j++) {
            hann_gob_state::Seg g{};
            g.cluster = integer(r, mt.key);
            g.n = (int64_t)r.count();
            g.row = rows;
            g.code = ncodes;
            g.at = r.i;
            g.bad_row = -1;
            for (int64_t t = 0; t < g.n; t++) g.ncodes += skim_entry(r, e);
            rows += g.n;
            ncodes += g.ncodes;
            st.segs.push_back(g);
        }
        const size_t end = r.i;
        // Vectors get rows x dim floats only when the stream is long enough to
        // hold them all at full length; when it is not, some entry's vector is
        // short (the index is rejected) and none is stored.
        st.vecs_stored = st.dimension > 0 && rows > 0 && (uint64_t)rows <= r.n / (uint64_t)st.dimension;
        st.ids.alloc((size_t)rows);
        st.ncodes.alloc((size_t)rows);
        st.codes.alloc((size_t)ncodes);
        st.vecs.alloc(st.vecs_stored ? (size_t)rows * (size_t)st.dimension : 0);
        std::atomic<int> failed{0};
        parallel_for((int64_t)st.segs.size(), [&](int64_t s) {
            if (failed.load(std::memory_order_relaxed)) return;
            try {
                In sub(r.p, r.n);
                sub.i = st.segs[s].at;
                decode_list(sub, e, st, st.segs[s]);
            } catch (const Err&) {
                failed.store(1);
            } catch (...) {
                failed.store(2);
            }
        });
        if (failed.load() == 1) throw Err();
        if (failed.load() == 2) throw std::bad_alloc();
        r.i = end;
    }

    void serialized(In& r, const WireType& wt, hann_gob_state& st) {
        int field = -1;
        for (;;) {
            const uint64_t d = r.uint();
            if (d == 0) return;
            if (d > wt.fields.size()) throw Err();
            field += (int)d;
            if (field < 0 || (size_t)field >= wt.fields.size()) throw Err();
            const std::string& nm = wt.fields[field].first;
            const int ft = wt.fields[field].second;
            const bool isint = ft == T_INT || ft == T_UINT;
            if (nm == "Dimension" && isint) {
                st.dimension = integer(r, ft);
            } else if (nm == "CoarseK" && isint) {
                st.coarse_k = integer(r, ft);
            } else if (nm == "NumSubquantizers" && isint) {
                st.num_subquantizers = integer(r, ft);
            } else if (nm == "PqK" && isint) {
                st.pq_k = integer(r, ft);
            } else if (nm == "KMeansIters" && isint) {
                st.kmeans_iters = integer(r, ft);
            } else if (nm == "FormatVersion" && isint) {
                st.format_version = integer(r, ft);
            } else if (nm == "NumCandidateClusters" && isint) {
                st.candidate_clusters = integer(r, ft);
            } else if (nm == "AllowBruteForceFallback" && ft == T_BOOL) {
                st.fallback = r.uint() != 0;
            } else if (nm == "Trained" && ft == T_BOOL) {
                st.trained = r.uint() != 0;
            } else if (nm == "CoarseCentroids") {
                bool bad = false;
                st.coarse.clear();
                st.coarse_rows = float_rows(r, ft, st.dimension, st.coarse, bad);
                if (bad && !st.shape_error) {
                    st.shape_error = true;
                    st.shape_msg = "a coarse centroid has the wrong dimension";
                }
            } else if (nm == "Codebooks") {
                const WireType& t3 = type(ft);
                if (t3.kind != 1 && t3.kind != 2) throw Err();
                const int64_t M = st.num_subquantizers;
                const int64_t ds = (M > 0 && st.dimension > 0 && st.dimension % M == 0) ? st.dimension / M : -1;
                const uint64_t n = r.count();
                st.codebooks.clear();
                st.cb_tables = (int64_t)n;
                for (uint64_t j = 0; j < n; j++) {
                    bool bad = false;
                    const int64_t words = float_rows(r, t3.elem, ds, st.codebooks, bad);
                    if (j == 0) st.cb_words = words;
                    if ((bad || words != st.cb_words) && !st.shape_error) {
                        st.shape_error = true;
                        st.shape_msg = bad ? "a codeword has the wrong dimension" : "codebooks of different sizes";
                    }
                }
            } else if (nm == "ClusterCounts") {
                const WireType& mt = type(ft);
                if (mt.kind != 4) throw Err();
                const uint64_t n = r.count();
                for (uint64_t j = 0; j < n; j++) {
                    const int64_t c = integer(r, mt.key);
                    st.counts.emplace_back(c, integer(r, mt.elem));
                }
            } else if (nm == "InvertedLists") {
                lists(r, ft, st);
            } else if (nm == "PendingVectors") {
                const WireType& mt = type(ft);
                if (mt.kind != 4) throw Err();
                float_slice(mt.elem);
                const int64_t dim = st.dimension;
                const uint64_t n = r.count();
                for (uint64_t j = 0; j < n; j++) {
                    st.pending_ids.push_back(integer(r, mt.key));
                    const uint64_t k = r.count();
                    if (dim > 0 && (int64_t)k == dim) {  // stored only at full length (see float_rows)
                        const size_t base = st.pending.size();
                        st.pending.resize(base + (size_t)k);
                        for (uint64_t i = 0; i < k; i++) st.pending[base + i] = r.flt();
                    } else {
                        for (uint64_t i = 0; i < k; i++) r.skip_uint();
                        if (st.bad_pending < 0) st.bad_pending = st.pending_ids.back();
                    }
                }
            } else {
                skip(r, ft);
            }
        }
    }
};

// Reads one gob stream: type definitions into dec, value messages to
// on_value until it returns false.
template <typename F> void each_value(const uint8_t* data, size_t len, Dec& dec, F on_value) {
    In r(data, len);
    while (!r.eof()) {
        const uint64_t n = r.uint();
        In m(r.take(n), (size_t)n);
        const int64_t tid = m.sint();
        if (tid < 0) {
            if (tid < -(int64_t)MAX_TYPE_ID) throw Err();
            dec.define((int)-tid, decode_wiretype(m));
            continue;
        }
        if (!on_value((int)tid, m)) return;
    }
}

int fail(int rc, const std::string& msg) {
    g_gob_error = msg;
    return rc;
}

}  // namespace

extern "C" {

const char* hann_gob_last_error(void) { return g_gob_error.c_str(); }

}  // extern "C"

namespace {

// wrap: the stream Save writes (the *pqivf.Index GobEncoder around the
// payload); otherwise the payload alone, GobEncode's bytes.
int encode_impl(const hann_pqivf_layout* L, const float* coarse, const float* codebooks, const int64_t* list_len,
                const uint8_t* list_key, const int64_t* cluster_counts, const int64_t* ids, const float* vectors,
                const int32_t* codes, const int64_t* pending_ids, const float* pending_vectors, uint8_t* out,
                int64_t capacity, int64_t* out_len, bool wrap) {
    if (!L || !out_len) return fail(HANN_E_INVALID, "null layout or length");
    const int64_t dim = L->dimension, M = L->num_subquantizers, nl = L->nlist, kq = L->pq_k_eff;
    if (dim <= 0 || M <= 0 || dim % M != 0 || nl < 0 || kq < 0 || L->n_rows < 0 || L->n_pending < 0)
        return fail(HANN_E_INVALID, "invalid layout");
    EncodeInput in{L, coarse, codebooks, vectors, pending_vectors, list_len, cluster_counts, ids, pending_ids,
                   list_key, codes, {}, {}};
    try {
        in.list_row.resize((size_t)nl);
        int64_t rows = 0, nkeys = 0;
        for (int64_t c = 0; c < nl; c++) {
            if (list_len[c] < 0) return fail(HANN_E_INVALID, "negative list length");
            in.list_row[c] = rows;
            rows += list_len[c];
            nkeys += list_key[c] ? 1 : 0;
        }
        if (rows != L->n_rows) return fail(HANN_E_INVALID, "list lengths do not add up to the row count");
        in.pend_order.resize((size_t)L->n_pending);
        for (int64_t i = 0; i < L->n_pending; i++) in.pend_order[i] = i;
        if (!std::is_sorted(pending_ids, pending_ids + L->n_pending))
            std::stable_sort(in.pend_order.begin(), in.pend_order.end(),
                             [&](int64_t a, int64_t b) { return pending_ids[a] < pending_ids[b]; });

        // The struct value in five parts: head (fields 0-4 up to the list
        // map's length), lists, middle (fields 5-11 up to the pending map's
        // length), pending blocks, tail (fields 12-13 and the end mark).
        Vec head, mid, tail;
        int last = -1;
        auto field = [&](Vec& s, int i) {
            s.uint((uint64_t)(i - last));
            last = i;
        };
        field(head, 0);
        put_int(head, dim);
        if (L->coarse_k) {
            field(head, 1);
            put_int(head, L->coarse_k);
        }
        if (nl > 0) {
            field(head, 2);
            head.uint((uint64_t)nl);
            for (int64_t c = 0; c < nl; c++) put_floats(head, coarse + c * dim, dim);
        }
        if (nkeys) {
            field(head, 3);
            head.uint((uint64_t)nkeys);
            for (int64_t c = 0; c < nl; c++)
                if (list_key[c]) {
                    put_int(head, c);
                    put_int(head, cluster_counts[c]);
                }
            field(head, 4);
            head.uint((uint64_t)nkeys);
        }
        field(mid, 5);
        put_int(mid, M);
        if (nl > 0) {
            field(mid, 6);
            const int64_t ds = dim / M;
            mid.uint((uint64_t)M);
            for (int64_t m = 0; m < M; m++) {
                mid.uint((uint64_t)kq);
                for (int64_t j = 0; j < kq; j++) put_floats(mid, codebooks + (m * kq + j) * ds, ds);
            }
        }
        if (L->pq_k) {
            field(mid, 7);
            put_int(mid, L->pq_k);
        }
        if (L->kmeans_iters) {
            field(mid, 8);
            put_int(mid, L->kmeans_iters);
        }
        if (L->fallback) {
            field(mid, 9);
            mid.uint(1);
        }
        if (L->trained) {
            field(mid, 10);
            mid.uint(1);
        }
        if (L->n_pending > 0) {
            field(mid, 11);
            mid.uint((uint64_t)L->n_pending);
        }
        field(tail, 12);
        put_int(tail, FORMAT_VERSION);
        if (L->candidate_clusters) {
            field(tail, 13);
            put_int(tail, L->candidate_clusters);
        }
        tail.uint(0);

        // sizes of the large parts, in parallel
        std::vector<size_t> list_bytes((size_t)nl, 0);
        parallel_for(nl, [&](int64_t c) {
            if (!list_key[c]) return;
            Counter k;
            put_list(k, in, c);
            list_bytes[c] = k.n;
        });
        const int64_t nblocks = (L->n_pending + PENDING_BLOCK - 1) / PENDING_BLOCK;
        std::vector<size_t> block_bytes((size_t)nblocks, 0);
        parallel_for(nblocks, [&](int64_t b) {
            Counter k;
            put_pending_block(k, in, b);
            block_bytes[b] = k.n;
        });
        size_t value_len = uint_len(zigzag(T_SER)) + head.b.size() + mid.b.size() + tail.b.size();
        for (size_t v : list_bytes) value_len += v;
        for (size_t v : block_bytes) value_len += v;

        Vec types;
        def_slice(types, T_F32S, T_FLOAT);
        def_slice(types, T_F32SS, T_F32S);
        def_map(types, T_MAPII, T_INT, T_INT);
        def_slice(types, T_INTS, T_INT);
        def_map(types, T_MAPLIST, T_INT, T_ENTRIES);
        def_slice(types, T_ENTRIES, T_ENTRY);
        def_struct(types, T_ENTRY, "pqEntry",
                   {{"ID", T_INT}, {"Vector", T_F32S}, {"Codes", T_INTS}, {"Cluster", T_INT}});
        def_slice(types, T_F32SSS, T_F32SS);
        def_map(types, T_MAPIVEC, T_INT, T_F32S);
        def_struct(types, T_SER, "serializedPQIVF",
                   {{"Dimension", T_INT}, {"CoarseK", T_INT}, {"CoarseCentroids", T_F32SS},
                    {"ClusterCounts", T_MAPII}, {"InvertedLists", T_MAPLIST}, {"NumSubquantizers", T_INT},
                    {"Codebooks", T_F32SSS}, {"PqK", T_INT}, {"KMeansIters", T_INT},
                    {"AllowBruteForceFallback", T_BOOL}, {"Trained", T_BOOL}, {"PendingVectors", T_MAPIVEC},
                    {"FormatVersion", T_INT}, {"NumCandidateClusters", T_INT}});
        // inner stream = types, then (value length)(T_SER)(value parts)
        const size_t inner_len = types.b.size() + uint_len(value_len) + value_len;
        // outer stream = the encoder's type, then (length)(65)(0)(inner length)(inner)
        Vec outer;
        def_gobencoder(outer, FIRST_USER_ID, "*pqivf.Index");
        const size_t payload = 1 + uint_len(inner_len) + inner_len;
        outer.uint(uint_len(zigzag(FIRST_USER_ID)) + payload);
        put_int(outer, FIRST_USER_ID);
        outer.uint(0);  // singleton prefix
        outer.uint(inner_len);
        if (!wrap) outer.b.clear();
        const size_t total = outer.b.size() + inner_len;
        *out_len = (int64_t)total;
        if (!out) return HANN_OK;  // size query
        if (capacity < 0 || (size_t)capacity < total)
            return fail(HANN_E_INVALID, "output buffer of " + std::to_string(capacity) + " bytes, " +
                                            std::to_string(total) + " needed");

        Writer w{out};
        w.raw(outer.b.data(), outer.b.size());
        w.raw(types.b.data(), types.b.size());
        w.uint(value_len);
        put_int(w, T_SER);
        w.raw(head.b.data(), head.b.size());
        uint8_t* lists_at = w.p;
        std::vector<size_t> list_off((size_t)nl, 0);
        size_t acc = 0;
        for (int64_t c = 0; c < nl; c++) {
            list_off[c] = acc;
            acc += list_bytes[c];
        }
        parallel_for(nl, [&](int64_t c) {
            if (!list_key[c]) return;
            Writer lw{lists_at + list_off[c]};
            put_list(lw, in, c);
        });
        w.p = lists_at + acc;
        w.raw(mid.b.data(), mid.b.size());
        uint8_t* pend_at = w.p;
        std::vector<size_t> block_off((size_t)nblocks, 0);
        acc = 0;
        for (int64_t b = 0; b < nblocks; b++) {
            block_off[b] = acc;
            acc += block_bytes[b];
        }
        parallel_for(nblocks, [&](int64_t b) {
            Writer bw{pend_at + block_off[b]};
            put_pending_block(bw, in, b);
        });
        w.p = pend_at + acc;
        w.raw(tail.b.data(), tail.b.size());
        if ((size_t)(w.p - out) != total) return fail(HANN_E_INVALID, "gob encoder size mismatch");
    } catch (const std::bad_alloc&) {
        return fail(HANN_E_NOMEM, "out of host memory encoding the gob stream");
    } catch (const std::system_error&) {
        return fail(HANN_E_NOMEM, "could not start encoder threads");
    }
    return HANN_OK;
}

}  // namespace

extern "C" {

int hann_gob_encode(const hann_pqivf_layout* L, const float* coarse, const float* codebooks, const int64_t* list_len,
                    const uint8_t* list_key, const int64_t* cluster_counts, const int64_t* ids, const float* vectors,
                    const int32_t* codes, const int64_t* pending_ids, const float* pending_vectors, uint8_t* out,
                    int64_t capacity, int64_t* out_len) {
    return encode_impl(L, coarse, codebooks, list_len, list_key, cluster_counts, ids, vectors, codes, pending_ids,
                       pending_vectors, out, capacity, out_len, true);
}

int hann_gob_encode_payload(const hann_pqivf_layout* L, const float* coarse, const float* codebooks,
                            const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                            const int64_t* ids, const float* vectors, const int32_t* codes,
                            const int64_t* pending_ids, const float* pending_vectors, uint8_t* out, int64_t capacity,
                            int64_t* out_len) {
    return encode_impl(L, coarse, codebooks, list_len, list_key, cluster_counts, ids, vectors, codes, pending_ids,
                       pending_vectors, out, capacity, out_len, false);
}

int hann_gob_decode(const uint8_t* data, int64_t len, hann_gob_state** out) {
    if (!out || len < 0 || (len > 0 && !data)) return fail(HANN_E_INVALID, "null stream");
    *out = nullptr;
    hann_gob_state* st = nullptr;
    try {
        st = new hann_gob_state();
        Dec od;
        bool got = false;
        each_value(data, (size_t)len, od, [&](int tid, In& m) {
            const WireType& wt = od.type(tid);
            if (wt.kind == 3) {  // the struct itself, not wrapped
                od.serialized(m, wt, *st);
                got = true;
                return false;
            }
            if (wt.kind != 5) throw Err();
            if (m.uint() != 0) throw Err();  // singleton prefix
            const uint64_t n = m.uint();
            const uint8_t* inner = m.take(n);
            Dec idec;
            each_value(inner, (size_t)n, idec, [&](int itid, In& im) {
                const WireType& it = idec.type(itid);
                if (it.kind != 3) throw Err();
                idec.serialized(im, it, *st);
                got = true;
                return false;
            });
            return false;
        });
        if (!got) {
            delete st;
            return fail(HANN_E_INVALID, "gob stream holds no index");
        }
    } catch (const Err&) {
        delete st;
        return fail(HANN_E_INVALID, "malformed gob stream");
    } catch (const std::bad_alloc&) {
        delete st;
        return fail(HANN_E_NOMEM, "out of host memory decoding the gob stream");
    } catch (const std::length_error&) {
        delete st;
        return fail(HANN_E_INVALID, "malformed gob stream");
    }
    *out = st;
    return HANN_OK;
}

int hann_gob_state_layout(const hann_gob_state* st, int32_t default_candidate_clusters, hann_pqivf_layout* L) {
    if (!st || !L) return fail(HANN_E_INVALID, "null state or layout");
    if (st->format_version > FORMAT_VERSION)
        return fail(HANN_E_INVALID, "index file has format version " + std::to_string(st->format_version) +
                                        ", but this build supports up to " + std::to_string(FORMAT_VERSION));
    const int64_t dim = st->dimension, M = st->num_subquantizers;
    if (dim <= 0) return fail(HANN_E_INVALID, "serialized index has invalid dimension " + std::to_string(dim));
    if (M <= 0 || dim % M != 0)
        return fail(HANN_E_INVALID, "serialized index has invalid subquantizer count " + std::to_string(M) +
                                        " for dimension " + std::to_string(dim));
    if (st->coarse_k <= 0 || st->pq_k <= 0 || st->kmeans_iters <= 0)
        return fail(HANN_E_INVALID, "serialized index has invalid training parameters: coarseK " +
                                        std::to_string(st->coarse_k) + ", pqK " + std::to_string(st->pq_k) +
                                        ", kMeansIters " + std::to_string(st->kmeans_iters));
    if (dim > INT32_MAX || st->coarse_k > INT32_MAX || st->pq_k > INT32_MAX || st->kmeans_iters > INT32_MAX ||
        st->candidate_clusters > INT32_MAX || st->coarse_rows > INT32_MAX || st->cb_words > INT32_MAX)
        return fail(HANN_E_UNSUPPORTED, "serialized index parameters exceed this build's limits");
    if (st->shape_error) return fail(HANN_E_INVALID, st->shape_msg);
    const int64_t nl = st->coarse_rows;
    const int64_t kq = st->cb_tables ? st->cb_words : 0;
    if (kq && st->cb_tables != M) return fail(HANN_E_INVALID, "codebook count does not match the subquantizer count");
    // A list or count key outside the centroids: the reference keeps it
    // (pqivf/index.go:1059-1081); this build holds lists by centroid.
    auto outside = [&](int64_t c, bool nonempty) { return c < 0 || (c >= std::max<int64_t>(nl, 1) && nonempty); };
    std::vector<int64_t> seg_of((size_t)nl, -1);
    for (size_t s = 0; s < st->segs.size(); s++) {
        const auto& g = st->segs[s];
        if (outside(g.cluster, g.n > 0))
            return fail(HANN_E_UNSUPPORTED, "inverted list " + std::to_string(g.cluster) + " has no coarse centroid");
        if (g.cluster < nl) seg_of[g.cluster] = (int64_t)s;
    }
    for (auto& kv : st->counts)
        if (kv.first < 0)
            return fail(HANN_E_UNSUPPORTED, "inverted list " + std::to_string(kv.first) + " has no coarse centroid");
    int64_t rows = 0;
    for (int64_t c = 0; c < nl; c++)
        if (seg_of[c] >= 0) {
            const auto& g = st->segs[seg_of[c]];
            if (g.bad_row >= 0)
                return fail(HANN_E_INVALID, "entry " + std::to_string(st->ids[g.bad_row]) +
                                                " has a vector of dimension " + std::to_string(g.bad_len));
            rows += g.n;
        }
    if (st->bad_pending >= 0)
        return fail(HANN_E_INVALID, "pending vector " + std::to_string(st->bad_pending) + " has the wrong dimension");
    std::memset(L, 0, sizeof(*L));
    L->dimension = (int32_t)dim;
    L->coarse_k = (int32_t)st->coarse_k;
    L->num_subquantizers = (int32_t)M;
    L->pq_k = (int32_t)st->pq_k;
    L->kmeans_iters = (int32_t)st->kmeans_iters;
    L->candidate_clusters = st->candidate_clusters > 0    ? (int32_t)st->candidate_clusters
                            : default_candidate_clusters > 0 ? default_candidate_clusters
                                                             : 3;
    L->fallback = st->fallback ? 1 : 0;
    L->trained = st->trained ? 1 : 0;
    L->nlist = (int32_t)nl;
    L->pq_k_eff = (int32_t)kq;
    L->n_rows = rows;
    // pending ids are a map's keys: one vector per id
    std::vector<int64_t> p(st->pending_ids);
    std::sort(p.begin(), p.end());
    L->n_pending = (int64_t)(std::unique(p.begin(), p.end()) - p.begin());
    return HANN_OK;
}

int hann_gob_state_arrays(const hann_gob_state* st, float* coarse, float* codebooks, int64_t* list_len,
                          uint8_t* list_key, int64_t* cluster_counts, int64_t* ids, float* vectors, int32_t* codes,
                          uint8_t* has_codes, int64_t* pending_ids, float* pending_vectors) {
    hann_pqivf_layout L;
    const int rc = hann_gob_state_layout(st, 3, &L);
    if (rc != HANN_OK) return rc;
    const int64_t dim = L.dimension, M = L.num_subquantizers, nl = L.nlist, kq = L.pq_k_eff, ds = dim / M;
    try {
        if (nl) std::memcpy(coarse, st->coarse.data(), sizeof(float) * (size_t)(nl * dim));
        if (kq) std::memcpy(codebooks, st->codebooks.data(), sizeof(float) * (size_t)(M * kq * ds));
        std::vector<int64_t> seg_of((size_t)nl, -1), count_of((size_t)nl, -1);
        for (size_t s = 0; s < st->segs.size(); s++)
            if (st->segs[s].cluster < nl) seg_of[st->segs[s].cluster] = (int64_t)s;
        for (size_t i = 0; i < st->counts.size(); i++)
            if (st->counts[i].first >= 0 && st->counts[i].first < nl) count_of[st->counts[i].first] = (int64_t)i;
        std::vector<int64_t> dst_row((size_t)nl, 0);
        int64_t r = 0;
        for (int64_t c = 0; c < nl; c++) {
            list_key[c] = (seg_of[c] >= 0 || count_of[c] >= 0) ? 1 : 0;
            cluster_counts[c] = count_of[c] >= 0 ? st->counts[count_of[c]].second : 0;
            list_len[c] = seg_of[c] >= 0 ? st->segs[seg_of[c]].n : 0;
            dst_row[c] = r;
            r += list_len[c];
        }
        parallel_for(nl, [&](int64_t c) {
            if (seg_of[c] < 0) return;
            const auto& g = st->segs[seg_of[c]];
            int64_t code_at = g.code;
            for (int64_t j = 0; j < g.n; j++) {
                const int64_t src = g.row + j, dst = dst_row[c] + j;
                ids[dst] = st->ids[src];
                std::memcpy(vectors + dst * dim, st->vecs.data() + src * dim, sizeof(float) * (size_t)dim);
                const int64_t nc = st->ncodes[src];
                bool ok = nc == M;
                for (int64_t m = 0; ok && m < nc; m++)
                    ok = st->codes[code_at + m] >= 0 && st->codes[code_at + m] < kq;
                for (int64_t m = 0; m < M; m++) codes[dst * M + m] = ok ? st->codes[code_at + m] : 0;
                if (has_codes) has_codes[dst] = ok ? 1 : 0;
                code_at += nc;
            }
        });
        // pending vectors by ascending id; for a repeated id the last one wins
        std::vector<int64_t> order(st->pending_ids.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = (int64_t)i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int64_t a, int64_t b) { return st->pending_ids[a] < st->pending_ids[b]; });
        int64_t k = 0;
        for (size_t i = 0; i < order.size(); i++) {
            if (i + 1 < order.size() && st->pending_ids[order[i + 1]] == st->pending_ids[order[i]]) continue;
            pending_ids[k] = st->pending_ids[order[i]];
            std::memcpy(pending_vectors + k * dim, st->pending.data() + order[i] * dim, sizeof(float) * (size_t)dim);
            k++;
        }
    } catch (const std::bad_alloc&) {
        return fail(HANN_E_NOMEM, "out of host memory");
    } catch (const std::system_error&) {
        return fail(HANN_E_NOMEM, "could not start decoder threads");
    }
    return HANN_OK;
}

void hann_gob_state_free(hann_gob_state* st) { delete st; }

}  // extern "C"
