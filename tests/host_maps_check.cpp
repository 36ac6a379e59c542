// Randomised check of hann::IdMap and hann::PendingStore against the standard
// containers: every operation's result and the final contents must agree.
// Built and run by tests/test_host_maps.py; prints "ok" and exits 0 on success.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <unordered_map>
#include <vector>

#include "host_maps.h"

#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);       \
            std::exit(1);                                          \
        }                                                          \
    } while (0)

static void check_idmap(uint64_t seed, int64_t key_range, int ops) {
    std::mt19937_64 rng(seed);
    hann::IdMap<int32_t> m;
    std::unordered_map<int64_t, int32_t> ref;
    for (int i = 0; i < ops; i++) {
        // keys from a small range (collisions, re-inserts after erase) and the
        // int64 extremes
        int64_t k = (int64_t)(rng() % (uint64_t)key_range) - key_range / 2;
        if (rng() % 97 == 0) k = (rng() & 1) ? INT64_MIN : INT64_MAX;
        const int op = (int)(rng() % 10);
        if (op < 5) {
            const int32_t v = (int32_t)rng();
            m.set(k, v);
            ref[k] = v;
        } else if (op < 8) {
            CHECK(m.erase(k) == (ref.erase(k) == 1));
        } else if (op == 8) {
            const int32_t* p = m.find(k);
            auto it = ref.find(k);
            CHECK((p != nullptr) == (it != ref.end()));
            if (p) CHECK(*p == it->second);
        } else if (rng() % 500 == 0) {
            m.clear();
            ref.clear();
        } else if (rng() % 50 == 0) {
            m.reserve(ref.size() + (size_t)(rng() % 1000));
        }
        CHECK(m.size() == ref.size());
    }
    for (auto& kv : ref) {
        const int32_t* p = m.find(kv.first);
        CHECK(p && *p == kv.second);
    }
    if (key_range <= 100000)
        for (int64_t k = -key_range / 2 - 5; k < key_range / 2 + 5; k++) CHECK(m.count(k) == (ref.count(k) == 1));
}

static void check_pending(uint64_t seed, int dim, int ops) {
    std::mt19937_64 rng(seed);
    hann::PendingStore p;
    std::map<int64_t, std::vector<float>> ref;
    std::vector<float> v(dim);
    for (int i = 0; i < ops; i++) {
        const int64_t id = (int64_t)(rng() % 20000) - 500;
        const int op = (int)(rng() % 10);
        if (op < 5) {
            for (int j = 0; j < dim; j++) v[j] = (float)(rng() % 100000) * 0.5f;
            if (rng() % 7 == 0) p.reserve_more(rng() % 100, dim);
            p.put(id, v.data(), dim);
            ref[id] = v;
        } else if (op < 9) {
            // many erasures: the store compacts its slots past 4096 dead ones
            CHECK(p.erase(id) == (ref.erase(id) == 1));
        } else {
            const float* f = p.find(id);
            auto it = ref.find(id);
            CHECK((f != nullptr) == (it != ref.end()));
            if (f) CHECK(std::memcmp(f, it->second.data(), sizeof(float) * dim) == 0);
        }
        CHECK(p.size() == ref.size());
    }
    // live slots: exactly the reference's ids, each slot's vector its id's
    const std::vector<int64_t> ids = p.sorted_ids();
    CHECK(ids.size() == ref.size());
    size_t j = 0;
    for (auto& kv : ref) {
        CHECK(ids[j++] == kv.first);
        CHECK(std::memcmp(p.find(kv.first), kv.second.data(), sizeof(float) * dim) == 0);
    }
    size_t live = 0;
    for (size_t s = 0; s < p.slot_id.size(); s++) {
        if (!p.slot_live[s]) continue;
        live++;
        auto it = ref.find(p.slot_id[s]);
        CHECK(it != ref.end());
        CHECK(std::memcmp(p.vec.data() + s * dim, it->second.data(), sizeof(float) * dim) == 0);
    }
    CHECK(live == ref.size());
    CHECK(p.vec.size() == p.slot_id.size() * (size_t)dim);
    p.clear();
    CHECK(p.size() == 0 && p.sorted_ids().empty() && p.find(0) == nullptr);
}

int main() {
    for (uint64_t s = 1; s <= 6; s++) {
        check_idmap(s, 64, 20000);
        check_idmap(s + 100, 5000, 200000);
        check_idmap(s + 200, 1 << 30, 100000);
    }
    check_pending(7, 3, 60000);
    check_pending(8, 16, 200000);
    // ids added in ascending order, no erasure: slots stay in id order
    hann::PendingStore p;
    std::vector<float> v(4, 1.0f);
    for (int64_t id = 0; id < 1000; id++) p.put(id, v.data(), 4);
    for (size_t s = 0; s < p.slot_id.size(); s++) CHECK(p.slot_id[s] == (int64_t)s);
    std::printf("ok\n");
    return 0;
}
