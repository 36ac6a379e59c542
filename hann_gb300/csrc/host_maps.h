// host_maps.h -- the host-side id containers of a PQIVF handle: the id ->
// list map of the trained rows and the store of vectors added before
// training. Plain C++ (no CUDA) so they compile and are tested on their own.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace hann {

// Map from 64-bit ids to values held in three flat arrays (open addressing,
// linear probing, power-of-two capacity at most half full, tombstones on
// erase): 13 bytes a slot, two to four slots an id, and no heap node an id,
// so building the id -> list map of a million-row index after training, and
// freeing it, cost a few passes over memory rather than an allocation per
// id.
template <typename V>
class IdMap {
    std::vector<int64_t> key_;
    std::vector<V> val_;
    std::vector<uint8_t> st_;  // 0 empty, 1 full, 2 erased
    size_t size_ = 0, used_ = 0;

    static size_t mix(int64_t k) {
        uint64_t z = (uint64_t)k + 0x9e3779b97f4a7c15ull;  // splitmix64 finalizer
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return (size_t)(z ^ (z >> 31));
    }
    // Slot holding k, or SIZE_MAX.
    size_t locate(int64_t k) const {
        if (key_.empty()) return SIZE_MAX;
        const size_t mask = key_.size() - 1;
        for (size_t i = mix(k) & mask;; i = (i + 1) & mask) {
            if (st_[i] == 0) return SIZE_MAX;
            if (st_[i] == 1 && key_[i] == k) return i;
        }
    }
    void rehash(size_t cap) {
        std::vector<int64_t> k2(cap);
        std::vector<V> v2(cap);
        std::vector<uint8_t> s2(cap, 0);
        const size_t mask = cap - 1;
        for (size_t i = 0; i < key_.size(); i++) {
            if (st_[i] != 1) continue;
            size_t j = mix(key_[i]) & mask;
            while (s2[j]) j = (j + 1) & mask;
            k2[j] = key_[i];
            v2[j] = val_[i];
            s2[j] = 1;
        }
        key_.swap(k2);
        val_.swap(v2);
        st_.swap(s2);
        used_ = size_;
    }

  public:
    size_t size() const { return size_; }
    void clear() {
        std::vector<int64_t>().swap(key_);
        std::vector<V>().swap(val_);
        std::vector<uint8_t>().swap(st_);
        size_ = used_ = 0;
    }
    // Room for n ids without a rehash.
    void reserve(size_t n) {
        size_t cap = 16;
        while (cap < 2 * n + 2) cap <<= 1;
        if (cap > key_.size()) rehash(cap);
    }
    bool count(int64_t k) const { return locate(k) != SIZE_MAX; }
    const V* find(int64_t k) const {
        const size_t i = locate(k);
        return i == SIZE_MAX ? nullptr : &val_[i];
    }
    V* find(int64_t k) {
        const size_t i = locate(k);
        return i == SIZE_MAX ? nullptr : &val_[i];
    }
    // Inserts k or replaces its value.
    void set(int64_t k, V v) {
        if (V* p = find(k)) {
            *p = v;
            return;
        }
        if (2 * (used_ + 1) > key_.size()) {  // at most a quarter full after the rehash
            size_t cap = std::max<size_t>(16, key_.size());
            while (cap < 4 * (size_ + 1)) cap <<= 1;
            rehash(cap);
        }
        const size_t mask = key_.size() - 1;
        size_t i = mix(k) & mask;
        while (st_[i] == 1) i = (i + 1) & mask;
        if (st_[i] == 0) used_++;
        key_[i] = k;
        val_[i] = v;
        st_[i] = 1;
        size_++;
    }
    bool erase(int64_t k) {
        const size_t i = locate(k);
        if (i == SIZE_MAX) return false;
        st_[i] = 2;
        size_--;
        return true;
    }
};

// Vectors added before training, keyed by id: one contiguous array of
// dim-float slots in insertion order, an id per slot, and the id -> slot map.
// Training uploads the array as it stands (erased slots are skipped by the
// gather), with no copy per vector on the host.
struct PendingStore {
    int dim = 0;
    std::vector<float> vec;         // slot-major
    std::vector<int64_t> slot_id;   // id of each slot
    std::vector<uint8_t> slot_live;  // 0 for an erased slot
    IdMap<int64_t> slot;            // id -> slot
    int64_t dead = 0;

    size_t size() const { return slot.size(); }
    bool count(int64_t id) const { return slot.count(id); }
    const float* find(int64_t id) const {
        const int64_t* s = slot.find(id);
        return s ? vec.data() + (size_t)*s * dim : nullptr;
    }
    void clear() {
        std::vector<float>().swap(vec);
        std::vector<int64_t>().swap(slot_id);
        std::vector<uint8_t>().swap(slot_live);
        slot.clear();
        dead = 0;
    }
    // Room for n more vectors of dimension d.
    void reserve_more(size_t n, int d) {
        if (slot_id.empty()) dim = d;
        vec.reserve(vec.size() + n * (size_t)dim);
        slot_id.reserve(slot_id.size() + n);
        slot_live.reserve(slot_live.size() + n);
        slot.reserve(slot.size() + n);
    }
    // Inserts id's vector or replaces it.
    void put(int64_t id, const float* v, int d) {
        if (slot_id.empty()) dim = d;
        if (int64_t* s = slot.find(id)) {
            std::memcpy(vec.data() + (size_t)*s * dim, v, sizeof(float) * dim);
            return;
        }
        slot.set(id, (int64_t)slot_id.size());
        slot_id.push_back(id);
        slot_live.push_back(1);
        vec.insert(vec.end(), v, v + dim);
    }
    bool erase(int64_t id) {
        const int64_t* s = slot.find(id);
        if (!s) return false;
        slot_live[(size_t)*s] = 0;
        slot.erase(id);
        if (++dead > 4096 && 2 * dead > (int64_t)slot_id.size()) compact();
        return true;
    }
    // Live ids in ascending order.
    std::vector<int64_t> sorted_ids() const {
        std::vector<int64_t> out;
        out.reserve(size());
        for (size_t i = 0; i < slot_id.size(); i++)
            if (slot_live[i]) out.push_back(slot_id[i]);
        if (!std::is_sorted(out.begin(), out.end())) std::sort(out.begin(), out.end());
        return out;
    }

  private:
    void compact() {
        size_t w = 0;
        for (size_t i = 0; i < slot_id.size(); i++) {
            if (!slot_live[i]) continue;
            if (w != i) {
                std::memmove(vec.data() + w * dim, vec.data() + i * dim, sizeof(float) * dim);
                slot_id[w] = slot_id[i];
            }
            slot_live[w] = 1;
            slot.set(slot_id[w], (int64_t)w);
            w++;
        }
        vec.resize(w * dim);
        slot_id.resize(w);
        slot_live.resize(w);
        dead = 0;
    }
};

}  // namespace hann
