// select.cuh -- block-level selection helpers shared by the probe and k-NN
// kernels: bitonic sort of (key, index) pairs and an n-th-smallest radix
// select over float keys.
#pragma once

#include "common.cuh"

namespace hann {

__device__ __forceinline__ bool ki_less(uint32_t ka, int32_t ia, uint32_t kb, int32_t ib) {
    return ka < kb || (ka == kb && ia < ib);
}

__device__ __forceinline__ void sort_ki(uint32_t* key, int32_t* idx, int P) {
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    if (up == ki_less(key[ixj], idx[ixj], key[i], idx[i])) {
                        const uint32_t tk = key[i];
                        key[i] = key[ixj];
                        key[ixj] = tk;
                        const int32_t ti = idx[i];
                        idx[i] = idx[ixj];
                        idx[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Key (float_key) of the n-th smallest value of row[0..len) (1-based n) in
// *s_prefix, and in *s_rem how many values with that key are needed to reach
// n. Shaped for rows whose keys share most high bits (distances of one
// query): digits start at the highest bit where the keys
// differ, every warp counts into its own histogram with one atomic per
// distinct bin (lanes agreeing on a bin are merged by __match_any_sync), and
// one warp scans the 256 bins. whist holds THREADS/32 x 256 counters; the
// block must have exactly THREADS threads.
template <int THREADS>
__device__ __forceinline__ void radix_nth_fast(const float* __restrict__ row, int len, int n, unsigned int* whist, uint32_t* s_prefix,
                               uint32_t* s_rem, uint32_t* s_and, uint32_t* s_or) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    constexpr int NW = THREADS / 32;
    if (threadIdx.x == 0) {
        *s_and = 0xffffffffu;
        *s_or = 0u;
        *s_rem = (uint32_t)n;
    }
    __syncthreads();
    uint32_t a = 0xffffffffu, o = 0u;
    for (int c = threadIdx.x; c < len; c += THREADS) {
        const uint32_t k = float_key(row[c]);
        a &= k;
        o |= k;
    }
    a = __reduce_and_sync(0xffffffffu, a);
    o = __reduce_or_sync(0xffffffffu, o);
    if (lane == 0) {
        atomicAnd(s_and, a);
        atomicOr(s_or, o);
    }
    __syncthreads();
    const uint32_t band = *s_and, diff = band ^ *s_or;
    if (diff == 0) {
        if (threadIdx.x == 0) *s_prefix = band;
        __syncthreads();
        return;
    }
    const int top = 31 - __clz(diff);
    if (threadIdx.x == 0) *s_prefix = top == 31 ? 0u : (band & (0xffffffffu << (top + 1)));
    for (int hi = top; hi >= 0; hi -= 8) {
        const int lo = hi >= 7 ? hi - 7 : 0;
        const uint32_t himask = hi == 31 ? 0u : (0xffffffffu << (hi + 1));
        const uint32_t dmask = (1u << (hi - lo + 1)) - 1u;
        for (int b = threadIdx.x; b < NW * 256; b += THREADS) whist[b] = 0;
        __syncthreads();
        const uint32_t prefix = *s_prefix;
        for (int c0 = 0; c0 < len; c0 += THREADS) {
            const int c = c0 + threadIdx.x;
            uint32_t bin = 0xffffffffu;
            if (c < len) {
                const uint32_t k = float_key(row[c]);
                if ((k & himask) == prefix) bin = (k >> lo) & dmask;
            }
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            if (bin != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&whist[w * 256 + bin], __popc(peers));
        }
        __syncthreads();
        if (w == 0) {
            // lane owns bins [8*lane, 8*lane+8)
            uint32_t cnt[8], tot = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                uint32_t v = 0;
                for (int ww = 0; ww < NW; ww++) v += whist[ww * 256 + lane * 8 + j];
                cnt[j] = v;
                tot += v;
            }
            uint32_t incl = tot;
#pragma unroll
            for (int o2 = 1; o2 < 32; o2 <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o2);
                if (lane >= o2) incl += t;
            }
            const uint32_t excl = incl - tot;
            const uint32_t rem = *s_rem;
            const bool mine = excl < rem && rem <= incl;
            if (mine) {
                uint32_t cum = excl;
                for (int j = 0; j < 8; j++) {
                    if (cum + cnt[j] >= rem) {
                        *s_prefix = prefix | ((uint32_t)(lane * 8 + j) << lo);
                        *s_rem = rem - cum;
                        break;
                    }
                    cum += cnt[j];
                }
            }
        }
        __syncthreads();
    }
}

// Bitonic sort of P (a power of two) 64-bit keys in shared memory, ascending.
__device__ __forceinline__ void sort_u64(unsigned long long* key, int P) {
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    const unsigned long long a = key[i], b = key[ixj];
                    if (up == (b < a)) {
                        key[i] = b;
                        key[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// The n-th smallest (1-based, 1 <= n <= len) of the 64-bit keys in the
// warp's shared memory, warp-synchronous: 8-bit digits from the highest bit
// where the keys differ, one warp-private histogram of 256 counters; once
// the chosen digit holds a single key, that key is the answer.
__device__ __forceinline__ unsigned long long warp_radix_nth_u64(const unsigned long long* keys, int len, int n,
                                                                 unsigned int* hist) {
    const int lane = threadIdx.x & 31;
    unsigned long long a = ~0ull, o = 0ull;
    for (int i = lane; i < len; i += 32) {
        a &= keys[i];
        o |= keys[i];
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        a &= __shfl_xor_sync(0xffffffffu, a, s);
        o |= __shfl_xor_sync(0xffffffffu, o, s);
    }
    const unsigned long long diff = a ^ o;
    if (diff == 0) return a;
    const int top = 63 - __clzll((long long)diff);
    unsigned long long prefix = top == 63 ? 0ull : (a & (~0ull << (top + 1)));
    uint32_t rem = (uint32_t)n;
    for (int hi = top; hi >= 0; hi -= 8) {
        const int lo = hi >= 7 ? hi - 7 : 0;
        const unsigned long long himask = hi == 63 ? 0ull : (~0ull << (hi + 1));
        const unsigned dmask = (1u << (hi - lo + 1)) - 1u;
#pragma unroll
        for (int b = 0; b < 8; b++) hist[b * 32 + lane] = 0;
        __syncwarp();
        for (int i0 = 0; i0 < len; i0 += 32) {
            const int i = i0 + lane;
            unsigned bin = 0xffffffffu;
            if (i < len) {
                const unsigned long long k = keys[i];
                if ((k & himask) == prefix) bin = (unsigned)(k >> lo) & dmask;
            }
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            if (bin != 0xffffffffu && lane == __ffs(peers) - 1) hist[bin] += __popc(peers);
            __syncwarp();
        }
        uint32_t cnt[8], tot = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            cnt[j] = hist[lane * 8 + j];
            tot += cnt[j];
        }
        uint32_t incl = tot;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, s);
            if (lane >= s) incl += t;
        }
        const uint32_t excl = incl - tot;
        const bool mine = excl < rem && rem <= incl;
        uint32_t pick = 0, below = 0, inbin = 0;
        if (mine) {
            uint32_t cum = excl;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (cum < rem && rem <= cum + cnt[j]) {
                    pick = (uint32_t)(lane * 8 + j);
                    below = cum;
                    inbin = cnt[j];
                }
                cum += cnt[j];
            }
        }
        const int owner = __ffs(__ballot_sync(0xffffffffu, mine)) - 1;
        pick = __shfl_sync(0xffffffffu, pick, owner);
        below = __shfl_sync(0xffffffffu, below, owner);
        inbin = __shfl_sync(0xffffffffu, inbin, owner);
        __syncwarp();
        prefix |= (unsigned long long)pick << lo;
        rem -= below;
        if (lo > 0 && inbin == 1) {
            // a single key carries the chosen prefix: it is the answer
            const unsigned long long pm = ~0ull << lo;
            unsigned long long found = 0ull;
            for (int i = lane; i < len; i += 32)
                if ((keys[i] & pm) == prefix) found = keys[i];
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) found |= __shfl_xor_sync(0xffffffffu, found, s);
            return found;
        }
    }
    return prefix;
}

// Warp-synchronous bitonic sort of P (a power of two) 64-bit keys in the
// warp's shared memory, ascending.
__device__ __forceinline__ void warp_sort_u64(unsigned long long* key, int P) {
    const int lane = threadIdx.x & 31;
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    const unsigned long long a = key[i], b = key[ixj];
                    if (up == (b < a)) {
                        key[i] = b;
                        key[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// The n-th smallest (1-based, 1 <= n <= len) of the 64-bit keys in
// shared memory, returned to every thread. Digits of 8 bits from the
// highest bit where the keys differ; one shared histogram per pass; once the
// chosen digit holds a single key, that key is the answer.
// hist holds 256 counters; the scalars live in shared memory (*s_and holds
// the chosen digit's count after each pass).
__device__ __forceinline__ unsigned long long radix_nth_u64(const unsigned long long* keys, int len, int n,
                                                            unsigned int* hist, unsigned long long* s_and,
                                                            unsigned long long* s_or,
                                                            unsigned long long* s_prefix, unsigned int* s_rem) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        *s_and = ~0ull;
        *s_or = 0ull;
        *s_rem = (unsigned)n;
    }
    __syncthreads();
    unsigned long long a = ~0ull, o = 0ull;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        a &= keys[i];
        o |= keys[i];
    }
    atomicAnd(s_and, a);
    atomicOr(s_or, o);
    __syncthreads();
    const unsigned long long band = *s_and, diff = band ^ *s_or;
    if (diff == 0) return band;
    const int top = 63 - __clzll((long long)diff);
    if (threadIdx.x == 0) *s_prefix = top == 63 ? 0ull : (band & (~0ull << (top + 1)));
    for (int hi = top; hi >= 0; hi -= 8) {
        const int lo = hi >= 7 ? hi - 7 : 0;
        const unsigned long long himask = hi == 63 ? 0ull : (~0ull << (hi + 1));
        const unsigned dmask = (1u << (hi - lo + 1)) - 1u;
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        const unsigned long long prefix = *s_prefix;
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            const unsigned long long k = keys[i];
            if ((k & himask) == prefix) atomicAdd(&hist[(unsigned)(k >> lo) & dmask], 1u);
        }
        __syncthreads();
        uint32_t chosen = 0;
        if (w == 0) {
            uint32_t cnt[8], tot = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                cnt[j] = hist[lane * 8 + j];
                tot += cnt[j];
            }
            uint32_t incl = tot;
#pragma unroll
            for (int o2 = 1; o2 < 32; o2 <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o2);
                if (lane >= o2) incl += t;
            }
            const uint32_t excl = incl - tot;
            const uint32_t rem = *s_rem;
            const bool mine = excl < rem && rem <= incl;
            if (mine) {
                uint32_t cum = excl;
                for (int j = 0; j < 8; j++) {
                    if (cum + cnt[j] >= rem) {
                        *s_prefix = prefix | ((unsigned long long)(lane * 8 + j) << lo);
                        *s_rem = rem - cum;
                        chosen = cnt[j];
                        break;
                    }
                    cum += cnt[j];
                }
            }
            chosen = __reduce_max_sync(0xffffffffu, mine ? chosen : 0u);
            if (lane == 0) *s_and = chosen;
        }
        __syncthreads();
        // (*s_and is rewritten only after the next pass's first barrier)
        if (lo > 0 && *s_and == 1ull) {
            // a single key carries the chosen prefix: it is the answer
            const unsigned long long pm = ~0ull << lo, pf = *s_prefix;
            __syncthreads();
            for (int i = threadIdx.x; i < len; i += blockDim.x)
                if ((keys[i] & pm) == pf) *s_prefix = keys[i];
            __syncthreads();
            return *s_prefix;
        }
    }
    return *s_prefix;
}

}  // namespace hann
