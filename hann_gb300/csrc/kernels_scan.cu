// kernels_scan.cu -- the bank-conflict-free ADC list scan with warp radix
// selection, for M up to 32 (larger M use scan_kernel in kernels_search.cu).
//
// Distance: ||q - c||^2 + term + sum_m T[m][code_m], term = ||r||^2 +
// 2 <c, r> stored per row, T[m][j] = -2 <q_m, codeword_mj> the lookup table
// built per query in shared memory, in FP16 (32 KB) or FP32.
//
// Lookup table without bank conflicts. The table holds every subquantizer's
// entries two or three times over (64 half-word slots per code value, see
// adc_slot_m), so that in each step of a warp the 32 lanes read 32 distinct
// banks whatever their codes. Each row's code bytes are stored permuted for
// the lane that scans it ("scan codes", MP = M rounded up to 8 bytes a row,
// rebuilt from the codes whenever rows are placed) and blocked by groups of
// 32 rows, so a warp loads a step with contiguous 16- and 8-byte loads: 24
// bytes a row at M = 24, the codes themselves. A lookup is a byte permute
// (code byte and the lane's offset byte into a table offset), a shift, a
// 16-bit shared load and an FP16-into-FP32 add.
//
// FP16 tables and the reference's results. The FP16 entries are centred per
// subquantizer and scaled per query; every entry's rounding error is bounded,
// so a row's screened distance is within a per-query eps of the exact PQ
// distance. In parity mode the scan reports the largest screened distance it
// kept when it left rows out; the rerank proves the top k with it (the k-th
// reference distance must lie below that cut minus eps) and lists the
// queries it cannot prove, which the host scans again with FP32 tables.
//
// Selection without sorting. Each warp appends rows below the block-wide
// threshold to its buffer; a full buffer is cut back to its R smallest keys
// by a radix select on 8-bit digits (warp-private histogram), whose R-th key
// lowers the threshold. At the end warp 0 selects the query's R best from the
// warps' survivors; or, given a candidate dump, every warp leaves its buffer
// there and exits, and scan_select_kernel (one warp per query, many per SM)
// makes that selection, so the scan block's table and buffers are free for
// the next query as soon as its walk ends. Candidates leave unsorted: the
// rerank sorts them by exact distance.
#include <cuda_fp16.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace hann {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t KEY_INF = 0xff800000u;  // float_key(+inf)
__device__ __forceinline__ float pos_inf() { return __int_as_float(0x7f800000); }
constexpr int SCAN_FLAT_LISTS = 128;        // probe lists held for the balanced schedule

// A query slot of the candidate dump: keys, positions and rows of the scan
// block's warps ([WARPS][CAPW] each), then the warps' counts (bit 31: the
// warp cut its buffer back, so rows were left out).
__host__ __device__ __forceinline__ size_t dump_slot_bytes(int CAPW) {
    return ((size_t)WARPS * CAPW * 12 + WARPS * 4 + 15) / 16 * 16;
}

// A warp's buffer held in the free halves of a striped lookup table (rows of
// 256 bytes whose first 128 hold the table): element i sits in row i / 32
// of the buffer's rows, at byte 128 + 4 (i % 32).
extern __shared__ __align__(16) unsigned char scan_smem[];  // the scan kernel's dynamic shared memory
template <class T>
struct Stripe {
    uint32_t off;  // byte offset of the buffer's first element in scan_smem
    __device__ __forceinline__ T& operator[](int i) const {
        return *reinterpret_cast<T*>(scan_smem + off + ((i >> 5) << 8) + ((i & 31) << 2));
    }
};

// Keeps the `R` smallest keys of entries [0, count) (ties at the cut broken
// by position), compacted in place to [0, R). Returns through *kth a key at
// or above the R-th smallest (exactly it unless the digit holding the cut
// came out whole). hist: the warp's 256 counters. Warp-synchronous.
template <class KB, class SB, class RB, class HB>
__device__ int warp_select(KB key, SB seq, RB row, int count, int R, uint32_t* kth, HB hist) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    if (count <= R) {
        *kth = KEY_INF;
        return count;
    }
    const int nch = (count + 31) >> 5;
    uint32_t band = 0xffffffffu, bor = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        if (i < count) {
            band &= key[i];
            bor |= key[i];
        }
    }
    band = __reduce_and_sync(FULL, band);
    bor = __reduce_or_sync(FULL, bor);
    const uint32_t diff = band ^ bor;
    if (diff == 0) {
        // every key equal: keep the first R
        *kth = band;
        return R;
    }
    const int top = 31 - __clz(diff);
    uint32_t prefix = top == 31 ? 0u : (band & (0xffffffffu << (top + 1)));
    uint32_t need = (uint32_t)R;
    int L = 0;  // bits below the resolved prefix
    for (int hi = top; hi >= 0; hi -= 8) {
        const int lo = hi >= 7 ? hi - 7 : 0;
        const uint32_t himask = hi == 31 ? 0u : (0xffffffffu << (hi + 1));
        const uint32_t dmask = (1u << (hi - lo + 1)) - 1u;
#pragma unroll
        for (int b = 0; b < 8; b++) hist[b * 32 + lane] = 0;
        __syncwarp();
        for (int ch = 0; ch < nch; ch++) {
            const int i = ch * 32 + lane;
            uint32_t bin = 0xffffffffu;
            if (i < count) {
                const uint32_t kk = key[i];
                if ((kk & himask) == prefix) bin = (kk >> lo) & dmask;
            }
            const unsigned peers = __match_any_sync(FULL, bin);
            if (bin != 0xffffffffu && lane == __ffs(peers) - 1) hist[bin] += __popc(peers);
            __syncwarp();
        }
        // lane owns bins [8 lane, 8 lane + 8)
        uint32_t cnt[8], tot = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            cnt[j] = hist[lane * 8 + j];
            tot += cnt[j];
        }
        uint32_t incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const uint32_t excl = incl - tot;
        const bool mine = excl < need && need <= incl;
        uint32_t pick = 0, below = 0, inbin = 0;
        if (mine) {
            uint32_t cum = excl;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                if (cum < need && need <= cum + cnt[j]) {
                    pick = (uint32_t)(lane * 8 + j);
                    below = cum;
                    inbin = cnt[j];
                }
                cum += cnt[j];
            }
        }
        const int owner = __ffs(__ballot_sync(FULL, mine)) - 1;
        pick = __shfl_sync(FULL, pick, owner);
        below = __shfl_sync(FULL, below, owner);
        inbin = __shfl_sync(FULL, inbin, owner);
        __syncwarp();
        prefix |= pick << lo;
        need -= below;
        L = lo;
        if (inbin == need) break;  // the whole digit is kept
    }
    const uint32_t pk = L == 0 ? prefix : (prefix >> L);
    int out = 0, eq_taken = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        const bool in = i < count;
        const uint32_t kk = in ? key[i] : 0xffffffffu;
        const uint32_t ss = in ? seq[i] : 0u;
        const int32_t rr = in ? row[i] : 0;
        const uint32_t kp = L == 0 ? kk : (kk >> L);
        const bool lt_k = in && kp < pk;
        const bool eq = in && kp == pk;
        const unsigned beq = __ballot_sync(FULL, eq);
        const bool keep = lt_k || (eq && (uint32_t)(eq_taken + __popc(beq & lt)) < need);
        const unsigned bk = __ballot_sync(FULL, keep);
        const int pos = out + __popc(bk & lt);
        __syncwarp();
        if (keep) {
            key[pos] = kk;
            seq[pos] = ss;
            row[pos] = rr;
        }
        out += __popc(bk);
        eq_taken += __popc(beq);
        __syncwarp();
    }
    *kth = L == 0 ? prefix : (prefix | ((1u << L) - 1u));
    return out;
}

// Cuts a full buffer back to a superset of its R smallest keys in one pass:
// below the keys' common prefix, the 8-bit digit's histogram gives the bin
// holding the R-th smallest; every key in that bin or below stays, and *tau
// becomes the bin's (exclusive) upper edge, at or above the R-th smallest.
// Falls back to warp_select when the kept keys would pass `limit`.
// Warp-synchronous.
template <class KB, class SB, class RB, class HB>
__device__ int warp_cut(KB key, SB seq, RB row, int count, int R, int limit, uint32_t* tau, HB hist) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nch = (count + 31) >> 5;
    uint32_t band = 0xffffffffu, bor = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        if (i < count) {
            band &= key[i];
            bor |= key[i];
        }
    }
    band = __reduce_and_sync(FULL, band);
    bor = __reduce_or_sync(FULL, bor);
    const uint32_t diff = band ^ bor;
    if (diff == 0 || count <= R) return warp_select(key, seq, row, count, R, tau, hist);
    const int top = 31 - __clz(diff);
    const int lo = top >= 7 ? top - 7 : 0;
    const uint32_t dmask = (1u << (top - lo + 1)) - 1u;
#pragma unroll
    for (int b = 0; b < 8; b++) hist[b * 32 + lane] = 0;
    __syncwarp();
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        if (i < count) atomicAdd(&hist[(key[i] >> lo) & dmask], 1u);  // hist[] is a reference
    }
    __syncwarp();
    uint32_t cnt[8], tot = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        cnt[j] = hist[lane * 8 + j];
        tot += cnt[j];
    }
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t excl = incl - tot;
    const uint32_t need = (uint32_t)R;
    const bool mine = excl < need && need <= incl;
    uint32_t pick = 0, keep = 0;
    if (mine) {
        uint32_t cum = excl;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (cum < need && need <= cum + cnt[j]) {
                pick = (uint32_t)(lane * 8 + j);
                keep = cum + cnt[j];
            }
            cum += cnt[j];
        }
    }
    const int owner = __ffs(__ballot_sync(FULL, mine)) - 1;
    pick = __shfl_sync(FULL, pick, owner);
    keep = __shfl_sync(FULL, keep, owner);
    __syncwarp();
    if ((int)keep > limit) return warp_select(key, seq, row, count, R, tau, hist);
    // keys of the common prefix in bins up to pick: below prefix + (pick + 1) << lo
    const uint32_t prefix = top == 31 ? 0u : (band & (0xffffffffu << (top + 1)));
    const unsigned long long edge = (unsigned long long)prefix + ((unsigned long long)(pick + 1) << lo);
    const uint32_t bound = edge > 0xffffffffull ? 0xffffffffu : (uint32_t)edge;
    int out = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        const bool in = i < count;
        const uint32_t kk = in ? key[i] : 0xffffffffu;
        const uint32_t ss = in ? seq[i] : 0u;
        const int32_t rr = in ? row[i] : 0;
        const bool kp = in && kk < bound;
        const unsigned bk = __ballot_sync(FULL, kp);
        const int pos = out + __popc(bk & lt);
        __syncwarp();
        if (kp) {
            key[pos] = kk;
            seq[pos] = ss;
            row[pos] = rr;
        }
        out += __popc(bk);
        __syncwarp();
    }
    *tau = bound;
    return out;
}

// Lookup-table slots. A table row (one code value j) is 32 banks of two
// 16-bit halves (FP16 entries: 128 bytes) or of two 32-bit words (FP32
// entries with more than 16 subquantizers: 256 bytes, half h in the row's
// h-th 128 bytes). Slot (b, h) holds the entries of subquantizer
// adc_slot_m(b, h, MP); in step s lane l reads slot (l ^ s, s >= 16). So the
// 32 lanes of a warp read 32 distinct banks in every step whatever their
// codes, and over its MP steps each lane reads every subquantizer once
// (MP = M rounded up to 8; subquantizers at or past M have zero entries).
__host__ __device__ __forceinline__ int adc_slot_m(int b, int h, int MP) {
    if (MP == 8) return b & 7;
    if (MP == 16) return b & 15;
    if (MP == 24) return h == 0 ? (b < 16 ? b : b - 8) : (b < 16 ? (b & 7) : 16 + (b & 7));
    return b;
}

// The slots of subquantizer m (at most four): banks b[], halves hh[].
__device__ __forceinline__ int adc_slots(int m, int MP, int* b, int* hh) {
    if (MP == 8) {
        for (int i = 0; i < 4; i++) {
            b[i] = m + 8 * i;
            hh[i] = 0;
        }
        return 4;
    }
    if (MP == 16) {
        b[0] = m;
        b[1] = m + 16;
        hh[0] = hh[1] = 0;
        return 2;
    }
    if (MP == 24) {
        if (m >= 8 && m < 16) {
            b[0] = m;
            b[1] = m + 8;
            hh[0] = hh[1] = 0;
            return 2;
        }
        b[0] = m < 8 ? m : m + 8;
        hh[0] = 0;
        b[1] = m;
        b[2] = m + 8;
        hh[1] = hh[2] = 1;
        return 3;
    }
    b[0] = b[1] = m;
    hh[0] = 0;
    hh[1] = 1;
    return 2;
}

// Position of step s's code byte of lane l in a group of 32 rows: planes of
// 16 bytes per lane, then a plane of 8 bytes per lane when MP is an odd
// multiple of 8, so a lane loads its row with one 16-byte load per full
// plane (and one 8-byte load) and the warp's loads are contiguous.
__host__ __device__ __forceinline__ int adc_code_pos(int l, int s, int MP) {
    const int full = MP / 16;
    return (s >> 4) < full ? 512 * (s >> 4) + 16 * l + (s & 15) : 512 * full + 8 * l + (s & 7);
}

// TAB: 0 FP32 entries, 1 FP16, 2 16-bit fixed point. STRIPED (16-bit
// entries only): 256-byte table rows whose second halves hold the warps'
// candidate buffers and histograms (one warp buffer of 256 entries, a rerank
// depth of at most 96), so that a table offset is the byte permute's result
// with no shift; otherwise 16-bit entries sit in 128-byte rows.
template <int MP, int TAB, bool STRIPED>
__global__ void __launch_bounds__(THREADS, 3) scan_adc_kernel(ScanParams p, const float* __restrict__ Q,
                                                           const float* __restrict__ probe_d,
                                                           const int32_t* __restrict__ probe_ids,
                                                           const int32_t* __restrict__ nprobe, int np_max,
                                                           const int32_t* __restrict__ fallback, int R, int CAPW,
                                                           int32_t* __restrict__ cand_row,
                                                           float* __restrict__ cand_d,
                                                           uint32_t* __restrict__ cand_seq,
                                                           unsigned long long* __restrict__ rows_scanned) {
    constexpr bool HALF = TAB >= 1;             // 16-bit entries
    constexpr bool FIXED = TAB == 2;
    static_assert(HALF || !STRIPED, "striped tables hold 16-bit entries");
    constexpr bool WIDE = !HALF && MP > 16;     // FP32 entries, 256-byte rows
    constexpr int ROWB = (WIDE || STRIPED) ? 256 : 128;  // bytes per table row
    constexpr int LUT_BYTES = ROWB * 256;
    constexpr int SHIFT = ROWB == 128 ? 1 : 0;  // table offset = (code * 256 + offset byte) >> SHIFT
    constexpr int NW = MP / 4;                  // code words per row
    constexpr int NOB = (MP + 2) / 3;           // offset registers: three offset bytes and a zero byte
    constexpr int G = 32;
    unsigned char* const smraw = scan_smem;
    unsigned char* lutb = smraw;
    // flat layout: [table][warp buffers][merge region][histograms];
    // striped: [table with buffers and histograms][merge region]
    uint32_t* wkey = reinterpret_cast<uint32_t*>(smraw + LUT_BYTES);
    uint32_t* wseq = wkey + (STRIPED ? 0 : WARPS * CAPW);
    int32_t* wrow = reinterpret_cast<int32_t*>(wseq + (STRIPED ? 0 : WARPS * CAPW));
    uint32_t* mkey = reinterpret_cast<uint32_t*>(wrow + (STRIPED ? 0 : WARPS * CAPW));  // [WARPS * R] merge region
    uint32_t* mseq = mkey + WARPS * R;
    int32_t* mrow = reinterpret_cast<int32_t*>(mseq + WARPS * R);
    uint32_t* whist = reinterpret_cast<uint32_t*>(mrow + WARPS * R);   // [WARPS][256] (flat layout)
    __shared__ uint32_t s_tau;
    __shared__ int s_big, s_dropped;
    __shared__ int s_wcount[WARPS];
    __shared__ int s_lstart[SCAN_FLAT_LISTS], s_lsw[SCAN_FLAT_LISTS];
    __shared__ int s_llen[SCAN_FLAT_LISTS], s_lsteps[SCAN_FLAT_LISTS + 1];
    __shared__ float s_lbase[SCAN_FLAT_LISTS];
    __shared__ float s_eps;
    const int M = p.M;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // The table build's first round of codeword loads (eight a lane) goes
    // out before anything that waits on the query, so its latency overlaps
    // the query's own loads.
    constexpr int U = 8;
    const float* cb = HALF ? p.adc_cb : p.codebooks_t;  // [pqK][M][dsub]
    const bool cb4 = p.dsub == 4 && (reinterpret_cast<uintptr_t>(cb) & 15) == 0;
    float4 cpre[U];
    if (lane < M && cb4) {
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int j = w + u * WARPS;
            if (j < p.pqK) cpre[u] = __ldg(reinterpret_cast<const float4*>(cb) + (int64_t)j * M + lane);
        }
    }
    if (p.qcount && (int)blockIdx.x >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[blockIdx.x] : blockIdx.x;
    const float* qv = Q + q * p.dim;
    const bool v4 = cb4 && (reinterpret_cast<uintptr_t>(qv) & 15) == 0;
    float4 qa = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (lane < M && v4) qa = __ldg(reinterpret_cast<const float4*>(qv) + lane);
    // 16-bit tables with every coordinate in some lane's float4: the query's
    // norm and its dot product with the subquantizers' means come from the
    // lanes' float4s (their mean coordinates loaded beside them)
    const bool vfull = HALF && v4 && M * 4 == p.dim && (reinterpret_cast<uintptr_t>(p.adc_mu) & 15) == 0;
    float4 mu4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (lane < M && vfull) mu4 = __ldg(reinterpret_cast<const float4*>(p.adc_mu) + lane);
    if (tid == 0) {
        s_tau = KEY_INF;
        s_big = 0;
        s_dropped = 0;
    }
    // Every warp works out the table's scale for itself (the same values in
    // each), so the build needs no barrier before it.
    float scale = 1.0f, inv = 1.0f, c0 = 0.0f;
    if (HALF) {
        // 16-bit entries of -2 <q_m, c_mj - mu_m>, |.| <= b_m = 2 ||q_m||
        // max_j ||c_mj - mu_m||; the means' part, -2 <q, mu>, joins each
        // list's base. FP16: scaled by 2^e so that the largest b_m is at most
        // 2^15; rounding one entry errs by at most 2^-11 of b_m (2^-25 below
        // FP16's normal range). Fixed point: integers of the entry times
        // 32767 / max_m b_m, rounded to nearest (at most half a unit, and a
        // row's sum of them is exact in 32-bit integers). Either way a row's
        // screened distance is within eps of the exact sum (with a relative
        // allowance for the FP32 roundings of the decomposition).
        float bm = 0.0f, qq = 0.0f;
        if (lane < M) {
            const float rm = p.adc_rm[lane];
            if (v4) {
                qq = fmaf(qa.x, qa.x, qq);
                qq = fmaf(qa.y, qa.y, qq);
                qq = fmaf(qa.z, qa.z, qq);
                qq = fmaf(qa.w, qa.w, qq);
            } else {
                for (int t = 0; t < p.dsub; t++) qq = fmaf(qv[lane * p.dsub + t], qv[lane * p.dsub + t], qq);
            }
            bm = 2.0f * sqrtf(qq) * rm;
        }
        float mx = bm, sum = bm, cq = 0.0f, qn = 0.0f;
        if (vfull) {
            qn = qq;
            cq = fmaf(qa.x, mu4.x, cq);
            cq = fmaf(qa.y, mu4.y, cq);
            cq = fmaf(qa.z, mu4.z, cq);
            cq = fmaf(qa.w, mu4.w, cq);
        } else {
            for (int e = lane; e < p.dim; e += 32) {
                cq = fmaf(qv[e], p.adc_mu[e], cq);
                qn = fmaf(qv[e], qv[e], qn);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
            sum += __shfl_xor_sync(FULL, sum, o);
            cq += __shfl_xor_sync(FULL, cq, o);
            qn += __shfl_xor_sync(FULL, qn, o);
        }
        const bool finite = mx > 0.0f && mx < pos_inf();
        float round_err;
        if (FIXED) {
            scale = finite ? 32767.0f / mx : 1.0f;
            inv = 1.0f / scale;
            round_err = (float)MP * 0.51f * inv;
        } else {
            int ex = 0;
            if (finite) frexpf(mx, &ex);
            const int e = finite ? max(-120, min(120, 15 - ex)) : 0;
            scale = ldexpf(1.0f, e);
            inv = ldexpf(1.0f, -e);
            round_err = 4.8828125e-4f * sum + (float)MP * 2.98023224e-8f * inv;
        }
        c0 = -2.0f * cq;
        if (tid == 0)
            s_eps = round_err + 1e-5f * (2.0f * sqrtf(qn) * p.adc_rfull + p.adc_tbound + 2.0f * fabsf(cq));
    }
    {
        // Table build: warp w takes code values w, w + 8, ...; lane l < M
        // computes subquantizer l's entry and writes it to each of its slots.
        // Eight codeword loads are in flight per lane (the codebooks come
        // from L2: shared memory leaves L1 little room).
        int bs[4] = {0, 0, 0, 0}, hs[4] = {0, 0, 0, 0};
        const int ns = lane < M ? adc_slots(lane, MP, bs, hs) : 0;
        auto put = [&](int j, float acc) {
            if (FIXED) {
                const int qi = max(-32767, min(32767, __float2int_rn(-2.0f * acc * scale)));
                for (int i = 0; i < ns; i++)
                    *reinterpret_cast<short*>(lutb + j * ROWB + 4 * bs[i] + 2 * hs[i]) = (short)qi;
            } else if (HALF) {
                const __half hv = __float2half_rn(-2.0f * acc * scale);
                for (int i = 0; i < ns; i++) *reinterpret_cast<__half*>(lutb + j * ROWB + 4 * bs[i] + 2 * hs[i]) = hv;
            } else {
                const float v = -2.0f * acc;
                for (int i = 0; i < ns; i++)
                    *reinterpret_cast<float*>(lutb + j * ROWB + 4 * bs[i] + 128 * hs[i]) = v;
            }
        };
        if (lane < M && v4) {
            // code values j0, j0 + WARPS, ... (U of them) from codewords c
            auto round = [&](int j0, const float4 (&c)[U]) {
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int j = j0 + u * WARPS;
                    if (j < p.pqK) {
                        float acc = 0.0f;
                        acc = fmaf(qa.x, c[u].x, acc);
                        acc = fmaf(qa.y, c[u].y, acc);
                        acc = fmaf(qa.z, c[u].z, acc);
                        acc = fmaf(qa.w, c[u].w, acc);
                        put(j, acc);
                    }
                }
            };
            round(w, cpre);
            for (int j0 = w + WARPS * U; j0 < p.pqK; j0 += WARPS * U) {
                float4 c[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int j = j0 + u * WARPS;
                    if (j < p.pqK) c[u] = __ldg(reinterpret_cast<const float4*>(cb) + (int64_t)j * M + lane);
                }
                round(j0, c);
            }
        } else if (lane < M) {
            const float* qm = qv + lane * p.dsub;
            for (int j = w; j < p.pqK; j += WARPS) {
                const float* cw = cb + ((int64_t)j * M + lane) * p.dsub;
                float acc = 0.0f;
                for (int t = 0; t < p.dsub; t++) acc = fmaf(qm[t], cw[t], acc);
                put(j, acc);
            }
        }
        // subquantizers past M (their codes are 0): zero entries
        for (int m = M + tid; m < MP; m += THREADS) {
            int b2[4], h2[4];
            const int n2 = adc_slots(m, MP, b2, h2);
            for (int i = 0; i < n2; i++) {
                if (HALF) *reinterpret_cast<unsigned short*>(lutb + 4 * b2[i] + 2 * h2[i]) = 0;
                else *reinterpret_cast<float*>(lutb + 4 * b2[i] + 128 * h2[i]) = 0.0f;
            }
        }
    }
    // the lane's table offset bytes, three to a register (the fourth byte
    // zero): offset byte of step s = the in-row offset of slot (lane ^ s,
    // s >= 16) << SHIFT
    uint32_t ob[NOB];
#pragma unroll
    for (int i = 0; i < NOB; i++) {
        uint32_t v = 0;
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            const int s = 3 * i + kk;
            if (s < MP) {
                const uint32_t b = (uint32_t)(lane ^ s), hh = s >= 16 ? 1u : 0u;
                const uint32_t io = HALF ? 4u * b + 2u * hh : 4u * b + 128u * hh;  // in-row offset
                const uint32_t o = io << SHIFT;
                v |= o << (8 * kk);
            }
        }
        ob[i] = v;
    }
    __syncthreads();
    // warp w's buffers: flat, or rows 24 w.. (keys, positions, rows: eight
    // rows of 32 each) and 192 + 8 w.. (histogram) of the striped table
    using KB = typename std::conditional<STRIPED, Stripe<uint32_t>, uint32_t*>::type;
    using RB = typename std::conditional<STRIPED, Stripe<int32_t>, int32_t*>::type;
    KB key, seq, hist;
    RB row;
    if constexpr (STRIPED) {
        key = KB{(uint32_t)(128 + (24 * w) * 256)};
        seq = KB{(uint32_t)(128 + (24 * w + 8) * 256)};
        row = RB{(uint32_t)(128 + (24 * w + 16) * 256)};
        hist = KB{(uint32_t)(128 + (192 + 8 * w) * 256)};
    } else {
        key = wkey + w * CAPW;
        seq = wseq + w * CAPW;
        row = wrow + w * CAPW;
        hist = whist + w * 256;
    }
    const bool fb = fallback[q] != 0;
    const int nl = fb ? p.nlist : min(nprobe[q], p.nlist);
    const unsigned ltm = (1u << lane) - 1u;
    int count = 0;
    unsigned long long scanned = 0;
    auto list_meta = [&](int i, int64_t& start, int64_t& sws, int& len, float& base) {
        const int l = fb ? i : probe_ids[q * np_max + i];
        if (fb) {
            float part = 0.0f;
            for (int j = lane; j < p.dim; j += 32) {
                const float t = qv[j] - p.coarse[(int64_t)l * p.dim + j];
                part = fmaf(t, t, part);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(FULL, part, o);
            base = part + c0;
        } else {
            base = probe_d[q * np_max + i] + c0;
        }
        start = p.list_start[l];
        sws = p.sw_start[l];
        len = p.list_len[l];
    };
    // one step's code words of the lane's row; gp: the group's first byte
    auto load_codes = [&](const uint8_t* gp, uint32_t (&cw)[NW]) {
#pragma unroll
        for (int pl = 0; pl < MP / 16; pl++) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(gp + 512 * pl) + lane);
            cw[4 * pl] = v.x;
            cw[4 * pl + 1] = v.y;
            cw[4 * pl + 2] = v.z;
            cw[4 * pl + 3] = v.w;
        }
        if (MP % 16) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(gp + 512 * (MP / 16)) + lane);
            cw[NW - 2] = v.x;
            cw[NW - 1] = v.y;
        }
    };
    // A lookup is one byte permute (code byte and offset byte into a table
    // offset; plus a shift in 128-byte rows), one shared load and an add:
    // FP32 and FP16 entries into four FP32 partial sums, fixed-point entries
    // two at a time into two integer sums (three-input adds).
    auto lookup = [&](const uint32_t (&cw)[NW], float bt) {
        if constexpr (FIXED) {
            int acc[2] = {0, 0};
#pragma unroll
            for (int s = 0; s < MP; s += 2) {
                const uint32_t sa = (uint32_t)(4 + s % 3) | ((uint32_t)(s % 4) << 4) | 0x7700u;
                const uint32_t sb = (uint32_t)(4 + (s + 1) % 3) | ((uint32_t)((s + 1) % 4) << 4) | 0x7700u;
                const uint32_t a = __byte_perm(cw[s / 4], ob[s / 3], sa) >> SHIFT;
                const uint32_t b = __byte_perm(cw[(s + 1) / 4], ob[(s + 1) / 3], sb) >> SHIFT;
                const int x = *reinterpret_cast<const short*>(lutb + a);
                const int y = *reinterpret_cast<const short*>(lutb + b);
                acc[(s >> 1) & 1] += x + y;
            }
            return float_key(fmaf((float)(acc[0] + acc[1]), inv, bt));
        }
        float part[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int s = 0; s < MP; s++) {
            const uint32_t sel = (uint32_t)(4 + s % 3) | ((uint32_t)(s % 4) << 4) | 0x7700u;
            const uint32_t a = __byte_perm(cw[s / 4], ob[s / 3], sel) >> SHIFT;
            if (HALF) {
                const unsigned short hb = *reinterpret_cast<const unsigned short*>(lutb + a);
                asm("add.rn.f32.f16 %0, %1, %0;" : "+f"(part[s & 3]) : "h"(hb));
            } else {
                part[s & 3] += *reinterpret_cast<const float*>(lutb + a);
            }
        }
        return float_key(fmaf((part[0] + part[1]) + (part[2] + part[3]), inv, bt));
    };
    bool cut = false;  // this warp cut its buffer back (rows were left out)
    auto cut_back = [&]() {
        __syncwarp();
        cut = true;
        uint32_t kth;
        count = warp_cut(key, seq, row, count, R, CAPW / 2, &kth, hist);
        if (lane == 0) {
            atomicMin(&s_tau, kth);
            s_dropped = 1;
        }
        __syncwarp();
    };
    auto offer = [&](uint32_t k, int li, int64_t grow) {
        const bool pass = k < *(volatile uint32_t*)&s_tau;
        const unsigned bal = __ballot_sync(FULL, pass);
        if (bal) {
            const int pos = count + __popc(bal & ltm);
            if (pass) {
                key[pos] = k;
                seq[pos] = (uint32_t)li;
                row[pos] = (int32_t)grow;
            }
            count += __popc(bal);
            if (count > CAPW - 32) cut_back();
        }
    };
    bool flat = !fb && nl <= SCAN_FLAT_LISTS;
    if (flat) {
        // Balanced schedule: the probed lists' steps (G rows each) are
        // numbered in probe order and split into equal contiguous ranges,
        // one per warp, so every warp gets the same number of rows to within
        // one step whatever the list sizes. Lists of nearly 2^24 rows (whose
        // positions do not fit a step's tag) take the list-by-list walk.
        for (int i = tid; i < nl; i += THREADS) {
            const int l = probe_ids[q * np_max + i];
            s_lstart[i] = (int)p.list_start[l];
            s_lsw[i] = (int)p.sw_start[l];
            const int len = p.list_len[l];
            s_llen[i] = len;
            s_lbase[i] = probe_d[q * np_max + i] + c0;
            s_lsteps[i] = (len + G - 1) / G;
            if (len > (1 << 24) - G) s_big = 1;
        }
        __syncthreads();
        flat = s_big == 0;
    }
    if (flat) {
        if (w == 0) {
            // exclusive prefix of the step counts into s_lsteps (in place)
            int carry = 0;
            for (int b = 0; b < nl; b += 32) {
                const int i = b + lane;
                const int v = i < nl ? s_lsteps[i] : 0;
                int incl = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += t;
                }
                if (i < nl) s_lsteps[i] = carry + incl - v;
                carry += __shfl_sync(FULL, incl, 31);
            }
            if (lane == 0) s_lsteps[nl] = carry;
            if (lane == 0 && rows_scanned) {
                unsigned long long tot = 0;
                for (int i = 0; i < nl; i++) tot += (unsigned long long)s_llen[i];
                scanned = tot;
            }
        }
        __syncthreads();
        // Warp w takes n contiguous steps from ub in the probe-order
        // numbering (every warp within one step of the same count) and walks
        // them with a cursor held in registers: list, its boundary, the
        // lane's row in it and the group's code bytes.
        const int total = s_lsteps[nl];
        const int per = total / WARPS, rem = total % WARPS;
        const int ub = w * per + min(w, rem);
        const int n = per + (w < rem ? 1 : 0);
        if (n > 0) {
            int cl;
            {
                int lo = 0, hi = nl - 1;  // the last list starting at or before ub
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_lsteps[mid] <= ub) lo = mid;
                    else hi = mid - 1;
                }
                cl = lo;
            }
            int cu = ub, cend = s_lsteps[cl + 1], crow = (ub - s_lsteps[cl]) * G + lane;
            int clen = s_llen[cl];
            const float* cterm = p.term + s_lstart[cl];
            const uint8_t* cgp = p.scanc + ((int64_t)s_lsw[cl] + (int64_t)(ub - s_lsteps[cl]) * G) * MP;
            // A step in flight: its code words, its term (+inf past the
            // list's end, where the codes are not initialised and the lookup
            // is skipped) and tag = probe position << 24 | row position.
            auto load_step = [&](uint32_t (&cw)[NW], float& term, int& tag) {
                load_codes(cgp, cw);
                term = crow < clen ? __ldg(cterm + crow) : pos_inf();
                tag = (cl << 24) | crow;
                cu++;
                if (cu < cend) {
                    crow += G;
                    cgp += G * MP;
                } else if (cu < ub + n) {
                    do {
                        cl++;
                    } while (s_lsteps[cl + 1] <= cu);
                    cend = s_lsteps[cl + 1];
                    crow = lane;
                    clen = s_llen[cl];
                    cterm = p.term + s_lstart[cl];
                    cgp = p.scanc + (int64_t)s_lsw[cl] * MP;
                }
            };
            auto offer_tag = [&](uint32_t k, int tag) {
                const bool pass = k < *(volatile uint32_t*)&s_tau;
                const unsigned bal = __ballot_sync(FULL, pass);
                if (bal) {
                    const int pos = count + __popc(bal & ltm);
                    if (pass) {
                        const int li = tag >> 24;
                        key[pos] = k;
                        seq[pos] = (uint32_t)li;
                        row[pos] = s_lstart[li] + (tag & 0xffffff);
                    }
                    count += __popc(bal);
                    if (count > CAPW - 32) cut_back();
                }
            };
            // Two steps in a ring: a step's codes are loaded one step before
            // it is computed.
            uint32_t cw[2][NW];
            float tm[2];
            int tg[2];
            load_step(cw[0], tm[0], tg[0]);
            if (n > 1) load_step(cw[1], tm[1], tg[1]);
            for (int i = 0; i < n; i += 2) {
#pragma unroll
                for (int d = 0; d < 2; d++) {
                    if (i + d >= n) break;
                    const int g0 = tg[d];
                    const uint32_t k = tm[d] < pos_inf() ? lookup(cw[d], s_lbase[g0 >> 24] + tm[d]) : KEY_INF;
                    if (i + d + 2 < n) load_step(cw[d], tm[d], tg[d]);
                    offer_tag(k, g0);
                }
            }
        }
    } else {
        // Fallback queries and very long probe lists: every WARPS-th list per
        // warp, the next step loaded before the current is computed.
        for (int li = w; li < nl; li += WARPS) {
            int64_t start, sws;
            int len;
            float base;
            list_meta(li, start, sws, len, base);
            scanned += (unsigned long long)len;
            const uint8_t* gp = p.scanc + sws * MP;
            uint32_t ca[NW], cbw[NW];
            float ta = 0.0f, tb = 0.0f;
            bool va = lane < len;
            if (va) {
                load_codes(gp, ca);
                ta = __ldg(p.term + start + lane);
            }
            for (int st = 0; st * G < len; st += 2) {
                const int r0 = st * G;
                const bool vb = r0 + G + lane < len;
                if (vb) {
                    load_codes(gp + (int64_t)(st + 1) * G * MP, cbw);
                    tb = __ldg(p.term + start + r0 + G + lane);
                }
                offer(va ? lookup(ca, base + ta) : KEY_INF, li, start + r0 + lane);
                if (r0 + G >= len) break;
                va = r0 + 2 * G + lane < len;
                if (va) {
                    load_codes(gp + (int64_t)(st + 2) * G * MP, ca);
                    ta = __ldg(p.term + start + r0 + 2 * G + lane);
                }
                offer(vb ? lookup(cbw, base + tb) : KEY_INF, li, start + r0 + G + lane);
            }
        }
    }
    if (p.dump) {
        // Each warp leaves its candidates for scan_select_kernel and ends
        // here: the block's life is its walk, with no barrier or selection.
        // Candidates above the block's current threshold are left out: some
        // warp holds at least R candidates at or below every value the
        // threshold takes, so the query's best R are all at or below it.
        __syncwarp();
        const uint32_t tau_end = *(volatile uint32_t*)&s_tau;
        uint32_t* dk = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(p.dump) +
                                                   (size_t)blockIdx.x * dump_slot_bytes(CAPW));
        uint32_t* ds = dk + WARPS * CAPW;
        int32_t* dr = reinterpret_cast<int32_t*>(ds + WARPS * CAPW);
        int32_t* dc = dr + WARPS * CAPW;
        int kept = 0;
        for (int i0 = 0; i0 < count; i0 += 32) {
            const int i = i0 + lane;
            const uint32_t kk = i < count ? key[i] : 0xffffffffu;
            const bool keep = i < count && kk <= tau_end;
            const unsigned bk = __ballot_sync(FULL, keep);
            if (keep) {
                const int pos = w * CAPW + kept + __popc(bk & ltm);
                dk[pos] = kk;
                ds[pos] = seq[i];
                dr[pos] = row[i];
            }
            kept += __popc(bk);
        }
        if (lane == 0) {
            dc[w] = (int32_t)((uint32_t)kept | (cut || kept < count ? 0x80000000u : 0u));
            if (rows_scanned) atomicAdd(rows_scanned, scanned);
        }
        if (HALF && p.scan_cut && tid == 0) p.scan_eps[q] = s_eps;
        return;
    }
    __syncwarp();
    {
        uint32_t kth;
        const int before = count;
        count = warp_select(key, seq, row, count, R, &kth, hist);
        if (lane == 0) {
            s_wcount[w] = count;
            if (before > count) s_dropped = 1;
            if (rows_scanned) atomicAdd(rows_scanned, scanned);
        }
    }
    __syncthreads();
    int off = 0, total = 0;
    for (int ww = 0; ww < WARPS; ww++) {
        if (ww < w) off += s_wcount[ww];
        total += s_wcount[ww];
    }
    for (int i = lane; i < count; i += 32) {
        mkey[off + i] = key[i];
        mseq[off + i] = seq[i];
        mrow[off + i] = row[i];
    }
    __syncthreads();
    if (w == 0) {
        uint32_t kth;
        const int Rq = p.kq ? min(R, rerank_depth_for(p.kq[q], p.mode, p.rerank_fixed)) : R;
        const int kept = warp_select(mkey, mseq, mrow, total, Rq, &kth, hist);
        uint32_t kmax = 0;
        for (int i = lane; i < R; i += 32) {
            const bool ok = i < kept;
            cand_row[q * R + i] = ok ? mrow[i] : -1;
            cand_d[q * R + i] = ok ? key_float(mkey[i]) : __int_as_float(0x7f800000);
            cand_seq[q * R + i] = ok ? mseq[i] : 0xffffffffu;
            if (ok) kmax = max(kmax, mkey[i]);
        }
        if (HALF && p.scan_cut) {
            // Every row left out has a screened distance at or above the
            // largest kept one: the rerank proves the top k with it.
            kmax = __reduce_max_sync(FULL, kmax);
            const bool dropped = s_dropped != 0 || total > kept;
            if (lane == 0) {
                p.scan_cut[q] = dropped && kept > 0 ? key_float(kmax) : pos_inf();
                p.scan_eps[q] = s_eps;
            }
        }
    }
}

// The end of a table scan run with a candidate dump: per query slot b, the
// query's best Rq of the candidates the scan block's warps left, taken in
// warp order then position (ties at the cut broken by that order, as the
// block's own selection breaks them), written to the candidate slots the
// rerank reads, with the parity-mode cut. One warp per slot, many slots per
// SM. The slot's keys are staged in shared memory first (eight segments, all
// loads in flight at once); the radix select runs there, and only the kept
// entries' rows and positions are read from the dump.
constexpr int SEL_WARPS = 4;
size_t select_smem(int CAPW, int R) { return (size_t)SEL_WARPS * (WARPS * CAPW + R) * sizeof(uint32_t); }

__global__ void __launch_bounds__(SEL_WARPS * 32) scan_select_kernel(ScanParams p, int64_t nslots, int R, int CAPW,
                                                                     int32_t* __restrict__ cand_row,
                                                                     float* __restrict__ cand_d,
                                                                     uint32_t* __restrict__ cand_seq) {
    extern __shared__ uint32_t sel_keys[];  // [SEL_WARPS][WARPS * CAPW + R]: staged keys, kept entries' sources
    __shared__ uint32_t hist_all[SEL_WARPS][256];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t b = (int64_t)blockIdx.x * SEL_WARPS + wl;
    if (b >= nslots) return;
    if (p.qcount && b >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[b] : b;
    const uint32_t* dk = reinterpret_cast<const uint32_t*>(static_cast<const unsigned char*>(p.dump) +
                                                           (size_t)b * dump_slot_bytes(CAPW));
    const uint32_t* ds = dk + WARPS * CAPW;
    const int32_t* dr = reinterpret_cast<const int32_t*>(ds + WARPS * CAPW);
    const int32_t* dc = dr + WARPS * CAPW;
    uint32_t* key = sel_keys + (size_t)wl * (WARPS * CAPW + R);
    int32_t* src_of = reinterpret_cast<int32_t*>(key + WARPS * CAPW);  // [R] dump index of each kept entry
    uint32_t* hist = &hist_all[wl][0];
    // the warps' counts (bit 31: that warp cut its buffer back) and where
    // each segment starts in the staged order
    const uint32_t c0 = lane < WARPS ? (uint32_t)__ldg(dc + lane) : 0u;
    const bool dropped_any = __any_sync(FULL, (c0 >> 31) != 0);
    int c[WARPS], off[WARPS], total = 0;
#pragma unroll
    for (int w = 0; w < WARPS; w++) {
        c[w] = (int)(__shfl_sync(FULL, c0, w) & 0x7fffffffu);
        off[w] = total;
        total += c[w];
    }
    {
        // 128 entries of every segment at a time, all their loads in flight
        constexpr int PER = 4;
        int cmax = 0;
#pragma unroll
        for (int w = 0; w < WARPS; w++) cmax = max(cmax, c[w]);
        for (int i0 = 0; i0 < cmax; i0 += 32 * PER) {
            uint32_t v[WARPS][PER];
#pragma unroll
            for (int w = 0; w < WARPS; w++)
#pragma unroll
                for (int u = 0; u < PER; u++) {
                    const int i = i0 + 32 * u + lane;
                    v[w][u] = i < c[w] ? __ldg(dk + w * CAPW + i) : 0u;
                }
#pragma unroll
            for (int w = 0; w < WARPS; w++)
#pragma unroll
                for (int u = 0; u < PER; u++) {
                    const int i = i0 + 32 * u + lane;
                    if (i < c[w]) key[off[w] + i] = v[w][u];
                }
        }
    }
    __syncwarp();
    const int Rq = p.kq ? min(R, rerank_depth_for(p.kq[q], p.mode, p.rerank_fixed)) : R;
    // Radix select on 8-bit digits below the keys' common prefix: pk (the
    // pivot's top bits, L bits below dropped) and need (keys equal to it that
    // stay). Every key stays when there are at most Rq.
    uint32_t pk = 0xffffffffu, need = 0xffffffffu;
    int L = 0;
    bool all = total <= Rq;
    if (!all) {
        uint32_t band = 0xffffffffu, bor = 0;
        for (int i = lane; i < total; i += 32) {
            band &= key[i];
            bor |= key[i];
        }
        band = __reduce_and_sync(FULL, band);
        bor = __reduce_or_sync(FULL, bor);
        const uint32_t diff = band ^ bor;
        uint32_t prefix = band;
        need = (uint32_t)Rq;
        if (diff != 0) {
            const int top = 31 - __clz(diff);
            prefix = top == 31 ? 0u : (band & (0xffffffffu << (top + 1)));
            for (int hi = top; hi >= 0; hi -= 8) {
                const int lo = hi >= 7 ? hi - 7 : 0;
                const uint32_t himask = hi == 31 ? 0u : (0xffffffffu << (hi + 1));
                const uint32_t dmask = (1u << (hi - lo + 1)) - 1u;
#pragma unroll
                for (int j = 0; j < 8; j++) hist[j * 32 + lane] = 0;
                __syncwarp();
                for (int i0 = 0; i0 < total; i0 += 32) {
                    const int i = i0 + lane;
                    uint32_t bin = 0xffffffffu;
                    if (i < total) {
                        const uint32_t kk = key[i];
                        if ((kk & himask) == prefix) bin = (kk >> lo) & dmask;
                    }
                    const unsigned peers = __match_any_sync(FULL, bin);
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
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o) incl += t;
                }
                const uint32_t excl = incl - tot;
                const bool mine = excl < need && need <= incl;
                uint32_t pick = 0, below = 0, inbin = 0;
                if (mine) {
                    uint32_t cum = excl;
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (cum < need && need <= cum + cnt[j]) {
                            pick = (uint32_t)(lane * 8 + j);
                            below = cum;
                            inbin = cnt[j];
                        }
                        cum += cnt[j];
                    }
                }
                const int owner = __ffs(__ballot_sync(FULL, mine)) - 1;
                pick = __shfl_sync(FULL, pick, owner);
                below = __shfl_sync(FULL, below, owner);
                inbin = __shfl_sync(FULL, inbin, owner);
                __syncwarp();
                prefix |= pick << lo;
                need -= below;
                L = lo;
                if (inbin == need) break;  // the whole digit stays
            }
        }
        pk = L == 0 ? prefix : (prefix >> L);
    }
    // The kept entries in staged order, compacted in place (each chunk read
    // before it is written, never past its source) with their dump indices
    // (segment w's entry i sits at staged index off[w] + i); then their rows
    // and positions are read from the dump, all loads in flight together.
    int out = 0;
    uint32_t eq_taken = 0, kmax = 0;
    for (int i0 = 0; i0 < total; i0 += 32) {
        const int i = i0 + lane;
        const bool in = i < total;
        const uint32_t kk = in ? key[i] : 0xffffffffu;
        const uint32_t kp = L == 0 ? kk : (kk >> L);
        const bool eq = in && !all && kp == pk;
        const unsigned beq = __ballot_sync(FULL, eq);
        const bool keep = in && (all || kp < pk || (eq && eq_taken + __popc(beq & lt) < need));
        const unsigned bk = __ballot_sync(FULL, keep);
        __syncwarp();
        if (keep) {
            int w = 0;
#pragma unroll
            for (int ww = 1; ww < WARPS; ww++) w += i >= off[ww] ? 1 : 0;
            const int pos = out + __popc(bk & lt);
            key[pos] = kk;
            src_of[pos] = w * CAPW + (i - off[w]);
            kmax = max(kmax, kk);
        }
        out += __popc(bk);
        eq_taken += __popc(beq);
        __syncwarp();
    }
    for (int i0 = 0; i0 < R; i0 += 32 * 4) {
        int32_t rr[4];
        uint32_t ss[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = i0 + 32 * u + lane;
            rr[u] = -1;
            ss[u] = 0xffffffffu;
            if (i < out) {
                rr[u] = __ldg(dr + src_of[i]);
                ss[u] = __ldg(ds + src_of[i]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int i = i0 + 32 * u + lane;
            if (i < R) {
                cand_row[q * R + i] = rr[u];
                cand_d[q * R + i] = i < out ? key_float(key[i]) : pos_inf();
                cand_seq[q * R + i] = ss[u];
            }
        }
    }
    if (p.scan_cut) {
        // every row left out screened at or above the largest kept one
        kmax = __reduce_max_sync(FULL, kmax);
        if (lane == 0) p.scan_cut[q] = (dropped_any || total > out) && out > 0 ? key_float(kmax) : pos_inf();
    }
}

// Scan codes of rows: for the row at position pos of its list (group
// pos / 32, lane l = pos mod 32), byte s is the code of the subquantizer lane
// l reads in step s (0 past M), at adc_code_pos(l, s, MP) in the group. A
// list's codes start at slot sw_start (MP bytes per slot).
__device__ __forceinline__ void write_scan_codes(const uint8_t* __restrict__ codes, int M, int MP, int pos,
                                                 uint8_t* __restrict__ list_codes) {
    const int g = pos >> 5, l = pos & 31;
    uint8_t* gp = list_codes + (int64_t)g * 32 * MP;
    for (int s = 0; s < MP; s++) {
        const int m = adc_slot_m(l ^ s, s >= 16 ? 1 : 0, MP);
        gp[adc_code_pos(l, s, MP)] = m < M ? codes[m] : (uint8_t)0;
    }
}

// One block per list: every slot in [start, start + len).
__global__ void scan_codes_lists_kernel(const uint8_t* __restrict__ codes, int code_stride, int M, int MP,
                                        const int64_t* __restrict__ list_start, const int32_t* __restrict__ list_len,
                                        const int64_t* __restrict__ sw_start, uint8_t* __restrict__ scanc) {
    const int l = blockIdx.x;
    const int64_t start = list_start[l];
    const int len = list_len[l];
    uint8_t* out = scanc + sw_start[l] * MP;
    for (int j = threadIdx.x; j < len; j += blockDim.x) write_scan_codes(codes + (start + j) * code_stride, M, MP, j, out);
}

// Rows at positions rows[i] of list cluster[i].
__global__ void scan_codes_rows_kernel(const uint8_t* __restrict__ codes, int code_stride, int M, int MP,
                                       const int64_t* __restrict__ list_start, const int64_t* __restrict__ sw_start,
                                       const int64_t* __restrict__ rows, const int32_t* __restrict__ cluster,
                                       int64_t n, uint8_t* __restrict__ scanc) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t g = rows[i];
    const int c = cluster[i];
    write_scan_codes(codes + g * code_stride, M, MP, (int)(g - list_start[c]), scanc + sw_start[c] * MP);
}

__global__ void order_count_kernel(const int32_t* __restrict__ probe_ids, int64_t nq, int np_max,
                                   int32_t* __restrict__ cnt) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nq) atomicAdd(&cnt[probe_ids[q * np_max]], 1);
}

// Exclusive prefix of cnt[0..n) in place, one block.
__global__ void order_scan_kernel(int32_t* __restrict__ cnt, int n) {
    constexpr int PER_MAX = 32;
    __shared__ int32_t wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (n + 1023) / 1024;
    // thread t owns elements [t * per, (t + 1) * per); up to PER_MAX of them
    // are loaded at once into registers (independent loads)
    int v[PER_MAX];
    int sum = 0;
    if (per <= PER_MAX) {
#pragma unroll
        for (int j = 0; j < PER_MAX; j++) {
            const int i = t * per + j;
            v[j] = (j < per && i < n) ? cnt[i] : 0;
            sum += v[j];
        }
    } else {
        for (int i = t * per; i < min(n, (t + 1) * per); i++) sum += cnt[i];
    }
    // block exclusive scan of the per-thread sums: warp shuffles, then the
    // warp totals by warp 0
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int tot = wsum[lane];
        int x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[lane] = x - tot;
    }
    __syncthreads();
    int run = incl - sum + wsum[w];
    if (per <= PER_MAX) {
#pragma unroll
        for (int j = 0; j < PER_MAX; j++) {
            const int i = t * per + j;
            if (j < per && i < n) {
                cnt[i] = run;
                run += v[j];
            }
        }
    } else {
        for (int i = t * per; i < min(n, (t + 1) * per); i++) {
            const int c = cnt[i];
            cnt[i] = run;
            run += c;
        }
    }
}

// Each query takes the next slot of its first list's range. The order
// within a list is whatever the atomics give; a query's result does not
// depend on which block runs it.
__global__ void order_scatter_kernel(const int32_t* __restrict__ probe_ids, int64_t nq, int np_max,
                                     int32_t* __restrict__ cursor, int32_t* __restrict__ order) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nq) order[atomicAdd(&cursor[probe_ids[q * np_max]], 1)] = (int32_t)q;
}

__global__ void transpose_codebooks_kernel(const float* __restrict__ cb, int M, int pqK, int dsub,
                                           float* __restrict__ out) {
    const int64_t total = (int64_t)M * pqK * dsub;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)(e % dsub);
        const int64_t r = e / dsub;
        const int m = (int)(r % M);
        const int j = (int)(r / M);
        out[e] = cb[((int64_t)m * pqK + j) * dsub + t];
    }
}

}  // namespace

cudaError_t launch_transpose_codebooks(const float* cb, int M, int pqK, int dsub, float* out, cudaStream_t s) {
    const int64_t total = (int64_t)M * pqK * dsub;
    if (total <= 0) return cudaSuccess;
    transpose_codebooks_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 1024), 256, 0, s>>>(cb, M, pqK,
                                                                                                      dsub, out);
    return cudaGetLastError();
}

cudaError_t launch_probe_order(const int32_t* probe_ids, int64_t nq, int np_max, int nlist, int32_t* scratch,
                               int32_t* order, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int32_t) * (size_t)nlist, s);
    if (e != cudaSuccess) return e;
    order_count_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(probe_ids, nq, np_max, scratch);
    order_scan_kernel<<<1, 1024, 0, s>>>(scratch, nlist);
    order_scatter_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(probe_ids, nq, np_max, scratch, order);
    return cudaGetLastError();
}

bool scan_adc_supported(int M) { return M >= 1 && M <= 32; }
int scan_codes_per_row(int M) { return (M + 7) / 8 * 8; }
int scan_group_rows(int) { return 32; }

int scan_adc_capw(int R) {
    int c = 128;
    while (c < 2 * R + 64) c <<= 1;
    return c;
}

size_t scan_dump_bytes(int R) { return dump_slot_bytes(scan_adc_capw(R)); }

size_t scan_adc_smem(int R, int M, int fp16) {
    const size_t lut = (!fp16 && scan_codes_per_row(M) > 16) ? 65536 : 32768;
    return lut + (size_t)WARPS * scan_adc_capw(R) * 12 + (size_t)WARPS * R * 12 + (size_t)WARPS * 256 * 4;
}

cudaError_t launch_scan_adc(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                            const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback, int R,
                            int32_t* cand_row, float* cand_d, uint32_t* cand_seq, unsigned long long* rows_scanned,
                            cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (!scan_adc_supported(p.M) || !p.scanc) return cudaErrorInvalidValue;
    const int tab = p.adc_cb != nullptr && p.adc_table >= 1 && p.adc_table <= 2 ? p.adc_table : 0;
    int CAPW = scan_adc_capw(R);
    const size_t smem = scan_adc_smem(R, p.M, tab != 0 ? 1 : 0);
    // 16-bit tables with one 256-entry warp buffer take the striped layout
    // (the same bytes as the flat one: 64 KB of table rows and buffers)
    const bool striped = tab != 0 && CAPW == 256;
    const int variant = tab == 0 ? 0 : 2 * tab - 1 + (striped ? 1 : 0);  // 0, F16 1-2, fixed 3-4
    const void* fn = nullptr;
#define HANN_SCAN_VARIANTS(MPV)                                                     \
    switch (variant) {                                                                \
    case 0: fn = (const void*)scan_adc_kernel<MPV, 0, false>; break;                  \
    case 1: fn = (const void*)scan_adc_kernel<MPV, 1, false>; break;                  \
    case 2: fn = (const void*)scan_adc_kernel<MPV, 1, true>; break;                   \
    case 3: fn = (const void*)scan_adc_kernel<MPV, 2, false>; break;                  \
    default: fn = (const void*)scan_adc_kernel<MPV, 2, true>; break;                  \
    }
    switch (scan_codes_per_row(p.M)) {
    case 8: HANN_SCAN_VARIANTS(8) break;
    case 16: HANN_SCAN_VARIANTS(16) break;
    case 24: HANN_SCAN_VARIANTS(24) break;
    case 32: HANN_SCAN_VARIANTS(32) break;
    default: return cudaErrorInvalidValue;
    }
#undef HANN_SCAN_VARIANTS
    ScanParams pp = p;
    if (tab == 0) pp.scan_cut = nullptr;  // the FP32 screen is not checked
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&pp, (void*)&queries, (void*)&probe_d, (void*)&probe_ids, (void*)&nprobe, (void*)&np_max,
                    (void*)&fallback, (void*)&R, (void*)&CAPW, (void*)&cand_row, (void*)&cand_d, (void*)&cand_seq,
                    (void*)&rows_scanned};
    e = cudaLaunchKernel(fn, dim3((unsigned)nq), dim3(THREADS), args, smem, s);
    if (e != cudaSuccess) return e;
    if (pp.dump) {
        const size_t ssm = select_smem(CAPW, R);
        e = cudaFuncSetAttribute(scan_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm);
        if (e != cudaSuccess) return e;
        scan_select_kernel<<<(unsigned)ceil_div(nq, SEL_WARPS), SEL_WARPS * 32, ssm, s>>>(pp, nq, R, CAPW, cand_row,
                                                                                         cand_d, cand_seq);
    }
    return cudaGetLastError();
}

cudaError_t launch_scan_codes_lists(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                    const int32_t* list_len, const int64_t* sw_start, int nlist, uint8_t* scanc,
                                    cudaStream_t s) {
    if (nlist <= 0 || !scan_adc_supported(M)) return cudaSuccess;
    scan_codes_lists_kernel<<<(unsigned)nlist, 128, 0, s>>>(codes, code_stride, M, scan_codes_per_row(M),
                                                            list_start, list_len, sw_start, scanc);
    return cudaGetLastError();
}

cudaError_t launch_scan_codes_rows(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                   const int64_t* sw_start, const int64_t* rows, const int32_t* cluster, int64_t n,
                                   uint8_t* scanc, cudaStream_t s) {
    if (n <= 0 || !scan_adc_supported(M)) return cudaSuccess;
    scan_codes_rows_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(codes, code_stride, M, scan_codes_per_row(M),
                                                                      list_start, sw_start, rows, cluster, n, scanc);
    return cudaGetLastError();
}

}  // namespace hann
