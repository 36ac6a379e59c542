// kernels_scan.cu -- bank-conflict-free ADC list scan with warp radix
// selection, for M up to 32. Larger M use scan_kernel in kernels_search.cu.
//
// Same distance as scan_kernel: ||q-c||^2 + term + sum_m T[m][code_m].
//
// Lookup table without bank conflicts. The table is 256 rows of 32 words,
// entry (m, j) at row j, bank (c * M + m) for every copy c < 32 / M. A warp
// takes G = M * (32 / M) rows of a list at a time; lane l (l < G) owns rows
// whose position in the list is l mod G, uses copy c = l / M, and walks the
// subquantizers in the rotated order m_s = (s + l) mod M, so in every step
// the G lanes read G distinct banks.
//
// Scan words. Rather than its code bytes, each row stores for every step s
// the byte offset of its table entry, (code_{m_s} * 32 + c * M + m_s) * 4,
// as a 16-bit word ("scan words", built from the codes whenever rows are
// placed; see launch_scan_words_*). A lookup is then one shift or mask, one
// shared load and one add. The words of G consecutive rows are stored plane
// by plane, so a warp step reads them with contiguous 16-byte loads: the
// scan is bound by the L1 data pipe's wavefronts (table reads plus these
// loads), and contiguous loads take the fewest.
//
// Selection without sorting. Each warp appends rows below the block-wide
// threshold to its buffer; a full buffer is cut back to its R smallest keys
// by a radix select on 8-bit digits (warp-private histogram), whose R-th key
// lowers the threshold. At the end warp 0 selects the query's R best from the
// warps' survivors. Candidates leave unsorted: the rerank sorts them by exact
// distance.
#include <algorithm>

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

// Keeps the `R` smallest keys of entries [0, count) (ties at the cut broken
// by position), compacted in place to [0, R). Returns through *kth a key at
// or above the R-th smallest (exactly it unless the digit holding the cut
// came out whole). hist: the warp's 256 counters. Warp-synchronous.
__device__ int warp_select(uint32_t* key, uint32_t* seq, int32_t* row, int count, int R, uint32_t* kth,
                           uint32_t* hist) {
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

template <int MP, int MX, int DEPTH>
__global__ void __launch_bounds__(THREADS, 3) scan_skew_kernel(ScanParams p, const float* __restrict__ Q,
                                                            const float* __restrict__ probe_d,
                                                            const int32_t* __restrict__ probe_ids,
                                                            const int32_t* __restrict__ nprobe, int np_max,
                                                            const int32_t* __restrict__ fallback, int R, int CAPW,
                                                            int32_t* __restrict__ cand_row,
                                                            float* __restrict__ cand_d,
                                                            uint32_t* __restrict__ cand_seq,
                                                            unsigned long long* __restrict__ rows_scanned) {
    // MP: scan words per row (M rounded up to 8); MX: M when it equals MP
    // (known at compile time), else 0. G rows per warp step.
    __shared__ __align__(16) float lut[256 * 32];
    extern __shared__ __align__(16) unsigned char smraw[];
    uint32_t* wkey = reinterpret_cast<uint32_t*>(smraw);
    uint32_t* wseq = wkey + WARPS * CAPW;
    int32_t* wrow = reinterpret_cast<int32_t*>(wseq + WARPS * CAPW);
    uint32_t* mkey = reinterpret_cast<uint32_t*>(wrow + WARPS * CAPW);  // [WARPS * R] merge region
    uint32_t* mseq = mkey + WARPS * R;
    int32_t* mrow = reinterpret_cast<int32_t*>(mseq + WARPS * R);
    uint32_t* whist = reinterpret_cast<uint32_t*>(mrow + WARPS * R);   // [WARPS][256]
    __shared__ uint32_t s_tau;
    __shared__ int s_big;
    __shared__ int s_wcount[WARPS];
    __shared__ int s_lstart[SCAN_FLAT_LISTS], s_lsw[SCAN_FLAT_LISTS];
    __shared__ int s_llen[SCAN_FLAT_LISTS], s_lsteps[SCAN_FLAT_LISTS + 1];
    __shared__ float s_lbase[SCAN_FLAT_LISTS];
    const int M = MX > 0 ? MX : p.M;
    const int copies = 32 / M;
    const int G = 32;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (p.qcount && (int)blockIdx.x >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[blockIdx.x] : blockIdx.x;
    const float* qv = Q + q * p.dim;
    if (tid == 0) {
        s_tau = KEY_INF;
        s_big = 0;
    }
    {
        // Lane l fills bank l of table rows w, w + WARPS, ...: subquantizer
        // m = l % M. Codeword j of every subquantizer sits in one row of the
        // transposed codebooks, so a warp's loads for one table row are one
        // contiguous read (the [M][pqK] layout spread them over M rows 1 KB+
        // apart).
        const bool own = lane < copies * M;
        const int m = lane % M;
        const float* qm = qv + m * p.dsub;
        const bool v4 = (p.dsub & 3) == 0 &&
                        ((reinterpret_cast<uintptr_t>(qv) | reinterpret_cast<uintptr_t>(p.codebooks_t)) & 15) == 0;
        for (int j = w; j < 256; j += WARPS) {
            float v = 0.0f;
            if (own && j < p.pqK) {
                const float* cw = p.codebooks_t + ((int64_t)j * M + m) * p.dsub;
                float acc = 0.0f;
                if (v4) {
                    for (int t = 0; t < p.dsub; t += 4) {
                        const float4 a = __ldg(reinterpret_cast<const float4*>(qm + t));
                        const float4 b = __ldg(reinterpret_cast<const float4*>(cw + t));
                        acc = fmaf(a.x, b.x, acc);
                        acc = fmaf(a.y, b.y, acc);
                        acc = fmaf(a.z, b.z, acc);
                        acc = fmaf(a.w, b.w, acc);
                    }
                } else {
                    for (int t = 0; t < p.dsub; t++) acc = fmaf(qm[t], cw[t], acc);
                }
                v = -2.0f * acc;
            }
            lut[j * 32 + lane] = v;
        }
    }
    __syncthreads();
    const unsigned char* lutb = reinterpret_cast<const unsigned char*>(lut);
    uint32_t* key = wkey + w * CAPW;
    uint32_t* seq = wseq + w * CAPW;
    int32_t* row = wrow + w * CAPW;
    uint32_t* hist = whist + w * 256;
    const bool fb = fallback[q] != 0;
    const int nl = fb ? p.nlist : min(nprobe[q], p.nlist);
    const unsigned ltm = (1u << lane) - 1u;
    const bool act = lane < G;
    int count = 0;
    unsigned long long scanned = 0;
    // The warp walks its lists G rows at a time and loads the next step's
    // rows -- in the same list or the next one -- before it computes the
    // current, so each lane keeps two rows in flight.
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
            base = part;
        } else {
            base = probe_d[q * np_max + i];
        }
        start = p.list_start[l];
        sws = p.sw_start[l];
        len = p.list_len[l];
    };
    // Scan words of one step: G rows, stored as MP / 8 planes of G
    // consecutive 16-byte chunks, so the warp's loads are contiguous.
    auto load_row = [&](int64_t sws, int step, int64_t grow, uint4 (&sw)[MP / 8], float& term) {
        const uint4* sp = reinterpret_cast<const uint4*>(p.scanw) + sws * (MP / 8) + (int64_t)step * G * (MP / 8) + lane;
#pragma unroll
        for (int t = 0; t < MP / 8; t++) sw[t] = __ldg(sp + t * G);
        term = __ldg(p.term + grow);
    };
    // four partial sums keep the adds off one long dependency chain
    auto lookup = [&](const uint4 (&sw)[MP / 8], float acc) {
        const uint32_t* wv = reinterpret_cast<const uint32_t*>(sw);
        float part[4] = {acc, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int s2 = 0; s2 < MP / 2; s2++) {
            const uint32_t word = wv[s2];
            if (2 * s2 < M) part[(2 * s2) & 3] += *reinterpret_cast<const float*>(lutb + (word & 0xffffu));
            if (2 * s2 + 1 < M) part[(2 * s2 + 1) & 3] += *reinterpret_cast<const float*>(lutb + (word >> 16));
        }
        return float_key((part[0] + part[1]) + (part[2] + part[3]));
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
            if (count > CAPW - 32) {
                __syncwarp();
                uint32_t kth;
                count = warp_select(key, seq, row, count, R, &kth, hist);
                if (lane == 0) atomicMin(&s_tau, kth);
                __syncwarp();
            }
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
            s_lbase[i] = probe_d[q * np_max + i];
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
        // lane's row in it and the scan-word pointer.
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
            const uint4* sw4 = reinterpret_cast<const uint4*>(p.scanw);
            int cu = ub, cend = s_lsteps[cl + 1], crow = (ub - s_lsteps[cl]) * G + lane;
            int clen = s_llen[cl];
            const float* cterm = p.term + s_lstart[cl];
            const uint4* csw = sw4 + ((int64_t)s_lsw[cl] + (int64_t)(ub - s_lsteps[cl]) * G) * (MP / 8) + lane;
            // A step in flight: its words, its term (+inf past the list's end,
            // where the words are not initialised and the lookup is skipped)
            // and tag = probe position << 24 | row position in the list.
            auto load_step = [&](uint4 (&sw)[MP / 8], float& term, int& tag) {
#pragma unroll
                for (int t = 0; t < MP / 8; t++) sw[t] = __ldg(csw + t * G);
                term = crow < clen ? __ldg(cterm + crow) : pos_inf();
                tag = (cl << 24) | crow;
                cu++;
                if (cu < cend) {
                    crow += G;
                    csw += G * (MP / 8);
                } else if (cu < ub + n) {
                    do {
                        cl++;
                    } while (s_lsteps[cl + 1] <= cu);
                    cend = s_lsteps[cl + 1];
                    crow = lane;
                    clen = s_llen[cl];
                    cterm = p.term + s_lstart[cl];
                    csw = sw4 + (int64_t)s_lsw[cl] * (MP / 8) + lane;
                }
            };
            auto compute = [&](const uint4 (&sw)[MP / 8], float term, int tag) {
                const int li = tag >> 24;
                const uint32_t k = term < pos_inf() ? lookup(sw, s_lbase[li] + term) : KEY_INF;
                return k;
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
                    if (count > CAPW - 32) {
                        __syncwarp();
                        uint32_t kth;
                        count = warp_select(key, seq, row, count, R, &kth, hist);
                        if (lane == 0) atomicMin(&s_tau, kth);
                        __syncwarp();
                    }
                }
            };
            // DEPTH steps in a ring: a step's words are loaded DEPTH - 1
            // steps before it is computed. Two: a deeper ring spills
            // registers at three blocks per SM, and the spills cost more
            // than the latency it hides (2.06 ms against 2.43 ms for three
            // and 4.19 ms for four on the 10M x 96 search).
            uint4 sw[DEPTH][MP / 8];
            float tm[DEPTH];
            int tg[DEPTH];
#pragma unroll
            for (int d = 0; d < DEPTH; d++)
                if (d < n) load_step(sw[d], tm[d], tg[d]);
            for (int i = 0; i < n; i += DEPTH) {
#pragma unroll
                for (int d = 0; d < DEPTH; d++) {
                    if (i + d >= n) break;
                    const uint32_t k = compute(sw[d], tm[d], tg[d]);
                    const int g0 = tg[d];
                    if (i + d + DEPTH < n) load_step(sw[d], tm[d], tg[d]);
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
            uint4 sa[MP / 8], sb[MP / 8];
            float ta = 0.0f, tb = 0.0f;
            bool va = act && lane < len;
            if (va) load_row(sws, 0, start + lane, sa, ta);
            for (int st = 0; st * G < len; st += 2) {
                const int r0 = st * G;
                const bool vb = act && r0 + G + lane < len;
                if (vb) load_row(sws, st + 1, start + r0 + G + lane, sb, tb);
                offer(va ? lookup(sa, base + ta) : KEY_INF, li, start + r0 + lane);
                if (r0 + G >= len) break;
                va = act && r0 + 2 * G + lane < len;
                if (va) load_row(sws, st + 2, start + r0 + 2 * G + lane, sa, ta);
                offer(vb ? lookup(sb, base + tb) : KEY_INF, li, start + r0 + G + lane);
            }
        }
    }
    __syncwarp();
    {
        uint32_t kth;
        count = warp_select(key, seq, row, count, R, &kth, hist);
        if (lane == 0) {
            s_wcount[w] = count;
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
        for (int i = lane; i < R; i += 32) {
            const bool ok = i < kept;
            cand_row[q * R + i] = ok ? mrow[i] : -1;
            cand_d[q * R + i] = ok ? key_float(mkey[i]) : __int_as_float(0x7f800000);
            cand_seq[q * R + i] = ok ? mseq[i] : 0xffffffffu;
        }
    }
}

// Scan words of rows: for the row at position pos of its list (group
// pos / G, lane l = pos mod G, copy c = l / M, rotation r = l mod M), word s
// is the table offset of subquantizer m = (s + r) mod M: (code_m * 32 + c * M
// + m) * 4; words past M are zero. A list's words start at slot sw_start
// (MP words per slot); group g of G rows holds MP / 8 planes of G 8-word
// chunks: word s of lane l sits at ((g * MP / 8 + s / 8) * G + l) * 8 + s % 8.
__device__ __forceinline__ void write_scan_words(const uint8_t* __restrict__ codes, int M, int MP, int pos,
                                                 uint16_t* __restrict__ list_words) {
    const int copies = 32 / M, G = 32;
    const int g = pos / G, l = pos - g * G, c = (l / M) % copies, r = l % M;
    for (int s = 0; s < MP; s++) {
        uint16_t v = 0;
        if (s < M) {
            int m = s + r;
            if (m >= M) m -= M;
            v = (uint16_t)(((int)codes[m] * 32 + c * M + m) * 4);
        }
        list_words[((int64_t)(g * (MP / 8) + s / 8) * G + l) * 8 + (s & 7)] = v;
    }
}

// One block per list: every slot in [start, start + len).
__global__ void scan_words_lists_kernel(const uint8_t* __restrict__ codes, int code_stride, int M, int MP,
                                        const int64_t* __restrict__ list_start, const int32_t* __restrict__ list_len,
                                        const int64_t* __restrict__ sw_start, uint16_t* __restrict__ scanw) {
    const int l = blockIdx.x;
    const int64_t start = list_start[l];
    const int len = list_len[l];
    uint16_t* words = scanw + sw_start[l] * MP;
    for (int j = threadIdx.x; j < len; j += blockDim.x) write_scan_words(codes + (start + j) * code_stride, M, MP, j, words);
}

// Rows at positions rows[i] of list cluster[i].
__global__ void scan_words_rows_kernel(const uint8_t* __restrict__ codes, int code_stride, int M, int MP,
                                       const int64_t* __restrict__ list_start, const int64_t* __restrict__ sw_start,
                                       const int64_t* __restrict__ rows, const int32_t* __restrict__ cluster,
                                       int64_t n, uint16_t* __restrict__ scanw) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t g = rows[i];
    const int c = cluster[i];
    write_scan_words(codes + g * code_stride, M, MP, (int)(g - list_start[c]), scanw + sw_start[c] * MP);
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

bool scan_skew_supported(int M) { return M >= 1 && M <= 32; }
int scan_words_per_row(int M) { return (M + 7) / 8 * 8; }
int scan_group_rows(int) { return 32; }

int scan_skew_capw(int R) {
    int c = 128;
    while (c < 2 * R + 64) c <<= 1;
    return c;
}

size_t scan_skew_smem(int R) {
    return (size_t)WARPS * scan_skew_capw(R) * 12 + (size_t)WARPS * R * 12 + (size_t)WARPS * 256 * 4;
}

cudaError_t launch_scan_skew(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                             const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback, int R,
                             int32_t* cand_row, float* cand_d, uint32_t* cand_seq, unsigned long long* rows_scanned,
                             cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (!scan_skew_supported(p.M) || !p.scanw) return cudaErrorInvalidValue;
    int CAPW = scan_skew_capw(R);
    const size_t smem = scan_skew_smem(R);
    const void* fn;
    switch (p.M) {
    case 8: fn = (const void*)scan_skew_kernel<8, 8, 2>; break;
    case 16: fn = (const void*)scan_skew_kernel<16, 16, 2>; break;
    case 24: fn = (const void*)scan_skew_kernel<24, 24, 2>; break;
    case 32: fn = (const void*)scan_skew_kernel<32, 32, 2>; break;
    default:
        switch (scan_words_per_row(p.M) / 8) {
        case 1: fn = (const void*)scan_skew_kernel<8, 0, 2>; break;
        case 2: fn = (const void*)scan_skew_kernel<16, 0, 2>; break;
        case 3: fn = (const void*)scan_skew_kernel<24, 0, 2>; break;
        case 4: fn = (const void*)scan_skew_kernel<32, 0, 2>; break;
        default: return cudaErrorInvalidValue;
        }
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&p, (void*)&queries, (void*)&probe_d, (void*)&probe_ids, (void*)&nprobe, (void*)&np_max,
                    (void*)&fallback, (void*)&R, (void*)&CAPW, (void*)&cand_row, (void*)&cand_d, (void*)&cand_seq,
                    (void*)&rows_scanned};
    e = cudaLaunchKernel(fn, dim3((unsigned)nq), dim3(THREADS), args, smem, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t launch_scan_words_lists(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                    const int32_t* list_len, const int64_t* sw_start, int nlist, uint16_t* scanw,
                                    cudaStream_t s) {
    if (nlist <= 0 || !scan_skew_supported(M)) return cudaSuccess;
    scan_words_lists_kernel<<<(unsigned)nlist, 128, 0, s>>>(codes, code_stride, M, scan_words_per_row(M),
                                                            list_start, list_len, sw_start, scanw);
    return cudaGetLastError();
}

cudaError_t launch_scan_words_rows(const uint8_t* codes, int code_stride, int M, const int64_t* list_start,
                                   const int64_t* sw_start, const int64_t* rows, const int32_t* cluster, int64_t n,
                                   uint16_t* scanw, cudaStream_t s) {
    if (n <= 0 || !scan_skew_supported(M)) return cudaSuccess;
    scan_words_rows_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(codes, code_stride, M, scan_words_per_row(M),
                                                                      list_start, sw_start, rows, cluster, n, scanw);
    return cudaGetLastError();
}

}  // namespace hann
