// kernels_scan.cu -- bank-conflict-free ADC list scan with warp radix
// selection, for M a multiple of 4 and at most 32 (the row's codes fill whole
// 32-bit words). Other M use scan_kernel in kernels_search.cu.
//
// Same distance as scan_kernel: ||q-c||^2 + term + sum_m T[m][code_m].
//
// Lookup table without bank conflicts. The table is stored as 256 rows of 32
// words, entry (m, j) at row j, bank (copy * M + m); when M divides 32 it is
// replicated 32 / M times. Lane l walks the subquantizers in the rotated order
// m_s = (s + l mod M) mod M and uses copy (l / M) mod copies, so in any step
// the 32 lanes read 32 distinct banks (M | 32), or at most two lanes share a
// bank (M = 24). The lane rotates its row's code bytes by l mod M once per row
// (word selects and funnel shifts) so step s reads byte s.
//
// Selection without sorting. Each warp appends rows below the block-wide
// threshold to its buffer; a full buffer is cut back to its R smallest keys
// by a ballot radix select, whose R-th key lowers the threshold. At the end
// warp 0 selects the query's R best from the warps' survivors. Candidates
// leave unsorted: the rerank sorts them by exact distance.
#include "common.cuh"
#include "kernels.h"

namespace hann {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t KEY_INF = 0xff800000u;  // float_key(+inf)

// Keeps the `R` smallest keys of entries [0, count) (ties at the cut broken
// by position), compacted in place to [0, R). Returns the R-th smallest key
// through *kth. Warp-synchronous.
__device__ int warp_select(uint32_t* key, uint32_t* seq, int32_t* row, int count, int R, uint32_t* kth) {
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
    for (int bit = top; bit >= 0; bit--) {
        const uint32_t hi = bit == 31 ? 0u : (0xffffffffu << (bit + 1));
        int c0 = 0;
        for (int ch = 0; ch < nch; ch++) {
            const int i = ch * 32 + lane;
            const uint32_t kk = i < count ? key[i] : 0xffffffffu;
            const bool m = i < count && (kk & hi) == prefix && !((kk >> bit) & 1u);
            c0 += __popc(__ballot_sync(FULL, m));
        }
        if ((uint32_t)c0 < need) {
            need -= (uint32_t)c0;
            prefix |= 1u << bit;
        }
    }
    int out = 0, eq_taken = 0;
    for (int ch = 0; ch < nch; ch++) {
        const int i = ch * 32 + lane;
        const bool in = i < count;
        const uint32_t kk = in ? key[i] : 0xffffffffu;
        const uint32_t ss = in ? seq[i] : 0u;
        const int32_t rr = in ? row[i] : 0;
        const bool lt_k = in && kk < prefix;
        const bool eq = in && kk == prefix;
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
    *kth = prefix;
    return out;
}

template <int MW>
__device__ __forceinline__ void rotate_bytes(uint32_t (&w)[MW], int a, int b) {
    // words left by a (0 <= a < MW), then bytes by b (0..3)
#pragma unroll
    for (int t = 0; (1 << t) < MW; t++) {
        const int sh = (1 << t) % MW;
        if ((a >> t) & 1) {
            uint32_t tmp[MW];
#pragma unroll
            for (int i = 0; i < MW; i++) tmp[i] = w[(i + sh) % MW];
#pragma unroll
            for (int i = 0; i < MW; i++) w[i] = tmp[i];
        }
    }
    if (b) {
        uint32_t tmp[MW];
#pragma unroll
        for (int i = 0; i < MW; i++) tmp[i] = __funnelshift_r(w[i], w[(i + 1) % MW], 8 * b);
#pragma unroll
        for (int i = 0; i < MW; i++) w[i] = tmp[i];
    }
}

template <int MW>
__global__ void __launch_bounds__(THREADS) scan_skew_kernel(ScanParams p, const float* __restrict__ Q,
                                                            const float* __restrict__ probe_d,
                                                            const int32_t* __restrict__ probe_ids,
                                                            const int32_t* __restrict__ nprobe, int np_max,
                                                            const int32_t* __restrict__ fallback, int R, int CAPW,
                                                            int32_t* __restrict__ cand_row,
                                                            float* __restrict__ cand_d,
                                                            uint32_t* __restrict__ cand_seq,
                                                            unsigned long long* __restrict__ rows_scanned) {
    constexpr int M = 4 * MW;
    constexpr int COPIES = (32 % M == 0) ? 32 / M : 1;
    extern __shared__ __align__(16) unsigned char smraw[];
    float* lut = reinterpret_cast<float*>(smraw);  // [256][32]
    uint32_t* wkey = reinterpret_cast<uint32_t*>(lut + 256 * 32);
    uint32_t* wseq = wkey + WARPS * CAPW;
    int32_t* wrow = reinterpret_cast<int32_t*>(wseq + WARPS * CAPW);
    uint32_t* mkey = reinterpret_cast<uint32_t*>(wrow + WARPS * CAPW);  // [WARPS * R] merge region
    uint32_t* mseq = mkey + WARPS * R;
    int32_t* mrow = reinterpret_cast<int32_t*>(mseq + WARPS * R);
    __shared__ uint32_t s_tau;
    __shared__ int s_wcount[WARPS];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t q = blockIdx.x;
    const float* qv = Q + q * p.dim;
    if (tid == 0) s_tau = KEY_INF;
    for (int e = tid; e < 256 * 32; e += THREADS) {
        const int j = e >> 5, bk = e & 31;
        float v = 0.0f;
        if (bk < COPIES * M && j < p.pqK) {
            const int m = bk % M;
            const float* cw = p.codebooks + ((int64_t)m * p.pqK + j) * p.dsub;
            const float* qm = qv + m * p.dsub;
            float s = 0.0f;
            for (int t = 0; t < p.dsub; t++) s = fmaf(qm[t], cw[t], s);
            v = -2.0f * s;
        }
        lut[e] = v;
    }
    // Lane constants: rotation r = lane mod M and the byte offset of each step's bank.
    const int r = lane % M;
    const int cb = (COPIES > 1 ? (lane / M) % COPIES : 0) * M;
    uint32_t boff[M];
#pragma unroll
    for (int s = 0; s < M; s++) {
        int m = s + r;
        if (m >= M) m -= M;
        boff[s] = (uint32_t)((cb + m) << 2);
    }
    __syncthreads();
    const unsigned char* lutb = reinterpret_cast<const unsigned char*>(lut);
    uint32_t* key = wkey + w * CAPW;
    uint32_t* seq = wseq + w * CAPW;
    int32_t* row = wrow + w * CAPW;
    const bool fb = fallback[q] != 0;
    const int nl = fb ? p.nlist : min(nprobe[q], p.nlist);
    const unsigned ltm = (1u << lane) - 1u;
    int count = 0;
    unsigned long long scanned = 0;
    // The warp walks its lists chunk by chunk (32 rows, one per lane) and
    // loads the next chunk -- in the same list or the next one -- before it
    // computes the current, so each lane keeps two rows in flight.
    auto list_meta = [&](int i, int64_t& start, int& len, float& base) {
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
        len = p.list_len[l];
    };
    auto load_row = [&](int64_t grow, uint32_t (&cw)[MW], float& term) {
        const uint8_t* cp = p.codes + grow * p.code_stride;
        if constexpr (MW % 2 == 0) {
#pragma unroll
            for (int t = 0; t < MW / 2; t++) {
                const uint2 v = __ldg(reinterpret_cast<const uint2*>(cp) + t);
                cw[2 * t] = v.x;
                cw[2 * t + 1] = v.y;
            }
        } else {
#pragma unroll
            for (int t = 0; t < MW; t++) cw[t] = __ldg(reinterpret_cast<const uint32_t*>(cp) + t);
        }
        term = __ldg(p.term + grow);
    };
    int ci = w, cr0 = 0, clen = 0;
    int64_t cstart = 0;
    float cbase = 0.0f;
    while (ci < nl) {
        list_meta(ci, cstart, clen, cbase);
        scanned += (unsigned long long)clen;
        if (clen > 0) break;
        ci += WARPS;
    }
    uint32_t ncw[MW];
    float nterm = 0.0f;
#pragma unroll
    for (int t = 0; t < MW; t++) ncw[t] = 0;
    if (ci < nl && lane < clen) load_row(cstart + lane, ncw, nterm);
    while (ci < nl) {
        uint32_t cw[MW];
#pragma unroll
        for (int t = 0; t < MW; t++) cw[t] = ncw[t];
        const float term = nterm;
        const int i = ci;
        const bool valid = cr0 + lane < clen;
        const int64_t grow = cstart + cr0 + lane;
        const float base = cbase;
        // advance, then prefetch the next chunk
        cr0 += 32;
        if (cr0 >= clen) {
            cr0 = 0;
            ci += WARPS;
            while (ci < nl) {
                list_meta(ci, cstart, clen, cbase);
                scanned += (unsigned long long)clen;
                if (clen > 0) break;
                ci += WARPS;
            }
        }
        if (ci < nl && cr0 + lane < clen) load_row(cstart + cr0 + lane, ncw, nterm);
        uint32_t k = KEY_INF;
        if (valid) {
            rotate_bytes<MW>(cw, r >> 2, r & 3);
            float acc = base + term;
#pragma unroll
            for (int s = 0; s < M; s++) {
                const uint32_t code = (cw[s >> 2] >> (8 * (s & 3))) & 255u;
                acc += *reinterpret_cast<const float*>(lutb + (code << 7) + boff[s]);
            }
            k = float_key(acc);
        }
        const bool pass = k < *(volatile uint32_t*)&s_tau;
        const unsigned bal = __ballot_sync(FULL, pass);
        if (bal) {
            const int pos = count + __popc(bal & ltm);
            if (pass) {
                key[pos] = k;
                seq[pos] = (uint32_t)i;
                row[pos] = (int32_t)grow;
            }
            count += __popc(bal);
            if (count > CAPW - 32) {
                __syncwarp();
                uint32_t kth;
                count = warp_select(key, seq, row, count, R, &kth);
                if (lane == 0) atomicMin(&s_tau, kth);
                __syncwarp();
            }
        }
    }
    __syncwarp();
    {
        uint32_t kth;
        count = warp_select(key, seq, row, count, R, &kth);
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
        const int kept = warp_select(mkey, mseq, mrow, total, Rq, &kth);
        for (int i = lane; i < R; i += 32) {
            const bool ok = i < kept;
            cand_row[q * R + i] = ok ? mrow[i] : -1;
            cand_d[q * R + i] = ok ? key_float(mkey[i]) : __int_as_float(0x7f800000);
            cand_seq[q * R + i] = ok ? mseq[i] : 0xffffffffu;
        }
    }
}

}  // namespace

bool scan_skew_supported(int M) { return M % 4 == 0 && M >= 4 && M <= 32; }

cudaError_t launch_scan_skew(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                             const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback, int R,
                             int32_t* cand_row, float* cand_d, uint32_t* cand_seq, unsigned long long* rows_scanned,
                             cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    int CAPW = 128;
    while (CAPW < 4 * R) CAPW <<= 1;
    const size_t smem = (size_t)256 * 32 * sizeof(float) + (size_t)WARPS * CAPW * 12 + (size_t)WARPS * R * 12;
    const void* fn;
    switch (p.M / 4) {
    case 1: fn = (const void*)scan_skew_kernel<1>; break;
    case 2: fn = (const void*)scan_skew_kernel<2>; break;
    case 3: fn = (const void*)scan_skew_kernel<3>; break;
    case 4: fn = (const void*)scan_skew_kernel<4>; break;
    case 5: fn = (const void*)scan_skew_kernel<5>; break;
    case 6: fn = (const void*)scan_skew_kernel<6>; break;
    case 7: fn = (const void*)scan_skew_kernel<7>; break;
    case 8: fn = (const void*)scan_skew_kernel<8>; break;
    default: return cudaErrorInvalidValue;
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

}  // namespace hann
