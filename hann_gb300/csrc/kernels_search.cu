// kernels_search.cu -- the PQIVF Search hot path on the device.
//
// Search (pqivf/index.go:850-949) becomes three kernels per query batch,
// after the coarse distance matrix (kernels_train.cu):
//   1. probe_select: the nprobe nearest lists per query in (distance, index)
//      order -- nearestCentroids + sort (pqivf/index.go:184-206, 875-888) --
//      and the brute-force fallback decision (pqivf/index.go:890-899);
//   2. scan: asymmetric-distance scan of the probed lists' uint8 codes with a
//      per-query lookup table in shared memory, keeping the R best rows per
//      query in per-warp candidate buffers;
//   3. rerank: the R candidates rescored with an exact FP32 distance in the
//      reference's summation order, sorted, truncated to k, sqrt in FP64
//      (pqivf/index.go:937-947).
//
// The scan's distance decomposes the reference's reconstructed-vector
// distance ||q - (c + r)||^2 as ||q - c||^2 + (||r||^2 + 2<c, r>) - 2<q, r>:
// the first term comes from the coarse distance matrix, the second is stored
// per row at encode time, and the third is a sum of M table entries
// T[m][code_m] = -2 <q_m, codebook_m[code_m]>, one table per query shared by
// every probed list. It only selects candidates; every returned distance is
// recomputed exactly.
#include "common.cuh"
#include "kernels.h"

namespace hann {

constexpr int PS_THREADS = 256;
constexpr int PS_MAX = 4096;

__device__ __forceinline__ bool less_ki(uint32_t ka, int32_t ia, uint32_t kb, int32_t ib) {
    return ka < kb || (ka == kb && ia < ib);
}

// Block-wide bitonic sort of P (power of two) (key, idx) pairs in shared memory.
__device__ void block_sort_ki(uint32_t* key, int32_t* idx, int P) {
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    const bool gt = less_ki(key[ixj], idx[ixj], key[i], idx[i]);
                    if (up == gt) {
                        uint32_t tk = key[i];
                        key[i] = key[ixj];
                        key[ixj] = tk;
                        int32_t ti = idx[i];
                        idx[i] = idx[ixj];
                        idx[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(PS_THREADS) probe_select_kernel(
    const float* __restrict__ D, int nlist, const int32_t* __restrict__ nprobe, int np_max,
    const int32_t* __restrict__ kq, const int32_t* __restrict__ list_len, int allow_fb,
    int32_t* __restrict__ probe_ids, float* __restrict__ probe_d, int32_t* __restrict__ fallback,
    unsigned long long* __restrict__ fb_count) {
    __shared__ unsigned int hist[256];
    __shared__ uint32_t s_key[PS_MAX];
    __shared__ int32_t s_idx[PS_MAX];
    __shared__ uint32_t s_prefix, s_remaining;
    __shared__ int s_cnt;
    __shared__ int warp_cnt[PS_THREADS / 32];
    __shared__ unsigned long long s_total;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int q = blockIdx.x;
    const float* row = D + (int64_t)q * nlist;
    const int np = min(nprobe[q], nlist);
    if (tid == 0) {
        s_prefix = 0;
        s_remaining = (uint32_t)np;
        s_cnt = 0;
        s_total = 0;
    }
    // Radix select of the np-th smallest distance key, 8 bits per pass.
    uint32_t mask = 0;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = tid; b < 256; b += PS_THREADS) hist[b] = 0;
        __syncthreads();
        const uint32_t prefix = s_prefix;
        for (int c = tid; c < nlist; c += PS_THREADS) {
            const uint32_t key = float_key(row[c]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid == 0) {
            const uint32_t rem = s_remaining;
            uint32_t cum = 0;
            for (int b = 0; b < 256; b++) {
                const uint32_t h = hist[b];
                if (cum + h >= rem) {
                    s_prefix = prefix | ((uint32_t)b << shift);
                    s_remaining = rem - cum;
                    break;
                }
                cum += h;
            }
        }
        __syncthreads();
        mask |= 255u << shift;
    }
    const uint32_t T = s_prefix;
    const int ties_needed = (int)s_remaining;
    for (int c = tid; c < nlist; c += PS_THREADS) {
        const uint32_t key = float_key(row[c]);
        if (key < T) {
            const int pos = atomicAdd(&s_cnt, 1);
            s_key[pos] = key;
            s_idx[pos] = c;
        }
    }
    __syncthreads();
    const int base = s_cnt;
    // Lists tied at the threshold: the lowest indices win, kept in index order.
    int taken = 0;
    for (int c0 = 0; c0 < nlist && taken < ties_needed; c0 += PS_THREADS) {
        const int c = c0 + tid;
        const bool flag = c < nlist && float_key(row[c]) == T;
        const unsigned bal = __ballot_sync(0xffffffffu, flag);
        if (lane == 0) warp_cnt[w] = __popc(bal);
        __syncthreads();
        int off = 0, tot = 0;
        for (int i = 0; i < PS_THREADS / 32; i++) {
            if (i < w) off += warp_cnt[i];
            tot += warp_cnt[i];
        }
        const int pos = taken + off + __popc(bal & ((1u << lane) - 1u));
        if (flag && pos < ties_needed) {
            s_key[base + pos] = T;
            s_idx[base + pos] = c;
        }
        __syncthreads();
        taken += tot;
    }
    int P = 1;
    while (P < np) P <<= 1;
    for (int i = np + tid; i < P; i += PS_THREADS) {
        s_key[i] = 0xffffffffu;
        s_idx[i] = 0x7fffffff;
    }
    __syncthreads();
    block_sort_ki(s_key, s_idx, P);
    unsigned long long part = 0;
    for (int i = tid; i < np; i += PS_THREADS) {
        probe_ids[(int64_t)q * np_max + i] = s_idx[i];
        probe_d[(int64_t)q * np_max + i] = key_float(s_key[i]);
        part += (unsigned long long)list_len[s_idx[i]];
    }
    atomicAdd(&s_total, part);
    __syncthreads();
    if (tid == 0) {
        const int fb = (allow_fb && s_total < (unsigned long long)kq[q]) ? 1 : 0;
        fallback[q] = fb;
        if (fb) atomicAdd(fb_count, 1ull);
    }
}

cudaError_t launch_probe_select(const float* D, int64_t nq, int nlist, const int32_t* nprobe, int np_max,
                                const int32_t* k, const int32_t* list_len, int allow_fallback, int32_t* probe_ids,
                                float* probe_d, int32_t* fallback, unsigned long long* fallback_count,
                                cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (np_max > PS_MAX) return cudaErrorInvalidValue;
    probe_select_kernel<<<(unsigned)nq, PS_THREADS, 0, s>>>(D, nlist, nprobe, np_max, k, list_len, allow_fallback,
                                                           probe_ids, probe_d, fallback, fallback_count);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Candidates are ordered by (distance, sequence, row). The sequence of a
// candidate is the probe rank of its list, so equal distances keep the
// reference's candidate order: probe order, then list order.
struct Cand {
    float d;
    uint32_t seq;
    int32_t row;
};

__device__ __forceinline__ bool cand_less(float da, uint32_t sa, int32_t ra, float db, uint32_t sb, int32_t rb) {
    if (da != db) return da < db;
    if (sa != sb) return sa < sb;
    return ra < rb;
}

// Warp-wide bitonic sort of CAP entries held in shared memory.
__device__ void warp_sort_cand(float* d, uint32_t* sq, int32_t* r, int CAP) {
    const int lane = threadIdx.x & 31;
    for (int kk = 2; kk <= CAP; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < CAP; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    const bool gt = cand_less(d[ixj], sq[ixj], r[ixj], d[i], sq[i], r[i]);
                    if (up == gt) {
                        float td = d[i]; d[i] = d[ixj]; d[ixj] = td;
                        uint32_t ts = sq[i]; sq[i] = sq[ixj]; sq[ixj] = ts;
                        int32_t tr = r[i]; r[i] = r[ixj]; r[ixj] = tr;
                    }
                }
            }
            __syncwarp();
        }
    }
}

__device__ void block_sort_cand(float* d, uint32_t* sq, int32_t* r, int P) {
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & kk) == 0;
                    const bool gt = cand_less(d[ixj], sq[ixj], r[ixj], d[i], sq[i], r[i]);
                    if (up == gt) {
                        float td = d[i]; d[i] = d[ixj]; d[ixj] = td;
                        uint32_t ts = sq[i]; sq[i] = sq[ixj]; sq[ixj] = ts;
                        int32_t tr = r[i]; r[i] = r[ixj]; r[ixj] = tr;
                    }
                }
            }
            __syncthreads();
        }
    }
}

constexpr int SC_THREADS = 256;
constexpr int SC_WARPS = SC_THREADS / 32;
constexpr float F_INF = __builtin_huge_valf();

// Sort the warp's buffer, keep the best R, and publish its R-th distance as a
// block-wide threshold: a row worse than R rows already seen by any one warp
// cannot enter the query's best R.
__device__ __forceinline__ int warp_flush(float* wd, uint32_t* ws, int32_t* wr, int count, int CAPW, int R,
                                          uint32_t* s_tau) {
    const int lane = threadIdx.x & 31;
    for (int i = count + lane; i < CAPW; i += 32) {
        wd[i] = F_INF;
        ws[i] = 0xffffffffu;
        wr[i] = 0x7fffffff;
    }
    __syncwarp();
    warp_sort_cand(wd, ws, wr, CAPW);
    const int kept = min(count, R);
    if (kept == R && lane == 0) atomicMin(s_tau, float_key(wd[R - 1]));
    __syncwarp();
    return kept;
}

template <int MW>
__device__ __forceinline__ void load_code_words(const uint8_t* __restrict__ codes, int64_t row, int stride,
                                                uint32_t (&cw)[MW]) {
    const uint8_t* p = codes + row * stride;
    if constexpr (MW % 4 == 0) {
#pragma unroll
        for (int i = 0; i < MW / 4; i++) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + i);
            cw[4 * i] = v.x; cw[4 * i + 1] = v.y; cw[4 * i + 2] = v.z; cw[4 * i + 3] = v.w;
        }
    } else if constexpr (MW % 2 == 0) {
#pragma unroll
        for (int i = 0; i < MW / 2; i++) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(p) + i);
            cw[2 * i] = v.x; cw[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < MW; i++) cw[i] = __ldg(reinterpret_cast<const uint32_t*>(p) + i);
    }
}

// One block per query. MW = code words (4 codes each) per row; MW = 0 is the
// generic path for any M.
template <int MW>
__global__ void __launch_bounds__(SC_THREADS) scan_kernel(ScanParams p, const float* __restrict__ Q,
                                                          const float* __restrict__ probe_d,
                                                          const int32_t* __restrict__ probe_ids,
                                                          const int32_t* __restrict__ nprobe, int np_max,
                                                          const int32_t* __restrict__ fallback, int R, int CAPW,
                                                          int32_t* __restrict__ cand_row, float* __restrict__ cand_d,
                                                          uint32_t* __restrict__ cand_seq,
                                                          unsigned long long* __restrict__ rows_scanned) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float* lut = reinterpret_cast<float*>(smraw);                 // [M][256]
    float* wdall = lut + p.M * 256;                               // [SC_WARPS][CAPW]
    uint32_t* wsall = reinterpret_cast<uint32_t*>(wdall + SC_WARPS * CAPW);
    int32_t* wrall = reinterpret_cast<int32_t*>(wsall + SC_WARPS * CAPW);
    __shared__ uint32_t s_tau;
    __shared__ int s_wcount[SC_WARPS];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (p.qcount && (int)blockIdx.x >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[blockIdx.x] : blockIdx.x;
    const float* qv = Q + q * p.dim;
    if (tid == 0) s_tau = float_key(F_INF);
    for (int e = tid; e < p.M * 256; e += SC_THREADS) {
        const int m = e >> 8, j = e & 255;
        float s = 0.0f;
        if (j < p.pqK) {
            const float* cw = p.codebooks + ((int64_t)m * p.pqK + j) * p.dsub;
            const float* qm = qv + m * p.dsub;
            for (int t = 0; t < p.dsub; t++) s = fmaf(qm[t], cw[t], s);
        }
        lut[e] = -2.0f * s;
    }
    __syncthreads();
    float* wd = wdall + w * CAPW;
    uint32_t* ws = wsall + w * CAPW;
    int32_t* wr = wrall + w * CAPW;
    const bool fb = fallback[q] != 0;
    const int nl = fb ? p.nlist : min(nprobe[q], p.nlist);
    const unsigned lt_mask = (1u << lane) - 1u;
    int count = 0;
    unsigned long long scanned = 0;
    for (int i = w; i < nl; i += SC_WARPS) {
        const int l = fb ? i : probe_ids[q * np_max + i];
        float base;
        if (fb) {
            // Fallback scans every list: its coarse distance, lane-parallel.
            float part = 0.0f;
            for (int j = lane; j < p.dim; j += 32) {
                const float t = qv[j] - p.coarse[(int64_t)l * p.dim + j];
                part = fmaf(t, t, part);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
            base = part;
        } else {
            base = probe_d[q * np_max + i];
        }
        const int64_t start = p.list_start[l];
        const int len = p.list_len[l];
        scanned += (unsigned long long)len;
        for (int r0 = 0; r0 < len; r0 += 32) {
            const int r = r0 + lane;
            float d = F_INF;
            int64_t row = start + r;
            if (r < len) {
                float acc = base + __ldg(p.term + row);
                if constexpr (MW > 0) {
                    uint32_t cw[MW];
                    load_code_words<MW>(p.codes, row, p.code_stride, cw);
#pragma unroll
                    for (int wi = 0; wi < MW; wi++) {
#pragma unroll
                        for (int b = 0; b < 4; b++) {
                            const int m = 4 * wi + b;
                            if (m < p.M) acc += lut[(m << 8) + ((cw[wi] >> (8 * b)) & 255u)];
                        }
                    }
                } else {
                    const uint8_t* cp = p.codes + row * p.code_stride;
                    for (int m = 0; m < p.M; m++) acc += lut[(m << 8) + cp[m]];
                }
                d = acc;
            }
            const float tau = key_float(*(volatile uint32_t*)&s_tau);
            const bool pass = d < tau;
            const unsigned bal = __ballot_sync(0xffffffffu, pass);
            if (bal) {
                const int pos = count + __popc(bal & lt_mask);
                if (pass) {
                    wd[pos] = d;
                    ws[pos] = (uint32_t)i;
                    wr[pos] = (int32_t)row;
                }
                count += __popc(bal);
                if (count > CAPW - 32) {
                    __syncwarp();
                    count = warp_flush(wd, ws, wr, count, CAPW, R, &s_tau);
                }
            }
        }
    }
    __syncwarp();
    count = warp_flush(wd, ws, wr, count, CAPW, R, &s_tau);
    if (lane == 0) {
        s_wcount[w] = count;
        if (rows_scanned) atomicAdd(rows_scanned, scanned);
    }
    __syncthreads();
    // Merge: the warps' best R each, packed, then one block sort.
    int P = 1;
    while (P < SC_WARPS * R) P <<= 1;
    // Pack in place into the front of the buffers: warp w's entries move to
    // offset w*R. Offsets never exceed the source positions (R <= CAPW), so
    // copying warp by warp in ascending order is safe.
    for (int ww = 1; ww < SC_WARPS; ww++) {
        for (int i0 = 0; i0 < R; i0 += SC_THREADS) {
            const int i = i0 + tid;
            const bool in = i < R;
            const bool ok = in && i < s_wcount[ww];
            const float dv = ok ? wdall[ww * CAPW + i] : F_INF;
            const uint32_t sv = ok ? wsall[ww * CAPW + i] : 0xffffffffu;
            const int32_t rv = ok ? wrall[ww * CAPW + i] : 0x7fffffff;
            __syncthreads();
            if (in) {
                wdall[ww * R + i] = dv;
                wsall[ww * R + i] = sv;
                wrall[ww * R + i] = rv;
            }
            __syncthreads();
        }
    }
    for (int i = s_wcount[0] + tid; i < R; i += SC_THREADS) {
        wdall[i] = F_INF;
        wsall[i] = 0xffffffffu;
        wrall[i] = 0x7fffffff;
    }
    for (int i = SC_WARPS * R + tid; i < P; i += SC_THREADS) {
        wdall[i] = F_INF;
        wsall[i] = 0xffffffffu;
        wrall[i] = 0x7fffffff;
    }
    __syncthreads();
    block_sort_cand(wdall, wsall, wrall, P);
    const int Rq = p.kq ? min(R, rerank_depth_for(p.kq[q], p.mode, p.rerank_fixed)) : R;
    for (int i = tid; i < R; i += SC_THREADS) {
        const bool ok = i < Rq && wrall[i] != 0x7fffffff;
        cand_row[q * R + i] = ok ? wrall[i] : -1;
        cand_d[q * R + i] = wdall[i];
        cand_seq[q * R + i] = wsall[i];
    }
}

static int cap_for(int R) {
    int c = 64;
    while (c < R + 32) c <<= 1;
    return c;
}

cudaError_t launch_scan(const ScanParams& p, const float* queries, int64_t nq, const int32_t* probe_ids,
                        const float* probe_d, const int32_t* nprobe, int np_max, const int32_t* fallback, int R,
                        int32_t* cand_row, float* cand_d, uint32_t* cand_seq, unsigned long long* rows_scanned,
                        cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    if (scan_adc_supported(p.M) && p.scanc && scan_adc_smem(R, p.M, p.adc_table && p.adc_cb) <= 224 * 1024)
        return launch_scan_adc(p, queries, nq, probe_ids, probe_d, nprobe, np_max, fallback, R, cand_row, cand_d,
                               cand_seq, rows_scanned, s);
    const int CAPW = cap_for(R);
    int P = 1;
    while (P < SC_WARPS * R) P <<= 1;
    const int buf = std::max(SC_WARPS * CAPW, P);
    const size_t smem = (size_t)p.M * 256 * sizeof(float) + (size_t)buf * 12;
    const int MW = p.code_stride / 4;
    const void* fn;
    switch (MW) {
    case 1: fn = (const void*)scan_kernel<1>; break;
    case 2: fn = (const void*)scan_kernel<2>; break;
    case 3: fn = (const void*)scan_kernel<3>; break;
    case 4: fn = (const void*)scan_kernel<4>; break;
    case 6: fn = (const void*)scan_kernel<6>; break;
    case 8: fn = (const void*)scan_kernel<8>; break;
    case 12: fn = (const void*)scan_kernel<12>; break;
    case 16: fn = (const void*)scan_kernel<16>; break;
    default: fn = (const void*)scan_kernel<0>; break;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&p, (void*)&queries, (void*)&probe_d, (void*)&probe_ids, (void*)&nprobe, (void*)&np_max,
                    (void*)&fallback, (void*)&R, (void*)&CAPW, (void*)&cand_row, (void*)&cand_d, (void*)&cand_seq,
                    (void*)&rows_scanned};
    e = cudaLaunchKernel(fn, dim3((unsigned)nq), dim3(SC_THREADS), args, smem, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The reference's reconstructed vector for a row: centroid + concatenated
// codewords, added in FP32 (decodePQCode + vectorAdd, pqivf/index.go:678-714).
struct ReconRow {
    const float* c;
    const float* cb;
    const uint8_t* code;
    int dsub, pqK;
    __device__ __forceinline__ float operator[](int i) const {
        const int m = i / dsub;
        const int e = i - m * dsub;
        return __fadd_rn(c[i], cb[((int64_t)m * pqK + code[m]) * dsub + e]);
    }
};

// Whether the k-th reference distance dk proves a screened query's top k:
// every row the scan left out has a screened distance at or above cut, so an
// exact PQ distance above cut - eps, and FP32 roundings of the reference's
// distance and of the screen are far below 2e-5 of the values compared.
__device__ __forceinline__ bool proven(float dk, float cut, float eps) {
    return cut == __int_as_float(0x7f800000) || dk + 2e-5f * (fabsf(cut) + fabsf(dk)) + eps < cut;
}

constexpr int RR_THREADS = 256;
constexpr int RW_MAX = 128;  // candidates per query up to which one warp reranks a query

// One warp per query for small candidate sets (RP <= RW_MAX): the same
// computation as rerank_kernel without block barriers, eight queries per
// block.
__global__ void __launch_bounds__(RR_THREADS) rerank_warp_kernel(ScanParams p, const float* __restrict__ Q, int64_t nq,
                                                                 const int32_t* __restrict__ cand_row,
                                                                 const uint32_t* __restrict__ cand_seq, int R, int RP,
                                                                 const int32_t* __restrict__ kq, int kmax, int mode,
                                                                 int64_t* __restrict__ ids, double* __restrict__ dist,
                                                                 int32_t* __restrict__ nout) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t qi = (int64_t)blockIdx.x * (RR_THREADS / 32) + w;
    if (qi >= nq) return;
    if (p.qcount && qi >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[qi] : qi;
    float* qv = reinterpret_cast<float*>(smraw) + (int64_t)w * (p.dim + 3 * RP);
    float* cd = qv + p.dim;
    uint32_t* cs = reinterpret_cast<uint32_t*>(cd + RP);
    int32_t* cr = reinterpret_cast<int32_t*>(cs + RP);
    for (int e = lane; e < p.dim; e += 32) qv[e] = Q[q * p.dim + e];
    __syncwarp();
    int valid = 0;
    for (int i = lane; i < RP; i += 32) {
        const int32_t row = i < R ? cand_row[q * R + i] : -1;
        if (row >= 0 && p.row_id[row] >= 0) {
            float d;
            if (mode == 0) {
                ReconRow rec{p.coarse + (int64_t)p.row_cluster[row] * p.dim, p.codebooks,
                             p.codes + (int64_t)row * p.code_stride, p.dsub, p.pqK};
                d = sqeuclid_ref(qv, rec, p.dim);
            } else if ((p.dim & 3) == 0) {
                d = sqeuclid_ref_v4(qv, p.vectors + (int64_t)row * p.dim, p.dim);
            } else {
                d = sqeuclid_ref(qv, p.vectors + (int64_t)row * p.dim, p.dim);
            }
            cd[i] = d;
            cs[i] = cand_seq[q * R + i];
            cr[i] = row;
            valid++;
        } else {
            cd[i] = F_INF;
            cs[i] = 0xffffffffu;
            cr[i] = 0x7fffffff;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, o);
    __syncwarp();
    warp_sort_cand(cd, cs, cr, RP);
    const int k = min(kq[q], valid);
    if (lane == 0 && mode == 0 && p.scan_cut && k > 0 && k == kq[q] && !proven(cd[k - 1], p.scan_cut[q], p.scan_eps[q])) {
        p.redo[atomicAdd(p.redo_count, 1)] = (int32_t)q;
        if (p.redo_total) atomicAdd(p.redo_total, 1ull);
    }
    for (int i = lane; i < kmax; i += 32) {
        if (i < k) {
            ids[q * kmax + i] = p.row_id[cr[i]];
            dist[q * kmax + i] = sqrt((double)cd[i]);
        } else {
            ids[q * kmax + i] = -1;
            dist[q * kmax + i] = 0.0;
        }
    }
    if (lane == 0) nout[q] = k;
}

__global__ void __launch_bounds__(RR_THREADS) rerank_kernel(ScanParams p, const float* __restrict__ Q,
                                                            const int32_t* __restrict__ cand_row,
                                                            const uint32_t* __restrict__ cand_seq, int R, int RP,
                                                            const int32_t* __restrict__ kq, int kmax, int mode,
                                                            int64_t* __restrict__ ids, double* __restrict__ dist,
                                                            int32_t* __restrict__ nout) {
    extern __shared__ __align__(16) unsigned char smraw[];
    float* qv = reinterpret_cast<float*>(smraw);
    float* cd = qv + p.dim;
    uint32_t* cs = reinterpret_cast<uint32_t*>(cd + RP);
    int32_t* cr = reinterpret_cast<int32_t*>(cs + RP);
    __shared__ int s_valid;
    if (p.qcount && (int)blockIdx.x >= *p.qcount) return;
    const int64_t q = p.qorder ? p.qorder[blockIdx.x] : blockIdx.x;
    const int tid = threadIdx.x;
    if (tid == 0) s_valid = 0;
    for (int e = tid; e < p.dim; e += RR_THREADS) qv[e] = Q[q * p.dim + e];
    __syncthreads();
    int valid = 0;
    for (int i = tid; i < RP; i += RR_THREADS) {
        const int32_t row = i < R ? cand_row[q * R + i] : -1;
        if (row >= 0 && p.row_id[row] >= 0) {
            float d;
            if (mode == 0) {
                ReconRow rec{p.coarse + (int64_t)p.row_cluster[row] * p.dim, p.codebooks,
                             p.codes + (int64_t)row * p.code_stride, p.dsub, p.pqK};
                d = sqeuclid_ref(qv, rec, p.dim);
            } else {
                d = sqeuclid_ref(qv, p.vectors + (int64_t)row * p.dim, p.dim);
            }
            cd[i] = d;
            cs[i] = cand_seq[q * R + i];
            cr[i] = row;
            valid++;
        } else {
            cd[i] = F_INF;
            cs[i] = 0xffffffffu;
            cr[i] = 0x7fffffff;
        }
    }
    atomicAdd(&s_valid, valid);
    __syncthreads();
    block_sort_cand(cd, cs, cr, RP);
    const int k = min(kq[q], s_valid);
    if (tid == 0 && mode == 0 && p.scan_cut && k > 0 && k == kq[q] && !proven(cd[k - 1], p.scan_cut[q], p.scan_eps[q])) {
        p.redo[atomicAdd(p.redo_count, 1)] = (int32_t)q;
        if (p.redo_total) atomicAdd(p.redo_total, 1ull);
    }
    for (int i = tid; i < kmax; i += RR_THREADS) {
        if (i < k) {
            ids[q * kmax + i] = p.row_id[cr[i]];
            dist[q * kmax + i] = sqrt((double)cd[i]);
        } else {
            ids[q * kmax + i] = -1;
            dist[q * kmax + i] = 0.0;
        }
    }
    if (tid == 0) nout[q] = k;
}

cudaError_t launch_rerank(const ScanParams& p, const float* queries, int64_t nq, const int32_t* cand_row,
                          const uint32_t* cand_seq, int R, const int32_t* k, int kmax, int mode, int64_t* ids,
                          double* dist, int32_t* nout, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    int RP = 1;
    while (RP < R) RP <<= 1;
    if (RP <= RW_MAX) {
        const size_t wsm = (size_t)(RR_THREADS / 32) * ((size_t)p.dim * sizeof(float) + (size_t)RP * 12);
        if (wsm <= 160 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(rerank_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 160 * 1024);
            if (e != cudaSuccess) return e;
            rerank_warp_kernel<<<(unsigned)ceil_div(nq, RR_THREADS / 32), RR_THREADS, wsm, s>>>(
                p, queries, nq, cand_row, cand_seq, R, RP, k, kmax, mode, ids, dist, nout);
            return cudaGetLastError();
        }
    }
    const size_t smem = (size_t)p.dim * sizeof(float) + (size_t)RP * 12;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(rerank_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    rerank_kernel<<<(unsigned)nq, RR_THREADS, smem, s>>>(p, queries, cand_row, cand_seq, R, RP, k, kmax, mode, ids,
                                                         dist, nout);
    return cudaGetLastError();
}

}  // namespace hann
