// kernels_lms.cu -- the list-major batched scan on the tensor cores (sm_103a).
//
// The reference scores every candidate of a query one at a time: it decodes
// the entry's PQ code to a vector and computes the FP32 distance
// (pqivf/index.go:905-936, decodePQCode + vectorAdd at 678-714). A batch of
// queries probes the same lists many times over (10,000 queries x 32 probes
// over 16,384 lists touch each list about 20 times), so here the work is
// grouped by list: the (query, probed list) pairs of a batch form a work
// queue sorted by list, and one work item is one list (or a range of its
// rows) against up to 64 of the queries that probe it. A persistent kernel
// takes items from the queue; for each 128-row tile of the item's list it
//
//   * decodes the rows' residuals r = concat_m codebook_m[code_m] to FP16 in
//     shared memory (the MMA's A operand, 128-byte swizzled, K-major),
//   * multiplies them with the item's queries (FP16, B operand) on the
//     tensor cores: tcgen05.mma kind::f16, FP32 accumulators in tensor
//     memory, one elected thread issuing,
//   * and turns each accumulator into the screened score
//       s~ = ||q - c||^2 + term - 2 <q~, r~>,   term = ||r||^2 + 2 <c, r>,
//     the decomposition of ||q - (c + r)||^2 the reference computes,
//     appending (s~, row) to the query's candidate buffer when s~ is at or
//     below the query's current threshold.
//
// A query's pairs are scanned in chunks of probe ranks (its nearest list
// first, then the next few, then the rest); between chunks the band merge of
// the batched k-NN (kernels_knn.cu, knn_merge_band) keeps per query every
// candidate that can still reach its final set and lowers its threshold, so
// later chunks append few rows. The first chunk writes every score of the
// query's nearest lists at fixed positions, without atomics.
//
// Exactness. |s~ - s| <= eps per query, where eps bounds the FP16 rounding of
// q and r (Cauchy-Schwarz on the rounding residuals: ||q - q~|| measured per
// query, the residual's bound from the codebooks' own rounding) and the FP32
// accumulation; the merge keeps every row with s~ <= T~ + 2 eps (+ a relative
// slack for the FP32 roundings of the reference's distance), T~ the k-th
// smallest s~, so the reference's top k always lies in the band, and the
// rerank rescores the band in the reference's FP32 order. Queries whose band
// or buffers overflow go to the table scan (kernels_scan.cu) instead.
//
// Block layout (320 threads, one block per SM): warp 9 claims items and
// writes each item's metadata and column information into a ring of eight
// slots and its queries (B) into one of two shared-memory buffers, so it runs
// up to a few items ahead; warps 0-3 decode the row tiles (A) into three or
// four shared-memory stages (as many as the FP16 codebooks leave room for)
// from the codebooks held in shared memory, each thread one row, the next
// tile's code words loaded while the current one decodes; warp 4 allocates
// all 512 tensor-memory columns and issues the MMAs into eight accumulator
// buffers of 64 columns, so the epilogue trails the MMAs by up to eight
// tiles; warps 5-8 drain the accumulators, one TMEM lane quarter each.
// Every mbarrier wait is bounded: past the limit the kernel records an
// error, the roles leave their loops, and the tensor memory is still
// released.
//
// Routing. The decode makes this scan pay off only where a list is shared
// by many of the batch's queries, i.e. at large nprobe; queries probing
// fewer lists than the index's min_nprobe take the table scan in the same
// batch. The choice depends on the query alone, never on the batch, so a
// query's exact-rerank result does not change with the batch it is in.
#include <cuda_fp16.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "select.cuh"

namespace hann {
namespace {

constexpr int LMS_THREADS = 320;
constexpr int TM = 128;            // rows per tile (MMA M)
constexpr int NQ = LMS_NQ;         // queries per item (largest MMA N)
constexpr int A_STAGES_MAX = 4;
constexpr int A_STAGE_BYTES = 2 * TM * 128;  // two 64-element K blocks, 128-byte rows
constexpr int B_BUF_BYTES = 2 * NQ * 128;
constexpr int T_BUFS = 8;            // accumulator buffers in tensor memory
constexpr int TMEM_COLS = T_BUFS * NQ;  // all 512 columns: one block per SM
constexpr uint32_t SPIN_LIMIT = 1u << 22;

struct ColInfo {
    int32_t q;     // query
    float base;    // ||q - c||^2 of the item's list
    float tau;     // the query's threshold
    int32_t off;   // first-chunk position of the list in the query's candidate buffer
};

// Fixed part of the shared memory (operand stages, column information,
// metadata, barriers, the epilogue warps' scratch); the FP16 codebooks
// follow it (at most 128 x 256 halves = 64 KiB), so one block runs per SM.
constexpr int CB_SMEM_MAX = 128 * 256 * 2;
__host__ __device__ constexpr int cb_smem_bytes(int dim, int pqK) { return (dim * pqK * 2 + 15) / 16 * 16; }
constexpr int M_RING = 8;       // items whose metadata and columns are staged at once
constexpr int BAR_BYTES = 384;  // the mbarriers, the TMEM address and the abort flag
__host__ __device__ constexpr int smem_fixed(int stages) {
    return 1024 + stages * A_STAGE_BYTES + 2 * B_BUF_BYTES + M_RING * NQ * (int)sizeof(ColInfo) +
           M_RING * (int)sizeof(LmsItem) + BAR_BYTES + 4 * 128 * 4;
}
// A stages: four while they fit beside the codebooks in 227 KiB, else three.
__host__ __device__ constexpr int a_stages(int dim, int pqK) {
    return smem_fixed(4) + cb_smem_bytes(dim, pqK) <= 227 * 1024 ? 4 : 3;
}

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; false (error recorded, abort flag raised) past the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err, volatile int* abort_flag) {
    for (uint32_t i = 0; i < SPIN_LIMIT; i++) {
        if (mbar_try(b, parity)) return true;
        if ((i & 1023u) == 1023u && *abort_flag) return false;
    }
    atomicExch(err, 1);
    *abort_flag = 1;
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart, descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor: FP16 x FP16 -> FP32, both K-major, M = 128, N = n.
__device__ __forceinline__ uint32_t idesc_f16(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
            dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

// 32 columns of the warp's 32 TMEM lanes into v[0..32), load and wait in one
// asm statement so no use of v is scheduled before the wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element e (0 <= e < 128) of row `row` in a two-block,
// 128-byte-swizzled K-major tile of `rows` rows.
__device__ __forceinline__ uint32_t sw_off(int row, int e, int rows) {
    const int kb = e >> 6, byte = (e & 63) * 2;
    return (uint32_t)(kb * rows * 128 + row * 128 + ((((byte >> 4) ^ (row & 7)) << 4) | (byte & 15)));
}

// A row's code bytes as 32-bit words (code_stride is a multiple of 4): the
// decoders load the next tile's words while they decode the current one.
constexpr int CW_MAX = 8;  // words a row may carry for the fast decode (M <= 32)
__device__ __forceinline__ void load_codes(const uint8_t* __restrict__ code, int nw, uint32_t (&cw)[CW_MAX]) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(code);
#pragma unroll
    for (int i = 0; i < CW_MAX; i++) cw[i] = i < nw ? __ldg(w + i) : 0u;
}

// Writes the FP16 residual of one row into its A-tile row: dsub elements per
// subquantizer, looked up in the FP16 codebooks [M][pqK][dsub] held in
// shared memory. The fast forms (dsub 4 or 8, M <= 32) take the row's code
// words from registers and issue every lookup of a group of eight before
// its stores.
template <int DSUB>
__device__ __forceinline__ void decode_row(unsigned char* tile, int prow, const uint32_t (&cw)[CW_MAX],
                                           const uint8_t* __restrict__ code, int M, int dsub, int pqK,
                                           const __half* cbs) {
    if constexpr (DSUB == 4 || DSUB == 8) {
        using V = typename std::conditional<DSUB == 4, uint2, uint4>::type;
        const V* cb = reinterpret_cast<const V*>(cbs);
#pragma unroll
        for (int g = 0; g < 4 * CW_MAX; g += 8) {
            if (g < M) {
                V v[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const uint32_t byte = (cw[g / 4 + e / 4] >> (8 * (e & 3))) & 0xffu;
                    if (g + e < M) v[e] = cb[(g + e) * pqK + (int)byte];
                }
                if constexpr (DSUB == 4) {
                    // two subquantizers per 16-byte store: a warp's 32 rows then
                    // fill 32 distinct banks per wavefront (the swizzle spreads
                    // rows r and r + 1 .. r + 7 over the eight chunk positions)
#pragma unroll
                    for (int e = 0; e < 8; e += 2) {
                        if (g + e + 1 < M)
                            *reinterpret_cast<uint4*>(tile + sw_off(prow, 4 * (g + e), TM)) =
                                make_uint4(v[e].x, v[e].y, v[e + 1].x, v[e + 1].y);
                        else if (g + e < M)
                            *reinterpret_cast<uint2*>(tile + sw_off(prow, 4 * (g + e), TM)) = v[e];
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < 8; e++)
                        if (g + e < M) *reinterpret_cast<V*>(tile + sw_off(prow, DSUB * (g + e), TM)) = v[e];
                }
            }
        }
    } else {
        for (int m = 0; m < M; m++) {
            const __half* w = cbs + ((int64_t)m * pqK + code[m]) * dsub;
            for (int e = 0; e < dsub; e++)
                *reinterpret_cast<__half*>(tile + sw_off(prow, m * dsub + e, TM)) = w[e];
        }
    }
}

// One accumulator row (this thread's list row against the item's columns)
// to candidates. NP, the item's column count rounded up to 16, makes every
// loop fully unrolled and branch-free, so the column information is read in
// groups of eight loads in flight rather than one latency per column.
//   dense (the first chunk): every score at the row's fixed position in its
//     query's buffer, no atomics;
//   otherwise: a pass mask of the scores at or below each query's threshold;
//     when a lane of the warp passes anything, one ballot per column into the
//     warp's scratch (wbal[0..64)), every column's slots reserved at once
//     (lane l for columns l and l + 32, both atomics in flight; wbal[64..128)
//     receives the first slots), then the passing rows written.
template <int NP>
__device__ __forceinline__ void epi_tile(const LmsParams& p, const ColInfo* ci, float (&acc)[NQ], int n_pairs,
                                         bool valid, int64_t grow, float term, int row_pos, uint32_t* wbal) {
    const int lane = threadIdx.x & 31;
    if (p.dense) {
#pragma unroll
        for (int g = 0; g < NP; g += 8) {
            ColInfo c[8];
#pragma unroll
            for (int u = 0; u < 8; u++) c[u] = ci[g + u];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int pos = c[u].off + row_pos;
                if (valid && g + u < n_pairs && pos < p.cap) {
                    const int64_t o = (int64_t)c[u].q * p.cap + pos;
                    p.cand_id[o] = (int32_t)grow;
                    p.cand_s[o] = __fmaf_rn(-2.0f, acc[g + u], c[u].base + term);
                }
            }
        }
        return;
    }
    uint64_t mask = 0;
#pragma unroll
    for (int g = 0; g < NP; g += 8) {
        ColInfo c[8];
#pragma unroll
        for (int u = 0; u < 8; u++) c[u] = ci[g + u];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const float sv = __fmaf_rn(-2.0f, acc[g + u], c[u].base + term);
            acc[g + u] = sv;
            const bool pass = valid && g + u < n_pairs && sv <= c[u].tau;
            mask |= (uint64_t)(pass ? 1u : 0u) << (g + u);
        }
    }
    if (!__any_sync(0xffffffffu, mask != 0ull)) return;
    int32_t* wbase = reinterpret_cast<int32_t*>(wbal + 64);
#pragma unroll
    for (int j = 0; j < NP; j++) {
        const unsigned bal = __ballot_sync(0xffffffffu, ((mask >> j) & 1ull) != 0ull);
        if (lane == 0) wbal[j] = bal;
    }
    __syncwarp();
    const uint32_t b0 = lane < n_pairs ? wbal[lane] : 0u;
    const uint32_t b1 = lane + 32 < n_pairs ? wbal[lane + 32] : 0u;
    int r0 = 0, r1 = 0;
    if (b0) r0 = atomicAdd(p.cnt + ci[lane].q, __popc(b0));
    if (b1) r1 = atomicAdd(p.cnt + ci[lane + 32].q, __popc(b1));
    if (lane < n_pairs) wbase[lane] = r0;
    if (lane + 32 < n_pairs) wbase[lane + 32] = r1;
    __syncwarp();
    const unsigned ltm = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < NP; j++) {
        if ((mask >> j) & 1ull) {
            const int pos = wbase[j] + __popc(wbal[j] & ltm);
            if (pos < p.cap) {
                const int64_t o = (int64_t)ci[j].q * p.cap + pos;
                p.cand_id[o] = (int32_t)grow;
                p.cand_s[o] = acc[j];
            }
        }
    }
    __syncwarp();
}

template <int DSUB>
__global__ void __launch_bounds__(LMS_THREADS, 1) lms_scan_kernel(LmsParams p) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int A_STAGES = a_stages(p.dim, p.pqK);
    unsigned char* sA = base;
    unsigned char* sB = sA + A_STAGES * A_STAGE_BYTES;
    ColInfo* cols = reinterpret_cast<ColInfo*>(sB + 2 * B_BUF_BYTES);  // [M_RING][NQ]
    LmsItem* meta = reinterpret_cast<LmsItem*>(cols + M_RING * NQ);    // [M_RING]
    uint64_t* bars = reinterpret_cast<uint64_t*>(meta + M_RING);
    uint64_t* a_full = bars;                    // [A_STAGES_MAX] tile decoded
    uint64_t* a_empty = a_full + A_STAGES_MAX;  // [A_STAGES_MAX] tile consumed by the MMAs
    uint64_t* m_full = a_empty + A_STAGES_MAX;  // [M_RING] item metadata and columns staged
    uint64_t* m_empty = m_full + M_RING;        // [M_RING] ... read by every role
    uint64_t* b_full = m_empty + M_RING;        // [2] item queries staged
    uint64_t* b_empty = b_full + 2;             // [2] ... consumed by the MMAs
    uint64_t* t_full = b_empty + 2;             // [T_BUFS] accumulator ready
    uint64_t* t_empty = t_full + T_BUFS;        // [T_BUFS] accumulator drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(t_empty + T_BUFS);
    volatile int* s_abort = reinterpret_cast<volatile int*>(t_empty + T_BUFS) + 2;
    uint32_t* escr = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(bars) + BAR_BYTES);  // [4][128]
    __half* cbs = reinterpret_cast<__half*>(escr + 4 * 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Every operand byte starts at zero: the K padding past the dimension and
    // rows or columns a partial tile or item leaves unwritten must hold finite
    // values, which the epilogue then ignores.
    for (int i = threadIdx.x; i < (A_STAGES * A_STAGE_BYTES + 2 * B_BUF_BYTES) / 16; i += LMS_THREADS)
        reinterpret_cast<uint4*>(sA)[i] = make_uint4(0, 0, 0, 0);
    {
        const int ncb = p.M * p.pqK * p.dsub;
        const unsigned short* src = static_cast<const unsigned short*>(p.cb16);
        for (int i = threadIdx.x; i < ncb; i += LMS_THREADS) reinterpret_cast<unsigned short*>(cbs)[i] = src[i];
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < A_STAGES_MAX; s++) {
            mbar_init(&a_full[s], 4);   // the four decoder warps
            mbar_init(&a_empty[s], 1);  // the MMA commit
        }
        for (int m = 0; m < M_RING; m++) {
            mbar_init(&m_full[m], 1);   // the loader warp
            mbar_init(&m_empty[m], 9);  // four decoder warps, the MMA thread, four epilogue warps
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&b_full[b], 1);   // the loader warp
            mbar_init(&b_empty[b], 1);  // the MMA commit
        }
        for (int b = 0; b < T_BUFS; b++) {
            mbar_init(&t_full[b], 1);
            mbar_init(&t_empty[b], 4);
        }
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int ksteps = (p.dim + 15) >> 4;

    if (warp < 4) {
        // ---------------- decoders: the item's row tiles into the A stages,
        // one row per thread, the next tile's code words loaded ahead
        const int pt = threadIdx.x;  // 0..127: the tile row this thread decodes
        const int nw = p.code_stride >> 2;
        const bool fast = (DSUB == 4 || DSUB == 8) && nw <= CW_MAX;
        int item_seq = 0, tile_seq = 0;
        uint32_t cw[CW_MAX], cn[CW_MAX];
#pragma unroll
        for (int i = 0; i < CW_MAX; i++) cw[i] = cn[i] = 0u;
        bool pre = false;  // cw already holds this item's first code words
        while (true) {
            const int m = item_seq % M_RING;
            if (!__all_sync(0xffffffffu, mbar_wait(&m_full[m], (item_seq / M_RING) & 1, p.err, s_abort))) break;
            const LmsItem it = meta[m];
            __syncwarp();
            if (lane == 0) mbar_arrive(&m_empty[m]);  // the item lives in registers from here
            if (it.n_rows < 0) break;
            const int ntiles = (it.n_rows + TM - 1) / TM;
            const uint8_t* rows = p.codes + it.row0 * p.code_stride;
            if (fast && !pre && pt < it.n_rows) load_codes(rows + (int64_t)pt * p.code_stride, nw, cw);
            pre = false;
            bool ok = true;
            for (int t = 0; t < ntiles; t++, tile_seq++) {
                const int s = tile_seq % A_STAGES;
                if (tile_seq >= A_STAGES &&
                    !__all_sync(0xffffffffu, mbar_wait(&a_empty[s], ((tile_seq / A_STAGES) - 1) & 1, p.err, s_abort))) {
                    ok = false;
                    break;
                }
                const int lr = t * TM + pt;
                const int ln = lr + TM;
                if (fast) {
                    if (t + 1 < ntiles) {
                        if (ln < it.n_rows) load_codes(rows + (int64_t)ln * p.code_stride, nw, cn);
                    } else {
                        // last tile: the next item's first rows, when the
                        // loader has staged its metadata already
                        const int mn = (item_seq + 1) % M_RING;
                        uint32_t rdy = lane == 0 ? (mbar_try(&m_full[mn], ((item_seq + 1) / M_RING) & 1) ? 1u : 0u) : 0u;
                        rdy = __shfl_sync(0xffffffffu, rdy, 0);
                        if (rdy) {
                            const LmsItem nx = meta[mn];
                            if (nx.n_rows > 0) {
                                if (pt < nx.n_rows)
                                    load_codes(p.codes + (nx.row0 + pt) * p.code_stride, nw, cn);
                                pre = true;
                            }
                        }
                    }
                }
                if (lr < it.n_rows)
                    decode_row<DSUB>(sA + s * A_STAGE_BYTES, pt, cw, rows + (int64_t)lr * p.code_stride, p.M, p.dsub,
                                     p.pqK, cbs);
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&a_full[s]);
                if (fast) {
#pragma unroll
                    for (int i = 0; i < CW_MAX; i++) cw[i] = cn[i];
                }
            }
            if (!ok) break;
            if (p.stats && pt == 0) {
                atomicAdd(p.stats, (unsigned long long)it.n_rows * (unsigned long long)it.n_pairs);
                atomicAdd(p.stats + 1, (unsigned long long)it.n_rows);
            }
            item_seq++;
        }
    } else if (warp == 9) {
        // ---------------- loader: claims items and stages their metadata and
        // column information (a ring of M_RING items, so the decoders run
        // ahead of the epilogue) and their queries (B, two buffers). An item
        // is claimed and its pair data loaded before any wait, and the
        // queries move with cp.async, all in flight at once.
        const int n_items = min(*p.n_items, p.item_cap);
        int item_seq = 0;
        while (true) {
            const int m = item_seq % M_RING, b = item_seq & 1;
            int idx = 0;
            if (lane == 0) idx = atomicAdd(p.item_counter, 1);
            idx = __shfl_sync(0xffffffffu, idx, 0);
            const bool last = idx >= n_items;
            LmsItem it;
            it.n_pairs = 0;
            ColInfo ca{0, 0.0f, 0.0f, 0}, cb{0, 0.0f, 0.0f, 0};
            if (!last) {
                it = p.items[idx];
                if (lane < it.n_pairs) {
                    const int64_t pr = (int64_t)it.pair_begin + lane;
                    ca.q = p.pair_q[pr];
                    ca.base = p.pair_base[pr];
                    ca.off = p.dense ? p.pair_off[pr] : 0;
                }
                if (lane + 32 < it.n_pairs) {
                    const int64_t pr = (int64_t)it.pair_begin + lane + 32;
                    cb.q = p.pair_q[pr];
                    cb.base = p.pair_base[pr];
                    cb.off = p.dense ? p.pair_off[pr] : 0;
                }
                ca.tau = p.dense || lane >= it.n_pairs ? __int_as_float(0x7f800000) : p.thr[ca.q];
                cb.tau = p.dense || lane + 32 >= it.n_pairs ? __int_as_float(0x7f800000) : p.thr[cb.q];
            }
            if (item_seq >= M_RING &&
                !__all_sync(0xffffffffu, mbar_wait(&m_empty[m], ((item_seq / M_RING) - 1) & 1, p.err, s_abort)))
                break;
            if (lane == 0) {
                if (last) meta[m].n_rows = -1;
                else meta[m] = it;
            }
            if (!last) {
                ColInfo* ci = cols + m * NQ;
                if (lane < it.n_pairs) ci[lane] = ca;
                if (lane + 32 < it.n_pairs) ci[lane + 32] = cb;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&m_full[m]);
            if (last) break;
            if (item_seq >= 2 &&
                !__all_sync(0xffffffffu, mbar_wait(&b_empty[b], ((item_seq >> 1) - 1) & 1, p.err, s_abort)))
                break;
            // the item's queries into B: row j = query j, 16 chunks of 16
            // bytes; rows past n_pairs keep earlier (finite) contents
            const int npad = (it.n_pairs + 15) & ~15;
            const uint32_t bt = su32(sB + b * B_BUF_BYTES);
            const __half* q16 = static_cast<const __half*>(p.q16);
            for (int i = 0; i < npad / 2; i++) {
                const int e = i * 32 + lane, j = e >> 4, c = e & 15;
                const int32_t va = __shfl_sync(0xffffffffu, ca.q, j & 31);
                const int32_t vb = __shfl_sync(0xffffffffu, cb.q, j & 31);
                if (j < it.n_pairs) {
                    const int32_t q = j < 32 ? va : vb;
                    const uint32_t dst = bt + (uint32_t)((c >> 3) * NQ * 128 + j * 128 + (((c & 7) ^ (j & 7)) << 4));
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                                 "l"(q16 + (int64_t)q * 128 + c * 8)
                                 : "memory");
                }
            }
            asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&b_full[b]);
            item_seq++;
        }
    } else if (warp == 4) {
        // ---------------- MMA issue (one thread)
        if (lane == 0) {
            int item_seq = 0, tile_seq = 0;
            while (true) {
                const int m = item_seq % M_RING, b = item_seq & 1;
                if (!mbar_wait(&m_full[m], (item_seq / M_RING) & 1, p.err, s_abort)) break;
                const LmsItem it = meta[m];
                mbar_arrive(&m_empty[m]);
                if (it.n_rows < 0) break;
                if (!mbar_wait(&b_full[b], (item_seq >> 1) & 1, p.err, s_abort)) break;
                const int npad = (it.n_pairs + 15) & ~15;
                const uint32_t idesc = idesc_f16(npad);
                const int ntiles = (it.n_rows + TM - 1) / TM;
                const uint32_t b_base = su32(sB + b * B_BUF_BYTES);
                bool ok = true;
                for (int t = 0; t < ntiles; t++, tile_seq++) {
                    const int s = tile_seq % A_STAGES, tb = tile_seq % T_BUFS;
                    if (!mbar_wait(&a_full[s], (tile_seq / A_STAGES) & 1, p.err, s_abort)) {
                        ok = false;
                        break;
                    }
                    if (tile_seq >= T_BUFS &&
                        !mbar_wait(&t_empty[tb], ((tile_seq / T_BUFS) - 1) & 1, p.err, s_abort)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = su32(sA + s * A_STAGE_BYTES);
                    for (int j = 0; j < ksteps; j++) {
                        const uint32_t ao = (uint32_t)((j >> 2) * TM * 128 + (j & 3) * 32);
                        const uint32_t bo = (uint32_t)((j >> 2) * NQ * 128 + (j & 3) * 32);
                        mma_f16(tmem + (uint32_t)(tb * NQ), sdesc(a_base + ao), sdesc(b_base + bo), idesc,
                                j > 0 ? 1u : 0u);
                    }
                    mma_commit(&a_empty[s]);
                    mma_commit(&t_full[tb]);
                }
                if (!ok) break;
                // the item's queries may be replaced once its MMAs are done
                if (ntiles > 0) mma_commit(&b_empty[b]);
                else mbar_arrive(&b_empty[b]);
                item_seq++;
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: one TMEM lane quarter per warp
        const int quarter = warp & 3;
        const int prow = quarter * 32 + lane;
        int item_seq = 0, tile_seq = 0;
        while (true) {
            const int m = item_seq % M_RING;
            if (!__all_sync(0xffffffffu, mbar_wait(&m_full[m], (item_seq / M_RING) & 1, p.err, s_abort))) break;
            const LmsItem it = meta[m];
            if (it.n_rows < 0) break;
            const ColInfo* ci = cols + m * NQ;
            const int ntiles = (it.n_rows + TM - 1) / TM;
            const int64_t row0 = it.row0;
            bool ok = true;
            for (int t = 0; t < ntiles; t++, tile_seq++) {
                const int tb = tile_seq % T_BUFS;
                // the row's term is loaded before the wait, so its latency
                // overlaps the MMA
                const int lr = t * TM + prow;
                const bool valid = lr < it.n_rows;
                const int64_t grow = row0 + lr;
                const float term = valid ? __ldg(p.term + grow) : __int_as_float(0x7f800000);
                if (!__all_sync(0xffffffffu, mbar_wait(&t_full[tb], (tile_seq / T_BUFS) & 1, p.err, s_abort))) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                float acc[NQ];
                const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(tb * NQ);
                tmem_ld32(ta, acc);
                if (it.n_pairs > 32) tmem_ld32(ta + 32, acc + 32);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&t_empty[tb]);
                const int np16 = (it.n_pairs + 15) >> 4;
                uint32_t* wbal = escr + (warp - 5) * 128;
                if (np16 <= 1) epi_tile<16>(p, ci, acc, it.n_pairs, valid, grow, term, it.row_begin + lr, wbal);
                else if (np16 == 2) epi_tile<32>(p, ci, acc, it.n_pairs, valid, grow, term, it.row_begin + lr, wbal);
                else if (np16 == 3) epi_tile<48>(p, ci, acc, it.n_pairs, valid, grow, term, it.row_begin + lr, wbal);
                else epi_tile<64>(p, ci, acc, it.n_pairs, valid, grow, term, it.row_begin + lr, wbal);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&m_empty[m]);
            if (!ok) break;
            item_seq++;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 4) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ---------------------------------------------------------------------------
// Batch preparation and the work queue.

// One warp per query: the FP16 query row (K padded to 128 with zeros), its
// error bound and slack scale for the band merge, the merge state, and the
// first chunk's candidate count (every row of its lists).
__global__ void lms_prep_kernel(const float* __restrict__ Q, int64_t nq, int dim, const int32_t* __restrict__ probe_ids,
                                const float* __restrict__ probe_d, const int32_t* __restrict__ nprobe, int np_max,
                                const int32_t* __restrict__ fallback, const int32_t* __restrict__ list_len, int first_w,
                                int min_nprobe, LmsBound bd, int mode, const int32_t* __restrict__ kq, int rfixed,
                                int32_t* __restrict__ bandk, float* __restrict__ eps_out, __half* __restrict__ q16,
                                float* __restrict__ e2,
                                float* __restrict__ asl, int32_t* __restrict__ cnt, int32_t* __restrict__ lcount,
                                float* __restrict__ thr, int32_t* __restrict__ need) {
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= nq) return;
    float s = 0.0f, e = 0.0f, amax = 0.0f;
    for (int j = lane; j < 128; j += 32) {
        const float v = j < dim ? Q[q * dim + j] : 0.0f;
        const __half h = __float2half_rn(v);
        q16[q * 128 + j] = h;
        const float d = v - __half2float(h);
        s = fmaf(v, v, s);
        e = fmaf(d, d, e);
        amax = fmaxf(amax, fabsf(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        e += __shfl_xor_sync(0xffffffffu, e, o);
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    }
    const int np = min(nprobe[q], np_max);
    int c0 = 0;
    for (int i = lane; i < min(first_w, np); i += 32) c0 += list_len[probe_ids[q * np_max + i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c0 += __shfl_xor_sync(0xffffffffu, c0, o);
    if (lane == 0) {
        const float qn = sqrtf(s) * 1.0001f, qd = sqrtf(e) * 1.0001f;
        const float u22 = 2.384185791015625e-7f;
        // |<q, r> - <q~, r~>| <= |q| |r - r~| + |q - q~| |r| + |q - q~| |r - r~|, plus the
        // tensor core's FP32 accumulation; the score carries the factor 2
        const float eps = 2.0f * (qn * bd.rd + qd * bd.rmax + qd * bd.rd) +
                          2.0f * (float)bd.kpad * u22 * (qn + qd) * (bd.rmax + bd.rd);
        const float bmax = np > 0 ? probe_d[q * np_max + np - 1] : 0.0f;
        eps_out[q] = eps;
        if (mode == 0) {
            e2[q] = 2.0f * eps;
            asl[q] = bmax + bd.tmax + 2.0f * qn * bd.rmax;
        } else {
            // exact rerank of the best R by s~: no band past the ties
            e2[q] = 0.0f;
            asl[q] = 0.0f;
        }
        // a component FP16 cannot hold (or a non-finite one) sends the query
        // to the table scan, as does the brute-force fallback
        // so does a query probing fewer lists than min_nprobe (the table scan
        // is faster there; the choice depends on the query alone)
        const bool fb = fallback[q] != 0 || !(amax <= 6.0e4f) || !(s < 3.0e38f) || np < min_nprobe;
        need[q] = fb ? 1 : 0;
        lcount[q] = 0;
        thr[q] = __int_as_float(0x7f800000);
        // the band keeps the query's k best (parity: every row the reference's
        // top k can be) or its rerank depth (exact rerank)
        bandk[q] = mode == 0 ? kq[q] : rerank_depth_for(kq[q], mode, rfixed);
        cnt[q] = fb ? 0 : c0;
    }
}

// (query, probe rank) pairs counted per (chunk, list).
__global__ void lms_count_kernel(const int32_t* __restrict__ probe_ids, const int32_t* __restrict__ nprobe,
                                 int64_t nq, int np_max, const int32_t* __restrict__ fallback, LmsChunks ch, int nlist,
                                 int32_t* __restrict__ counts) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nq * np_max) return;
    const int64_t q = e / np_max;
    const int i = (int)(e - q * np_max);
    if (fallback[q] || i >= nprobe[q]) return;
    int c = 0;
    while (c + 1 < ch.n && i >= ch.bound[c + 1]) c++;
    atomicAdd(&counts[(int64_t)c * nlist + probe_ids[e]], 1);
}

// Exclusive prefix of n ints in place (one block of 1024 threads), the total
// in *total.
__global__ void lms_scan_counts_kernel(int32_t* __restrict__ v, int n, int32_t* __restrict__ total) {
    __shared__ int32_t wsum[32];
    __shared__ int32_t carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < n; b += 1024) {
        const int i = b + t;
        const int x = i < n ? v[i] : 0;
        int incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            const int tot = wsum[lane];
            int y = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int z = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) y += z;
            }
            wsum[lane] = y - tot;
        }
        __syncthreads();
        const int c = carry;
        if (i < n) v[i] = c + wsum[w] + incl - x;
        __syncthreads();
        if (t == 1023) carry = c + wsum[w] + incl;
        __syncthreads();
    }
    if (t == 0) *total = carry;
}

// Work items of every (chunk, list) with pairs: ceil(pairs / NQ) query
// groups times ceil(len / rows_max) row ranges, placed in the chunk's item
// region by an atomic counter. cursor receives a copy of the offsets (the
// scatter's fill pointers).
__global__ void lms_items_kernel(const int32_t* __restrict__ offsets, const int32_t* __restrict__ total, int nch,
                                 int nlist, const int32_t* __restrict__ list_len,
                                 const int64_t* __restrict__ list_start, int rows_max, int item_cap,
                                 LmsItem* __restrict__ items, int32_t* __restrict__ n_items,
                                 int32_t* __restrict__ cursor, int32_t* __restrict__ overflow) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)nch * nlist) return;
    const int c = (int)(e / nlist), l = (int)(e - (int64_t)c * nlist);
    const int32_t off = offsets[e];
    const int32_t end = e + 1 < (int64_t)nch * nlist ? offsets[e + 1] : *total;
    cursor[e] = off;
    const int n = end - off, len = list_len[l];
    if (n <= 0 || len <= 0) return;
    const int gq = (n + NQ - 1) / NQ, gr = (len + rows_max - 1) / rows_max;
    const int base = atomicAdd(&n_items[c], gq * gr);
    if (base + gq * gr > item_cap) {
        atomicExch(overflow, 1);
        return;
    }
    LmsItem* out = items + (int64_t)c * item_cap + base;
    for (int a = 0; a < gq; a++)
        for (int r = 0; r < gr; r++) {
            LmsItem it;
            it.list = l;
            it.pair_begin = off + a * NQ;
            it.n_pairs = min(NQ, n - a * NQ);
            it.row_begin = r * rows_max;
            it.n_rows = min(rows_max, len - r * rows_max);
            it.pad = 0;
            it.row0 = list_start[l] + (int64_t)it.row_begin;
            out[a * gr + r] = it;
        }
}

// Every pair to its (chunk, list) group: query, ||q - c||^2 and, for the
// first chunk, the position of the list's rows in the query's buffer (the
// lengths of the query's nearer lists in that chunk).
__global__ void lms_scatter_kernel(const int32_t* __restrict__ probe_ids, const float* __restrict__ probe_d,
                                   const int32_t* __restrict__ nprobe, int64_t nq, int np_max,
                                   const int32_t* __restrict__ fallback, LmsChunks ch, int nlist,
                                   const int32_t* __restrict__ list_len, int32_t* __restrict__ cursor,
                                   int32_t* __restrict__ pair_q, float* __restrict__ pair_base,
                                   int32_t* __restrict__ pair_off) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nq * np_max) return;
    const int64_t q = e / np_max;
    const int i = (int)(e - q * np_max);
    if (fallback[q] || i >= nprobe[q]) return;
    int c = 0;
    while (c + 1 < ch.n && i >= ch.bound[c + 1]) c++;
    const int l = probe_ids[e];
    const int slot = atomicAdd(&cursor[(int64_t)c * nlist + l], 1);
    pair_q[slot] = (int32_t)q;
    pair_base[slot] = probe_d[e];
    int off = 0;
    if (c == 0)
        for (int j = 0; j < i; j++) off += list_len[probe_ids[q * np_max + j]];
    pair_off[slot] = off;
}

// Band lists to the rerank's candidates, one warp per query: the R best keys
// (all of them when they fit; in parity mode a band that does not fit sends
// the query to the table scan), each with its list's probe position as the
// tie-breaking sequence. Queries flagged for the table scan are appended to
// redo (count in redo[nq]).
__global__ void lms_finish_kernel(int64_t nq, int mode, int R, int lcap, const int32_t* __restrict__ kq, int rfixed,
                                  const unsigned long long* __restrict__ list, const int32_t* __restrict__ lcount,
                                  const int32_t* __restrict__ need, const int32_t* __restrict__ probe_ids,
                                  const int32_t* __restrict__ nprobe, int np_max,
                                  const int32_t* __restrict__ row_cluster, const int32_t* __restrict__ overflow,
                                  int32_t* __restrict__ cand_row, uint32_t* __restrict__ cand_seq,
                                  int32_t* __restrict__ redo) {
    extern __shared__ __align__(16) unsigned long long fk[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + w;
    if (q >= nq) return;
    unsigned long long* keys = fk + (int64_t)w * (lcap + 64);
    unsigned int* hist = reinterpret_cast<unsigned int*>(fk + (int64_t)(blockDim.x >> 5) * (lcap + 64)) + w * 256;
    const int L = lcount[q];
    const int Rq = min(R, rerank_depth_for(kq[q], mode, rfixed));
    const bool flag = need[q] != 0 || (mode == 0 && L > R) || *overflow != 0;
    if (flag) {
        if (lane == 0) redo[atomicAdd(&redo[nq], 1)] = (int32_t)q;
        for (int i = lane; i < R; i += 32) {
            cand_row[q * R + i] = -1;
            cand_seq[q * R + i] = 0xffffffffu;
        }
        return;
    }
    int take = L;
    unsigned long long K = ~0ull;
    if (mode != 0 && L > Rq) {
        for (int i = lane; i < L; i += 32) keys[i] = list[q * lcap + i];
        __syncwarp();
        K = warp_radix_nth_u64(keys, L, Rq, hist);
        take = Rq;
    }
    const int np = min(nprobe[q], np_max);
    int m = 0;
    for (int i0 = 0; i0 < L; i0 += 32) {
        const int i = i0 + lane;
        const unsigned long long key = i < L ? list[q * lcap + i] : ~0ull;
        const bool keep = i < L && key <= K;
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int pos = m + __popc(b & ((1u << lane) - 1u));
            const int32_t row = (int32_t)(key & 0xffffffffull);
            const int32_t cl = row_cluster[row];
            uint32_t seq = 0xffffffffu;
            for (int j = 0; j < np; j++)
                if (probe_ids[q * np_max + j] == cl) {
                    seq = (uint32_t)j;
                    break;
                }
            if (pos < R) {
                cand_row[q * R + pos] = row;
                cand_seq[q * R + pos] = seq;
            }
        }
        m += __popc(b);
    }
    for (int i = min(take, R) + lane; i < R; i += 32) {
        cand_row[q * R + i] = -1;
        cand_seq[q * R + i] = 0xffffffffu;
    }
}

}  // namespace

// The first threshold of every query from the table scan of its nearest list
// (cand_d [nq][R]: the best scores, +inf past the count; their largest is at
// or above the R-th best of that list). Every row the final band can hold
// has a screened score at or below
//   the band's k-th best + e2 + slack <= (that largest + eps) + e2 + slack,
// eps covering the FP16 screen against the table's FP32 scores, so the
// threshold below drops none of them. Queries whose nearest list holds fewer
// rows than their band start at +inf.
__global__ void lms_seed_kernel(int64_t nq, int R, const float* __restrict__ cand_d, const int32_t* __restrict__ bandk,
                                const float* __restrict__ eps, const float* __restrict__ e2,
                                const float* __restrict__ asl, float* __restrict__ thr) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int cnt = 0;
    float mx = -__int_as_float(0x7f800000);
    for (int i = 0; i < R; i++) {
        const float d = cand_d[q * R + i];
        if (d < __int_as_float(0x7f800000)) {
            cnt++;
            mx = fmaxf(mx, d);
        }
    }
    float t = __int_as_float(0x7f800000);
    if (cnt >= bandk[q] && cnt > 0) {
        const float a = fabsf(mx) + asl[q];
        t = mx + eps[q] + e2[q] + 2e-5f * a + 1e-6f * fabsf(mx);
    }
    thr[q] = t;
}

cudaError_t launch_lms_seed(int64_t nq, int R, const float* cand_d, const int32_t* bandk, const float* eps,
                            const float* e2, const float* asl, float* thr, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    lms_seed_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(nq, R, cand_d, bandk, eps, e2, asl, thr);
    return cudaGetLastError();
}

int lms_smem_bytes() { return smem_fixed(3) + CB_SMEM_MAX; }

bool lms_supported(int dim, int M, int pqK) {
    return dim > 0 && dim <= 128 && M > 0 && dim % M == 0 && pqK >= 1 && pqK <= 256;
}

cudaError_t launch_lms_prep(const float* Q, int64_t nq, int dim, const int32_t* probe_ids, const float* probe_d,
                            const int32_t* nprobe, int np_max, const int32_t* fallback, const int32_t* list_len,
                            int first_w, int min_nprobe, const LmsBound& bd, int mode, const int32_t* kq, int rfixed,
                            int32_t* bandk, float* eps, void* q16, float* e2, float* asl, int32_t* cnt,
                            int32_t* lcount, float* thr, int32_t* need, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    lms_prep_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(Q, nq, dim, probe_ids, probe_d, nprobe, np_max, fallback,
                                                              list_len, first_w, min_nprobe, bd, mode, kq, rfixed, bandk,
                                                              eps,
                                                              static_cast<__half*>(q16), e2, asl, cnt, lcount, thr,
                                                              need);
    return cudaGetLastError();
}

cudaError_t launch_lms_queue(const int32_t* probe_ids, const float* probe_d, const int32_t* nprobe, int64_t nq,
                             int np_max, const int32_t* fallback, const LmsChunks& ch, int nlist,
                             const int32_t* list_len, const int64_t* list_start, int rows_max, int item_cap,
                             int32_t* counts, int32_t* cursor,
                             int32_t* totals, LmsItem* items, int32_t* n_items, int32_t* pair_q, float* pair_base,
                             int32_t* pair_off, cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    const int64_t ncl = (int64_t)ch.n * nlist;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int32_t) * ncl, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(totals, 0, 2 * sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(n_items, 0, sizeof(int32_t) * ch.n, s);
    if (e != cudaSuccess) return e;
    const int64_t np = nq * np_max;
    lms_count_kernel<<<(unsigned)ceil_div(np, 256), 256, 0, s>>>(probe_ids, nprobe, nq, np_max, fallback, ch, nlist,
                                                                 counts);
    lms_scan_counts_kernel<<<1, 1024, 0, s>>>(counts, (int)ncl, totals);
    lms_items_kernel<<<(unsigned)ceil_div(ncl, 256), 256, 0, s>>>(counts, totals, ch.n, nlist, list_len, list_start,
                                                                  rows_max, item_cap, items, n_items, cursor,
                                                                  totals + 1);
    lms_scatter_kernel<<<(unsigned)ceil_div(np, 256), 256, 0, s>>>(probe_ids, probe_d, nprobe, nq, np_max, fallback,
                                                                   ch, nlist, list_len, cursor, pair_q, pair_base,
                                                                   pair_off);
    return cudaGetLastError();
}

cudaError_t launch_lms_scan(const LmsParams& p, int grid, cudaStream_t s) {
    const void* fn;
    switch (p.dsub) {
    case 4: fn = (const void*)lms_scan_kernel<4>; break;
    case 8: fn = (const void*)lms_scan_kernel<8>; break;
    default: fn = (const void*)lms_scan_kernel<0>; break;
    }
    const int smem = smem_fixed(a_stages(p.dim, p.pqK)) + cb_smem_bytes(p.dim, p.pqK);
    if (cb_smem_bytes(p.dim, p.pqK) > CB_SMEM_MAX) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(p.item_counter, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    LmsParams pp = p;
    void* args[] = {(void*)&pp};
    e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(LMS_THREADS), args, smem, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

size_t lms_finish_smem(int lcap) { return 8 * ((size_t)(lcap + 64) * 8 + 256 * 4); }

cudaError_t launch_lms_finish(int64_t nq, int mode, int R, int lcap, const int32_t* kq, int rfixed,
                              const unsigned long long* list, const int32_t* lcount, const int32_t* need,
                              const int32_t* probe_ids, const int32_t* nprobe, int np_max, const int32_t* row_cluster,
                              const int32_t* overflow, int32_t* cand_row, uint32_t* cand_seq, int32_t* redo,
                              cudaStream_t s) {
    if (nq <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(redo + nq, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    const size_t smem = lms_finish_smem(lcap);
    e = cudaFuncSetAttribute(lms_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lms_finish_kernel<<<(unsigned)ceil_div(nq, 8), 256, smem, s>>>(nq, mode, R, lcap, kq, rfixed, list, lcount, need,
                                                                  probe_ids, nprobe, np_max, row_cluster, overflow,
                                                                  cand_row, cand_seq, redo);
    return cudaGetLastError();
}

}  // namespace hann
