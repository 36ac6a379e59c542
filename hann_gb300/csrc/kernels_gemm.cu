// kernels_gemm.cu -- BF16 tensor-core distance GEMM for sm_103a (tcgen05 +
// TMA + TMEM), used to preselect coarse lists and k-means centroids.
//
// For rows a (queries or points) and columns b (centroids) it computes the
// ranking score s(a, b) = ||b||^2 - 2 <a, b> with BF16 operands and FP32
// accumulation: tcgen05.mma.kind::f16 issued by one thread, operands staged
// in shared memory by TMA (128-byte swizzle), the accumulator in tensor
// memory, read back by four epilogue warps with tcgen05.ld. The score is an
// approximation; the callers turn it into the reference's exact result by
// rescoring, in FP32 and the reference's summation order, every column whose
// score lies within 2*eps of the boundary, where eps bounds the BF16 and
// FP32 rounding (bf16_score_eps in common.cuh).
//
// Block layout: warp 0 issues TMA loads, warp 1 allocates tensor memory and
// issues the MMAs, warps 2..5 drain the accumulator. The A tile (128 rows x
// K <= 128) is loaded once; B tiles of 256 columns stream through two shared
// memory stages; two 256-column accumulators in tensor memory let the
// epilogue of one tile overlap the MMAs of the next.
//
// Every wait on an mbarrier is bounded: after SPIN_LIMIT polls the kernel
// records an error in *err, stops issuing work, and still reaches the final
// barrier and the tensor-memory release.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace hann {
namespace {

constexpr int BM = 128;       // rows per CTA (MMA M)
constexpr int BN = 256;       // columns per tile (MMA N)
constexpr int BKE = 64;       // bf16 elements per 128-byte swizzle row
constexpr int KB_MAX = 2;     // K <= 128
constexpr int STAGES = 2;
// Warp 0 loads, warp 1 issues the MMAs, then EW epilogue warps per quarter
// of the accumulator's 128 lanes: two for the score mode, four for the
// top-8 and filter modes, each taking its share of a tile's columns, so
// several warps per SM sub-partition hide each other's latency. In the top-8
// mode each warp keeps a list over its columns and the lists of a row are
// merged at the end.
template <int MODE>
struct Epi {
    static constexpr int EW = MODE == 0 ? 2 : 4;
    static constexpr int THREADS = 64 + 128 * EW;
    static constexpr int CW = 256 / EW;  // columns per epilogue warp
    static constexpr int LDC = MODE == 0 ? 64 : 32;  // accumulator columns per TMEM wait
};
constexpr int TOPC = 8;       // argmin mode: candidates kept per row
constexpr uint32_t SPIN_LIMIT = 1u << 22;

constexpr int A_BYTES = KB_MAX * BM * 128;           // 32 KiB
constexpr int B_STAGE_BYTES = KB_MAX * BN * 128;     // 64 KiB
constexpr int TR_BYTES = 8 * 32 * 33 * 4;               // epilogue transpose tiles (up to 8 warps)
constexpr int CT_BYTES = 4 * 2 * BN * 8;                // column terms of two tiles, split over the warps
constexpr int SMEM_BYTES = 1024 + A_BYTES + STAGES * B_STAGE_BYTES + 256 + TR_BYTES + CT_BYTES;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(su32(b)),
                 "r"(bytes)
                 : "memory");
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
// Bounded wait; false (and *err set) when the limit is reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err) {
    for (uint32_t i = 0; i < SPIN_LIMIT; i++)
        if (mbar_try(b, parity)) return true;
    atomicExch(err, 1);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            su32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(su32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// Instruction descriptor: BF16 x BF16 -> FP32, both K-major, M=128, N=256.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
            dtmem),
        "l"(ad), "l"(bd), "r"(IDESC), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 columns of the warp's 32 lanes into v[0..32), load and wait in one asm
// statement.
__device__ __forceinline__ void tmem_ld32w(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 64 columns of the warp's 32 lanes into v[0..64): two 32-column loads in
// flight, then one wait, all in one asm statement so no use of v can be
// scheduled before the wait.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 64; i++) v[i] = __uint_as_float(r[i]);
}

// MODE 0: write the score matrix S[row][col] (ld = ncols).
// MODE 1: per row, the TOPC smallest scores and their columns, ascending.
// MODE 2: columns [col_begin, ncols) only; the score is
//         cterm[col].x + cterm[col].y * <a~, b~> (one rounding) and every
//         column with score <= rthr[row] is appended to the row's candidate
//         buffer (cand_idx / cand_val, cap entries, count in cnt[row]; the
//         count keeps growing past cap so the caller sees the overflow).
//         cmode 0: cterm[col].y is -2 for every column; cmode 1: cterm[col].x
//         is 0 for every column (so one float per column is staged).
template <int MODE>
__global__ void __launch_bounds__(Epi<MODE>::THREADS, 1) dist_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
                                                              const __grid_constant__ CUtensorMap map_b, int nrows,
                                                              int ncols, int kp, int tiles_per_split,
                                                              const float* __restrict__ bias,
                                                              float* __restrict__ out, int32_t* __restrict__ cand_idx,
                                                              float* __restrict__ cand_val, int* __restrict__ err,
                                                              int col_begin, const float2* __restrict__ cterm,
                                                              int cmode, const float* __restrict__ rthr, int cap,
                                                              int32_t* __restrict__ cnt, int dense) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = base;
    unsigned char* sB = base + A_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + STAGES * B_STAGE_BYTES);
    uint64_t* full = bars;            // [STAGES] B stage loaded
    uint64_t* empty = bars + 2;       // [STAGES] B stage consumed by the MMAs
    uint64_t* tfull = bars + 4;       // [2] accumulator ready
    uint64_t* tempty = bars + 6;      // [2] accumulator drained
    uint64_t* afull = bars + 8;       // A tile loaded
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 9);
    int* s_abort = reinterpret_cast<int*>(bars + 10);
    float* trans = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(bars) + 256);
    float2* cts = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(trans) + TR_BYTES);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * BM;
    const int kb = (kp + BKE - 1) / BKE;
    const int ksteps = (kp + 15) / 16;
    // this CTA's column tiles: [t0, t0 + ntiles) of columns [col_begin, ncols)
    const int t0 = blockIdx.y * tiles_per_split;
    const int ntiles = max(0, min((ncols - col_begin + BN - 1) / BN - t0, tiles_per_split));

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4 * Epi<MODE>::EW);
        }
        mbar_init(afull, 1);
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            mbar_expect_tx(afull, (uint32_t)(kb * BM * 128));
            for (int b = 0; b < kb; b++) tma_load_2d(sA + b * BM * 128, &map_a, b * BKE, row0, afull);
            for (int t = 0; t < ntiles; t++) {
                const int s = t % STAGES;
                if (t >= STAGES && !mbar_wait(&empty[s], ((t / STAGES) - 1) & 1, err)) {
                    *s_abort = 1;
                    break;
                }
                if (*(volatile int*)s_abort) break;
                mbar_expect_tx(&full[s], (uint32_t)(kb * BN * 128));
                for (int b = 0; b < kb; b++)
                    tma_load_2d(sB + s * B_STAGE_BYTES + b * BN * 128, &map_b, b * BKE, col_begin + (t0 + t) * BN,
                                &full[s]);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = mbar_wait(afull, 0, err);
            const uint32_t a_base = su32(sA);
            for (int t = 0; ok && t < ntiles; t++) {
                const int s = t % STAGES, buf = t & 1;
                if (!mbar_wait(&full[s], (t / STAGES) & 1, err)) break;
                if (t >= 2 && !mbar_wait(&tempty[buf], ((t >> 1) - 1) & 1, err)) break;
                if (*(volatile int*)s_abort) break;
                tc_fence_after();
                const uint32_t b_base = su32(sB + s * B_STAGE_BYTES);
                for (int j = 0; j < ksteps; j++) {
                    const uint32_t off = (uint32_t)((j >> 2) * BM * 128 + (j & 3) * 32);
                    const uint32_t offb = (uint32_t)((j >> 2) * BN * 128 + (j & 3) * 32);
                    mma_bf16(tmem + (uint32_t)(buf * BN), sdesc(a_base + off), sdesc(b_base + offb), j > 0 ? 1u : 0u);
                }
                mma_commit(&empty[s]);
                mma_commit(&tfull[buf]);
            }
        }
    } else {
        // Epilogue: warp w drains tensor-memory lanes 32*(w%4) .. +31, one
        // row per lane. Each warp stages the tile's per-column terms (bias,
        // scale) in its own shared-memory slice, fetched one tile ahead, so
        // the 256 columns are read as broadcasts instead of 256 global loads
        // per lane; the accumulator comes out 64 columns per wait.
        constexpr int CW = Epi<MODE>::CW;
        // tcgen05.ld lets warp w read only TMEM lanes 32 (w % 4) .. + 31
        const int ew = warp - 2, quarter = warp & 3, cbeg = (ew >> 2) * CW;
        const int row = row0 + quarter * 32 + lane;
        // this warp's columns of two tiles: the bias (scores b - 2v) or, in
        // filter mode 1, the scale (scores w v)
        float* wct = reinterpret_cast<float*>(cts) + ew * 2 * CW;
        float best_v[TOPC];
        int best_i[TOPC];
#pragma unroll
        for (int c = 0; c < TOPC; c++) {
            best_v[c] = __int_as_float(0x7f800000);
            best_i[c] = -1;
        }
        const float rt = (MODE == 2 && row < nrows) ? rthr[row] : -__int_as_float(0x7f800000);
        // invalid columns: +inf scores (modes 0, 1), NaN (mode 2, never passes)
        const float pad = MODE == 2 ? __int_as_float(0x7fc00000) : __int_as_float(0x7f800000);
        const bool scaled = MODE == 2 && cmode == 1;
        float pre[CW / 32];
        auto fetch = [&](int t) {
            const int colb = col_begin + (t0 + t) * BN + cbeg;
#pragma unroll
            for (int j = 0; j < CW / 32; j++) {
                const int col = colb + 32 * j + lane;
                if (col < ncols) {
                    if (MODE == 2) {
                        const float2 tt = __ldg(cterm + col);
                        pre[j] = scaled ? tt.y : tt.x;
                    } else {
                        pre[j] = __ldg(bias + col);
                    }
                } else {
                    pre[j] = pad;
                }
            }
        };
        auto score = [&](float tc, float v) { return scaled ? __fmul_rn(tc, v) : __fmaf_rn(-2.0f, v, tc); };
        if (ntiles > 0) fetch(0);
        for (int t = 0; t < ntiles; t++) {
            const int buf = t & 1;
            float* ct = wct + buf * CW;
#pragma unroll
            for (int j = 0; j < CW / 32; j++) ct[32 * j + lane] = pre[j];
            __syncwarp();
            if (t + 1 < ntiles) fetch(t + 1);
            // a warp leaves together when a wait runs out
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], (t >> 1) & 1, err));
            if (!ok) break;
            tc_fence_after();
            const int col0 = col_begin + (t0 + t) * BN + cbeg;
            constexpr int LDC = Epi<MODE>::LDC;
            for (int c = 0; c < CW; c += LDC) {
                float v[LDC];
                const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * BN + cbeg + c);
                if constexpr (LDC == 64) tmem_ld64(ta, *reinterpret_cast<float(*)[64]>(v));
                else tmem_ld32w(ta, v);
                if (MODE == 0) {
                    // Transpose 32 rows x 32 columns at a time through shared
                    // memory so each store writes 128 contiguous bytes of a row.
                    float* tw = trans + ew * 32 * 33;
                    const int rbase = row0 + quarter * 32;
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int cb = col0 + c + 32 * h;
                        const float bl = ct[c + 32 * h + lane];
#pragma unroll
                        for (int i = 0; i < 32; i++) tw[lane * 33 + i] = v[32 * h + i];
                        __syncwarp();
                        if (cb + lane < ncols) {
                            for (int rr = 0; rr < 32; rr++) {
                                if (rbase + rr < nrows)
                                    out[(int64_t)(rbase + rr) * ncols + cb + lane] =
                                        __fmaf_rn(-2.0f, tw[rr * 33 + lane], bl);
                            }
                        }
                        __syncwarp();
                    }
                } else if (MODE == 2 && dense) {
                    // First chunk (every threshold +inf, every column kept):
                    // column col_begin + i goes to slot i, four at a time,
                    // and the row's count is the chunk's width.
                    if (row < nrows) {
                        const int width = ncols - col_begin;
                        const int pos0 = col0 + c - col_begin;
                        int32_t* ri = cand_idx + (int64_t)row * cap;
                        float* rv = cand_val + (int64_t)row * cap;
#pragma unroll
                        for (int i4 = 0; i4 < LDC / 4; i4++) {
                            const int pos = pos0 + 4 * i4;
                            if (pos + 3 < width) {
                                *reinterpret_cast<int4*>(ri + pos) =
                                    make_int4(col0 + c + 4 * i4, col0 + c + 4 * i4 + 1, col0 + c + 4 * i4 + 2,
                                              col0 + c + 4 * i4 + 3);
                                *reinterpret_cast<float4*>(rv + pos) = make_float4(
                                    score(ct[c + 4 * i4], v[4 * i4]), score(ct[c + 4 * i4 + 1], v[4 * i4 + 1]),
                                    score(ct[c + 4 * i4 + 2], v[4 * i4 + 2]), score(ct[c + 4 * i4 + 3], v[4 * i4 + 3]));
                            } else {
#pragma unroll
                                for (int u = 0; u < 4; u++) {
                                    if (pos + u < width) {
                                        ri[pos + u] = col0 + c + 4 * i4 + u;
                                        rv[pos + u] = score(ct[c + 4 * i4 + u], v[4 * i4 + u]);
                                    }
                                }
                            }
                        }
                        if (blockIdx.y == 0 && t == 0 && cbeg == 0 && c == 0) cnt[row] = width;
                    }
                } else if (MODE == 2) {
                    // Most rows pass no column of a tile: test the minimum
                    // score first (fminf skips the NaN pads) and build the
                    // pass mask, with the same scores, only when it passes.
                    const float4* ct4 = reinterpret_cast<const float4*>(ct + c);
                    float mn = __int_as_float(0x7f800000);
#pragma unroll
                    for (int i4 = 0; i4 < LDC / 4; i4++) {
                        const float4 tt = ct4[i4];
                        mn = fminf(mn, fminf(fminf(score(tt.x, v[4 * i4 + 0]), score(tt.y, v[4 * i4 + 1])),
                                             fminf(score(tt.z, v[4 * i4 + 2]), score(tt.w, v[4 * i4 + 3]))));
                    }
                    unsigned long long pass = 0;
                    if (mn <= rt) {
#pragma unroll
                        for (int i4 = 0; i4 < LDC / 4; i4++) {
                            const float4 tt = ct4[i4];
                            if (score(tt.x, v[4 * i4 + 0]) <= rt) pass |= 1ull << (4 * i4 + 0);
                            if (score(tt.y, v[4 * i4 + 1]) <= rt) pass |= 1ull << (4 * i4 + 1);
                            if (score(tt.z, v[4 * i4 + 2]) <= rt) pass |= 1ull << (4 * i4 + 2);
                            if (score(tt.w, v[4 * i4 + 3]) <= rt) pass |= 1ull << (4 * i4 + 3);
                        }
                    }
                    if (pass) {
                        int pos = atomicAdd(&cnt[row], __popcll(pass));
#pragma unroll
                        for (int i = 0; i < LDC; i++) {
                            if (pass & (1ull << i)) {
                                if (pos < cap) {
                                    cand_idx[(int64_t)row * cap + pos] = col0 + c + i;
                                    cand_val[(int64_t)row * cap + pos] = score(ct[c + i], v[i]);
                                }
                                pos++;
                            }
                        }
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < LDC; i++) {
                        const float sc = __fmaf_rn(-2.0f, v[i], ct[c + i]);
                        if (sc < best_v[TOPC - 1]) {
                            // insert into the ascending list
                            float cv = sc;
                            int ci = col0 + c + i;
#pragma unroll
                            for (int p = 0; p < TOPC; p++) {
                                if (cv < best_v[p]) {
                                    const float tv = best_v[p];
                                    const int ti = best_i[p];
                                    best_v[p] = cv;
                                    best_i[p] = ci;
                                    cv = tv;
                                    ci = ti;
                                }
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[buf]);
        }
        if (MODE == 1) {
            // every epilogue warp reaches this point, also after a timed-out wait
            constexpr int EW = Epi<MODE>::EW;
            float* lv = trans;                                           // [4 EW][32][TOPC]
            int* li = reinterpret_cast<int*>(trans + 4 * EW * 32 * TOPC);  // same shape
#pragma unroll
            for (int c = 0; c < TOPC; c++) {
                lv[(ew * 32 + lane) * TOPC + c] = best_v[c];
                li[(ew * 32 + lane) * TOPC + c] = best_i[c];
            }
            asm volatile("bar.sync 1, %0;" ::"n"(128 * EW) : "memory");
            if (ew < 4 && row < nrows) {
                // merge the row's other lists in, ties to the lower column
                for (int h = 1; h < EW; h++) {
                    const int src = ((ew + 4 * h) * 32 + lane) * TOPC;
                    for (int c = 0; c < TOPC; c++) {
                        float cv = lv[src + c];
                        int ci = li[src + c];
                        if (ci < 0) break;
#pragma unroll
                        for (int p = 0; p < TOPC; p++) {
                            if (cv < best_v[p] || (cv == best_v[p] && (unsigned)ci < (unsigned)best_i[p])) {
                                const float tv = best_v[p];
                                const int ti = best_i[p];
                                best_v[p] = cv;
                                best_i[p] = ci;
                                cv = tv;
                                ci = ti;
                            }
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < TOPC; c++) {
                    cand_idx[(int64_t)row * TOPC + c] = best_i[c];
                    cand_val[(int64_t)row * TOPC + c] = best_v[c];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

// Rows of x (FP32 [n][dim]) to BF16 [n][kp] with zero padding, plus the
// FP32 squared norm of each row (summed in FP32 in natural order).
__global__ void to_bf16_kernel(const float* __restrict__ x, int64_t n, int dim, int kp, __nv_bfloat16* __restrict__ out,
                               float* __restrict__ sqnorm, float* __restrict__ resid) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y;
    if (r >= n) return;
    float s = 0.0f, e = 0.0f;
    for (int j = threadIdx.x; j < kp; j += 32) {
        const float v = j < dim ? x[r * dim + j] : 0.0f;
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        out[r * kp + j] = b;
        const float d = v - __bfloat162float(b);
        s = fmaf(v, v, s);
        e = fmaf(d, d, e);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        e += __shfl_xor_sync(0xffffffffu, e, o);
    }
    if (threadIdx.x == 0) {
        if (sqnorm) sqnorm[r] = s;
        // rounded up slightly so the bound stays a bound after FP32 rounding
        if (resid) resid[r] = sqrtf(e) * 1.0001f;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

cudaError_t get_encoder() {
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return g_encode ? cudaSuccess : cudaErrorNotSupported;
}

cudaError_t make_map(CUtensorMap* m, const void* ptr, int64_t rows, int kp, int box_rows) {
    cudaError_t e = get_encoder();
    if (e != cudaSuccess) return e;
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)BKE, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int MODE>
cudaError_t launch_gemm(const __nv_bfloat16* a, int64_t nrows, const __nv_bfloat16* b, int ncols, int kp,
                        const float* bias, float* out, int32_t* cand_idx, float* cand_val, int* err, cudaStream_t s,
                        int col_begin = 0, const float2* cterm = nullptr, int cmode = 0, const float* rthr = nullptr,
                        int cap = 0, int32_t* cnt = nullptr, int dense = 0) {
    if (nrows <= 0 || ncols <= col_begin) return cudaSuccess;
    if (kp <= 0 || kp > KB_MAX * BKE || (kp & 7)) return cudaErrorInvalidValue;
    if (nrows > ((int64_t)1 << 31) - BM) return cudaErrorInvalidValue;
    CUtensorMap ma, mb;
    cudaError_t e = make_map(&ma, a, nrows, kp, BM);
    if (e != cudaSuccess) return e;
    e = make_map(&mb, b, ncols, kp, BN);
    if (e != cudaSuccess) return e;
    // set on every launch: the attribute belongs to the current device's
    // context, and launches may come from several threads and devices
    e = cudaFuncSetAttribute(dist_gemm_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    // Score matrices split the columns over CTAs so that small row counts
    // still fill the GPU (about four CTAs per SM in total).
    const int mtiles = (int)ceil_div(nrows, BM);
    const int ntiles = (int)ceil_div(ncols - col_begin, BN);
    int splits = 1;
    if (MODE == 0) splits = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, ceil_div(4 * 152, mtiles)));
    // filter mode: about eight waves of CTAs, as many as the column tiles allow
    if (MODE == 2) splits = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, ceil_div(8 * 152, mtiles)));
    const int per = (int)ceil_div(ntiles, splits);
    splits = (int)ceil_div(ntiles, per);
    dist_gemm_kernel<MODE><<<dim3((unsigned)mtiles, (unsigned)splits), Epi<MODE>::THREADS, SMEM_BYTES, s>>>(
        ma, mb, (int)nrows, ncols, kp, per, bias, out, cand_idx, cand_val, err, col_begin, cterm, cmode, rthr, cap,
        cnt, dense);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm_filter(const void* a_bf16, int64_t nrows, const void* b_bf16, int64_t nb, int kp,
                               int col_begin, int col_end, const float2* cterm, int cmode, const float* rthr, int cap,
                               int32_t* cnt, int32_t* cand_id, float* cand_s, int* err, cudaStream_t s, bool first) {
    // the tensor map spans all nb rows of b; the CTAs cover [col_begin, col_end)
    if (col_end > nb) return cudaErrorInvalidValue;
    const int dense = first && col_end - col_begin <= cap ? 1 : 0;
    return launch_gemm<2>(static_cast<const __nv_bfloat16*>(a_bf16), nrows, static_cast<const __nv_bfloat16*>(b_bf16),
                          (int)col_end, kp, nullptr, nullptr, cand_id, cand_s, err, s, col_begin, cterm, cmode, rthr,
                          cap, cnt, dense);
}

int gemm_kpad(int dim) { return (dim + 7) / 8 * 8; }
int gemm_topc() { return TOPC; }

cudaError_t launch_to_bf16(const float* x, int64_t n, int dim, int kp, void* out_bf16, float* sqnorm, float* resid,
                           cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    dim3 blk(32, 8);
    to_bf16_kernel<<<(unsigned)ceil_div(n, 8), blk, 0, s>>>(x, n, dim, kp, static_cast<__nv_bfloat16*>(out_bf16),
                                                            sqnorm, resid);
    return cudaGetLastError();
}

cudaError_t launch_gemm_scores(const void* a_bf16, int64_t nrows, const void* b_bf16, int ncols, int kp,
                               const float* bias, float* out, int* err, cudaStream_t s) {
    return launch_gemm<0>(static_cast<const __nv_bfloat16*>(a_bf16), nrows, static_cast<const __nv_bfloat16*>(b_bf16),
                          ncols, kp, bias, out, nullptr, nullptr, err, s);
}

cudaError_t launch_gemm_top8(const void* a_bf16, int64_t nrows, const void* b_bf16, int ncols, int kp,
                             const float* bias, int32_t* cand_idx, float* cand_val, int* err, cudaStream_t s) {
    return launch_gemm<1>(static_cast<const __nv_bfloat16*>(a_bf16), nrows, static_cast<const __nv_bfloat16*>(b_bf16),
                          ncols, kp, bias, nullptr, cand_idx, cand_val, err, s);
}

}  // namespace hann

// ---------------------------------------------------------------------------
// Diagnostic entry point (include/hann_gb300_diag.h).
#include "hann_gb300.h"
#include "hann_gb300_diag.h"

extern "C" int hann_gpu_bf16_scores(const float* a, int64_t n, const float* b, int32_t m, int32_t dim, float* scores,
                                    int32_t* top_idx, float* top_val) {
    using namespace hann;
    if (n <= 0 || m <= 0 || dim <= 0 || dim > 128 || !a || !b || !top_idx || !top_val) return HANN_E_INVALID;
    const int kp = gemm_kpad(dim);
    float *da = nullptr, *db = nullptr, *dbias = nullptr, *ds = nullptr, *dtv = nullptr;
    void *abf = nullptr, *bbf = nullptr;
    int32_t* dti = nullptr;
    int* derr = nullptr;
    int rc = HANN_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == HANN_OK) rc = HANN_E_CUDA;
        return e == cudaSuccess;
    };
    if (ok(cudaMalloc(&da, sizeof(float) * n * dim)) && ok(cudaMalloc(&db, sizeof(float) * (size_t)m * dim)) &&
        ok(cudaMalloc(&dbias, sizeof(float) * m)) && ok(cudaMalloc(&abf, 2 * (size_t)n * kp)) &&
        ok(cudaMalloc(&bbf, 2 * (size_t)m * kp)) && ok(cudaMalloc(&dti, sizeof(int32_t) * n * 8)) &&
        ok(cudaMalloc(&dtv, sizeof(float) * n * 8)) && ok(cudaMalloc(&derr, sizeof(int))) &&
        (scores == nullptr || ok(cudaMalloc(&ds, sizeof(float) * n * m)))) {
        ok(cudaMemcpy(da, a, sizeof(float) * n * dim, cudaMemcpyHostToDevice));
        ok(cudaMemcpy(db, b, sizeof(float) * (size_t)m * dim, cudaMemcpyHostToDevice));
        ok(cudaMemset(derr, 0, sizeof(int)));
        ok(launch_to_bf16(da, n, dim, kp, abf, nullptr, nullptr, nullptr));
        ok(launch_to_bf16(db, m, dim, kp, bbf, dbias, nullptr, nullptr));
        if (scores) ok(launch_gemm_scores(abf, n, bbf, m, kp, dbias, ds, derr, nullptr));
        ok(launch_gemm_top8(abf, n, bbf, m, kp, dbias, dti, dtv, derr, nullptr));
        ok(cudaDeviceSynchronize());
        int herr = 0;
        ok(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr && rc == HANN_OK) rc = HANN_E_CUDA;
        if (scores) ok(cudaMemcpy(scores, ds, sizeof(float) * n * m, cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(top_idx, dti, sizeof(int32_t) * n * 8, cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(top_val, dtv, sizeof(float) * n * 8, cudaMemcpyDeviceToHost));
    }
    cudaFree(da); cudaFree(db); cudaFree(dbias); cudaFree(abf); cudaFree(bbf); cudaFree(dti); cudaFree(dtv);
    cudaFree(derr); cudaFree(ds);
    return rc;
}
