/*
 * hann_oracle.c -- CPU restatement of the reference PQIVF path, used ONLY as
 * test infrastructure: tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it as the checker. Nothing in the hann_gb300 product
 * path links, loads or calls this file.
 *
 * What it restates (file:line within habedi/hann):
 *   - the FP32 distance kernels of core/simd_kernels.inc.h:64-264 and the
 *     scalar fallbacks of core/simd_distance.c:28-97, with the summation order
 *     of each CPU tier (scalar fallback, AVX, AVX2+FMA, NEON) reproduced lane
 *     by lane in portable C, so the same binary gives the reference's tier-3
 *     (NEON, the Grace host's tier) result on any machine;
 *   - assignPoints (pqivf/index.go:738-789): argmin with the lowest index
 *     winning a tie;
 *   - runKMeans (pqivf/index.go:795-847): FP32 sums in point order, FP32
 *     divide, empty clusters reseeded from a caller-supplied index stream
 *     (the reference draws them from Go's math/rand, which is not
 *     reproducible without Go, so init and reseed indices are inputs);
 *   - encodeWithCodebooks (pqivf/index.go:641-666): residual, split, argmin
 *     per subquantizer with the lowest code winning a tie;
 *   - Search (pqivf/index.go:850-949): probe order by coarse rank distance,
 *     candidate concatenation in probe order, brute-force fallback, the FP32
 *     reconstructed-vector rank distance of decodePQCode + vectorAdd
 *     (pqivf/index.go:678-714, 909-928), sort, truncate, sqrt.
 *
 * Compile with -ffp-contract=off: every fused multiply-add below is an
 * explicit fmaf(), placed exactly where the reference tier fuses.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 8

/* Reference CPU tiers, numbered as core/cpu_check.go:17-27 numbers them. */
enum { TIER_FALLBACK = 0, TIER_AVX = 1, TIER_AVX2 = 2, TIER_NEON = 3 };

static int g_tier = TIER_NEON;

void hann_oracle_set_tier(int tier) { g_tier = tier; }
int hann_oracle_get_tier(void) { return g_tier; }

/* Lane count, unroll factor and FMA fusion of a tier's vector body
 * (core/simd_kernels_{avx,avx2,neon}.inc.h). */
static void tier_shape(int tier, int manhattan, int* lanes, int* unroll, int* fused) {
    switch (tier) {
    case TIER_NEON: *lanes = 4; *unroll = 4; *fused = 1; break;
    case TIER_AVX2:
        /* Manhattan in the AVX2 tier aliases the AVX body
         * (core/simd_distance.c:143-149). */
        *lanes = 8; *unroll = manhattan ? 1 : 4; *fused = 1; break;
    case TIER_AVX: *lanes = 8; *unroll = 1; *fused = 0; break;
    default: *lanes = 1; *unroll = 1; *fused = 0; break;
    }
}

static inline float madd(float x, float y, float acc, int fused) {
    if (fused) return fmaf(x, y, acc);
    float p = x * y;
    return acc + p;
}

/* HANN_REDUCE: horizontal sum of one vector register.
 * NEON vaddvq_f32 adds adjacent pairs, then the pair sums.
 * AVX horizontal_sum256 (core/simd_isa.h:26-35) first folds the high half
 * onto the low half, then adds adjacent pairs, then the pair sums. */
static inline float reduce_lanes(const float* v, int lanes) {
    if (lanes == 4) return (v[0] + v[1]) + (v[2] + v[3]);
    if (lanes == 8) {
        float w0 = v[0] + v[4], w1 = v[1] + v[5], w2 = v[2] + v[6], w3 = v[3] + v[7];
        return (w0 + w1) + (w2 + w3);
    }
    return v[0];
}

/* sum_squared_diff, core/simd_kernels.inc.h:64-102, for the active tier;
 * squared_euclidean_fallback, core/simd_distance.c:37-44, for tier 0. */
float hann_oracle_sqeuclid_tier(const float* a, const float* b, size_t n, int tier) {
    int L, U, F;
    tier_shape(tier, 0, &L, &U, &F);
    if (L == 1) {
        float sum = 0.0f;
        for (size_t i = 0; i < n; i++) {
            float d = a[i] - b[i];
            float p = d * d;
            sum = sum + p;
        }
        return sum;
    }
    float acc[4][MAXL];
    memset(acc, 0, sizeof(acc));
    size_t i = 0;
    if (U == 4) {
        size_t lim4 = n - (n % (size_t)(4 * L));
        for (; i < lim4; i += 4 * L)
            for (int u = 0; u < 4; u++)
                for (int l = 0; l < L; l++) {
                    float d = a[i + u * L + l] - b[i + u * L + l];
                    acc[u][l] = madd(d, d, acc[u][l], F);
                }
    }
    size_t lim = n - (n % (size_t)L);
    for (; i < lim; i += L)
        for (int l = 0; l < L; l++) {
            float d = a[i + l] - b[i + l];
            acc[0][l] = madd(d, d, acc[0][l], F);
        }
    float v[MAXL];
    for (int l = 0; l < L; l++)
        v[l] = (U == 4) ? ((acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l])) : acc[0][l];
    float sum = reduce_lanes(v, L);
    /* The scalar tail is a separate multiply and add in every tier: the
     * reference build does not contract `sum += diff * diff` (checked
     * against the compiled reference kernels for tiers 0-2). */
    for (; i < n; i++) {
        float d = a[i] - b[i];
        float p = d * d;
        sum = sum + p;
    }
    return sum;
}

/* manhattan, core/simd_kernels.inc.h:115-149 and core/simd_distance.c:46-52. */
float hann_oracle_manhattan_tier(const float* a, const float* b, size_t n, int tier) {
    int L, U, F;
    tier_shape(tier, 1, &L, &U, &F);
    if (L == 1) {
        float sum = 0.0f;
        for (size_t i = 0; i < n; i++) sum += fabsf(a[i] - b[i]);
        return sum;
    }
    float acc[4][MAXL];
    memset(acc, 0, sizeof(acc));
    size_t i = 0;
    if (U == 4) {
        size_t lim4 = n - (n % (size_t)(4 * L));
        for (; i < lim4; i += 4 * L)
            for (int u = 0; u < 4; u++)
                for (int l = 0; l < L; l++)
                    acc[u][l] = acc[u][l] + fabsf(a[i + u * L + l] - b[i + u * L + l]);
    }
    size_t lim = n - (n % (size_t)L);
    for (; i < lim; i += L)
        for (int l = 0; l < L; l++) acc[0][l] = acc[0][l] + fabsf(a[i + l] - b[i + l]);
    float v[MAXL];
    for (int l = 0; l < L; l++)
        v[l] = (U == 4) ? ((acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l])) : acc[0][l];
    float sum = reduce_lanes(v, L);
    for (; i < n; i++) sum += fabsf(a[i] - b[i]);
    return sum;
}

/* Cosine pieces: dot, |a|^2, |b|^2, accumulated in the tier's order.
 * The three accumulations are independent, so each can also be computed on
 * its own (a norm is the dot of a vector with itself) with identical bits. */
static void cosine_parts(const float* a, const float* b, size_t n, int tier,
                         float* dot_o, float* na_o, float* nb_o) {
    int L, U, F;
    tier_shape(tier, 0, &L, &U, &F);
    if (L == 1) {
        float dot = 0, na = 0, nb = 0;
        for (size_t i = 0; i < n; i++) {
            float p1 = a[i] * b[i], p2 = a[i] * a[i], p3 = b[i] * b[i];
            dot = dot + p1; na = na + p2; nb = nb + p3;
        }
        *dot_o = dot; *na_o = na; *nb_o = nb;
        return;
    }
    float dt[4][MAXL], xa[4][MAXL], xb[4][MAXL];
    memset(dt, 0, sizeof(dt)); memset(xa, 0, sizeof(xa)); memset(xb, 0, sizeof(xb));
    size_t i = 0;
    if (U == 4) {
        size_t lim4 = n - (n % (size_t)(4 * L));
        for (; i < lim4; i += 4 * L)
            for (int u = 0; u < 4; u++)
                for (int l = 0; l < L; l++) {
                    float va = a[i + u * L + l], vb = b[i + u * L + l];
                    dt[u][l] = madd(va, vb, dt[u][l], F);
                    xa[u][l] = madd(va, va, xa[u][l], F);
                    xb[u][l] = madd(vb, vb, xb[u][l], F);
                }
    }
    size_t lim = n - (n % (size_t)L);
    for (; i < lim; i += L)
        for (int l = 0; l < L; l++) {
            float va = a[i + l], vb = b[i + l];
            dt[0][l] = madd(va, vb, dt[0][l], F);
            xa[0][l] = madd(va, va, xa[0][l], F);
            xb[0][l] = madd(vb, vb, xb[0][l], F);
        }
    float v1[MAXL], v2[MAXL], v3[MAXL];
    for (int l = 0; l < L; l++) {
        if (U == 4) {
            v1[l] = (dt[0][l] + dt[1][l]) + (dt[2][l] + dt[3][l]);
            v2[l] = (xa[0][l] + xa[1][l]) + (xa[2][l] + xa[3][l]);
            v3[l] = (xb[0][l] + xb[1][l]) + (xb[2][l] + xb[3][l]);
        } else {
            v1[l] = dt[0][l]; v2[l] = xa[0][l]; v3[l] = xb[0][l];
        }
    }
    float dot = reduce_lanes(v1, L), na = reduce_lanes(v2, L), nb = reduce_lanes(v3, L);
    /* The cosine tail is contracted to fused multiply-adds in the tiers that
     * have FMA (checked against the compiled reference kernels). */
    for (; i < n; i++) {
        dot = madd(a[i], b[i], dot, F);
        na = madd(a[i], a[i], na, F);
        nb = madd(b[i], b[i], nb, F);
    }
    *dot_o = dot; *na_o = na; *nb_o = nb;
}

/* cosine_distance, core/simd_kernels.inc.h:153-229: a zero norm gives 1,
 * the similarity is clamped to [-1, 1]. */
float hann_oracle_cosine_tier(const float* a, const float* b, size_t n, int tier) {
    float dot, na, nb;
    cosine_parts(a, b, n, tier, &dot, &na, &nb);
    float A = sqrtf(na), B = sqrtf(nb);
    if (A == 0.0f || B == 0.0f) return 1.0f;
    float s = dot / (A * B);
    if (s > 1.0f) s = 1.0f;
    if (s < -1.0f) s = -1.0f;
    return 1.0f - s;
}

void hann_oracle_cosine_parts(const float* a, const float* b, size_t n, int tier, float* out3) {
    cosine_parts(a, b, n, tier, &out3[0], &out3[1], &out3[2]);
}

/* The NEON tier of sum_squared_diff (4 lanes, 4 accumulators, fused
 * multiply-add; core/simd_kernels.inc.h:64-102 with simd_kernels_neon.inc.h)
 * written with one small array per accumulator so that the compiler can keep
 * each in a vector register: the same operations in the same order as the
 * generic path of hann_oracle_sqeuclid_tier, only faster, for the timed CPU
 * baseline and the large parity checks. */
static float sqeuclid_neon(const float* a, const float* b, size_t n) {
    float c0[4] = {0, 0, 0, 0}, c1[4] = {0, 0, 0, 0}, c2[4] = {0, 0, 0, 0}, c3[4] = {0, 0, 0, 0};
    size_t i = 0;
    const size_t lim4 = n - (n % 16);
    for (; i < lim4; i += 16) {
        for (int l = 0; l < 4; l++) {
            const float d0 = a[i + l] - b[i + l], d1 = a[i + 4 + l] - b[i + 4 + l];
            const float d2 = a[i + 8 + l] - b[i + 8 + l], d3 = a[i + 12 + l] - b[i + 12 + l];
            c0[l] = fmaf(d0, d0, c0[l]);
            c1[l] = fmaf(d1, d1, c1[l]);
            c2[l] = fmaf(d2, d2, c2[l]);
            c3[l] = fmaf(d3, d3, c3[l]);
        }
    }
    const size_t lim = n - (n % 4);
    for (; i < lim; i += 4)
        for (int l = 0; l < 4; l++) {
            const float d = a[i + l] - b[i + l];
            c0[l] = fmaf(d, d, c0[l]);
        }
    float v[4];
    for (int l = 0; l < 4; l++) v[l] = (c0[l] + c1[l]) + (c2[l] + c3[l]);
    float sum = (v[0] + v[1]) + (v[2] + v[3]);
    for (; i < n; i++) {
        const float d = a[i] - b[i];
        const float p = d * d;
        sum = sum + p;
    }
    return sum;
}

static inline float sqeuclid(const float* a, const float* b, size_t n) {
    if (g_tier == TIER_NEON) return sqeuclid_neon(a, b, n);
    return hann_oracle_sqeuclid_tier(a, b, n, g_tier);
}

/* The four batch kernels (core/simd_kernels.inc.h:235-264): one query
 * against n rows of a flat buffer, each result widened to double.
 * metric: 0 squared Euclidean, 1 Euclidean, 2 Manhattan, 3 cosine. */
void hann_oracle_batch(int metric, const float* q, const float* flat, size_t dim, size_t n, double* out) {
    for (size_t i = 0; i < n; i++) {
        const float* x = flat + i * dim;
        float r;
        switch (metric) {
        case 0: r = sqeuclid(q, x, dim); break;
        case 1: r = sqrtf(sqeuclid(q, x, dim)); break;
        case 2: r = hann_oracle_manhattan_tier(q, x, dim, g_tier); break;
        default: r = hann_oracle_cosine_tier(q, x, dim, g_tier); break;
        }
        out[i] = (double)r;
    }
}

/* ---------------------------------------------------------------------- */
/* Thread pool helper: run fn(ctx, begin, end) over [0, n) in contiguous
 * chunks, like the reference's goroutine fan-out (pqivf/index.go:747-762). */
typedef void (*range_fn)(void* ctx, int64_t begin, int64_t end);
struct range_job { range_fn fn; void* ctx; int64_t b, e; };
static void* range_thread(void* p) {
    struct range_job* j = (struct range_job*)p;
    j->fn(j->ctx, j->b, j->e);
    return NULL;
}
static void parallel_for(int64_t n, int nthreads, range_fn fn, void* ctx) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = (int)(n > 0 ? n : 1);
    if (nthreads == 1) { fn(ctx, 0, n); return; }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    struct range_job* jobs = (struct range_job*)malloc(sizeof(struct range_job) * nthreads);
    int64_t chunk = (n + nthreads - 1) / nthreads;
    int started = 0;
    for (int w = 0; w < nthreads; w++) {
        int64_t b = w * chunk, e = b + chunk;
        if (b >= n) break;
        if (e > n) e = n;
        jobs[w].fn = fn; jobs[w].ctx = ctx; jobs[w].b = b; jobs[w].e = e;
        pthread_create(&th[w], NULL, range_thread, &jobs[w]);
        started++;
    }
    for (int w = 0; w < started; w++) pthread_join(th[w], NULL);
    free(th); free(jobs);
}

/* ---------------------------------------------------------------------- */
/* assignPoints, pqivf/index.go:738-789. */
struct assign_ctx { const float* data; const float* cent; int dim; int k; int32_t* out; };
static void assign_range(void* p, int64_t b, int64_t e) {
    struct assign_ctx* c = (struct assign_ctx*)p;
    for (int64_t i = b; i < e; i++) {
        const float* x = c->data + (size_t)i * c->dim;
        double best_d = (double)sqeuclid(x, c->cent, c->dim);
        int best = 0;
        for (int j = 1; j < c->k; j++) {
            double d = (double)sqeuclid(x, c->cent + (size_t)j * c->dim, c->dim);
            if (d < best_d) { best_d = d; best = j; }
        }
        c->out[i] = best;
    }
}
void hann_oracle_assign(const float* data, int64_t n, int dim, const float* cent, int k,
                        int32_t* out, int nthreads) {
    struct assign_ctx c = {data, cent, dim, k, out};
    parallel_for(n, nthreads, assign_range, &c);
}

/* runKMeans, pqivf/index.go:795-847. Returns the effective k (k clamps to n),
 * or -1 when the reseed stream runs out. centroids_out holds k_eff rows.
 * init_idx: k_eff row indices (the reference's perm[:k]).
 * reseed_idx: the stream of rows used, in order, for empty clusters (the
 * reference's successive Intn(n) draws). *reseeds_used reports how many. */
int hann_oracle_kmeans(const float* data, int64_t n, int dim, int k, int iters,
                       const int64_t* init_idx, const int64_t* reseed_idx, int64_t n_reseed,
                       float* centroids_out, int64_t* reseeds_used, int nthreads) {
    if (n <= 0) return -2;
    if (n < k) k = (int)n;
    float* cent = centroids_out;
    for (int i = 0; i < k; i++)
        memcpy(cent + (size_t)i * dim, data + (size_t)init_idx[i] * dim, sizeof(float) * dim);
    int32_t* assign = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    float* sums = (float*)malloc(sizeof(float) * (size_t)k * dim);
    int64_t* counts = (int64_t*)malloc(sizeof(int64_t) * (size_t)k);
    int64_t used = 0;
    int rc = k;
    for (int it = 0; it < iters; it++) {
        hann_oracle_assign(data, n, dim, cent, k, assign, nthreads);
        memset(sums, 0, sizeof(float) * (size_t)k * dim);
        memset(counts, 0, sizeof(int64_t) * (size_t)k);
        for (int64_t p = 0; p < n; p++) {
            int c = assign[p];
            counts[c]++;
            float* s = sums + (size_t)c * dim;
            const float* x = data + (size_t)p * dim;
            for (int j = 0; j < dim; j++) s[j] += x[j];
        }
        for (int i = 0; i < k; i++) {
            if (counts[i] == 0) {
                if (used >= n_reseed) { rc = -1; goto out; }
                memcpy(cent + (size_t)i * dim, data + (size_t)reseed_idx[used] * dim, sizeof(float) * dim);
                used++;
            } else {
                float cnt = (float)counts[i];
                for (int j = 0; j < dim; j++) cent[(size_t)i * dim + j] = sums[(size_t)i * dim + j] / cnt;
            }
        }
    }
out:
    if (reseeds_used) *reseeds_used = used;
    free(assign); free(sums); free(counts);
    return rc;
}

/* encodeWithCodebooks, pqivf/index.go:641-666. codebooks: [M][pqK][dsub]. */
struct enc_ctx {
    const float* x; const int32_t* cluster; const float* coarse; int dim; int M; int pqK;
    const float* cb; int32_t* codes;
};
static void encode_range(void* p, int64_t b, int64_t e) {
    struct enc_ctx* c = (struct enc_ctx*)p;
    int dsub = c->dim / c->M;
    float* res = (float*)malloc(sizeof(float) * c->dim);
    for (int64_t i = b; i < e; i++) {
        const float* v = c->x + (size_t)i * c->dim;
        const float* ce = c->coarse + (size_t)c->cluster[i] * c->dim;
        for (int j = 0; j < c->dim; j++) res[j] = v[j] - ce[j];
        for (int m = 0; m < c->M; m++) {
            const float* sub = res + m * dsub;
            const float* cbm = c->cb + (size_t)m * c->pqK * dsub;
            double best_d = (double)sqeuclid(sub, cbm, dsub);
            int best = 0;
            for (int j = 1; j < c->pqK; j++) {
                double d = (double)sqeuclid(sub, cbm + (size_t)j * dsub, dsub);
                if (d < best_d) { best_d = d; best = j; }
            }
            c->codes[(size_t)i * c->M + m] = best;
        }
    }
    free(res);
}
void hann_oracle_encode(const float* x, int64_t n, int dim, const int32_t* cluster, const float* coarse,
                        int M, int pqK, const float* codebooks, int32_t* codes_out, int nthreads) {
    struct enc_ctx c = {x, cluster, coarse, dim, M, pqK, codebooks, codes_out};
    parallel_for(n, nthreads, encode_range, &c);
}

/* ---------------------------------------------------------------------- */
/* Search, pqivf/index.go:850-949, over an index held in CSR form:
 *   list_off[nlist+1]  row range of each coarse cluster's inverted list
 *   ids[N], vectors[N][dim], codes[N][M], has_codes[N], entry_cluster[N]
 * Results: ids_out[k], dist_out[k] (true Euclidean, sqrt of the FP32 rank
 * widened to double), *n_out, *fallback_out. */
typedef struct {
    int dim, M, pqK, nlist;
    const float* coarse;      /* [nlist][dim] */
    const float* codebooks;   /* [M][pqK][dsub] */
    const int64_t* list_off;  /* [nlist+1] */
    const int64_t* ids;
    const float* vectors;
    const int32_t* codes;
    const uint8_t* has_codes;
    const int32_t* entry_cluster;
} oracle_index;

struct cand { double d; int64_t pos; int64_t seq; };
static int cmp_cand(const void* x, const void* y) {
    const struct cand* a = (const struct cand*)x;
    const struct cand* b = (const struct cand*)y;
    if (a->d < b->d) return -1;
    if (a->d > b->d) return 1;
    return (a->seq < b->seq) ? -1 : (a->seq > b->seq);
}
struct probe { double d; int c; };
static int cmp_probe(const void* x, const void* y) {
    const struct probe* a = (const struct probe*)x;
    const struct probe* b = (const struct probe*)y;
    if (a->d < b->d) return -1;
    if (a->d > b->d) return 1;
    return (a->c < b->c) ? -1 : (a->c > b->c);
}

static double entry_rank(const oracle_index* ix, const float* q, int64_t pos, float* recon) {
    int dim = ix->dim, M = ix->M, dsub = dim / M;
    if (ix->has_codes[pos]) {
        const int32_t* code = ix->codes + (size_t)pos * M;
        int ok = 1;
        for (int m = 0; m < M; m++) if (code[m] < 0 || code[m] >= ix->pqK) ok = 0;
        if (ok) {
            const float* ce = ix->coarse + (size_t)ix->entry_cluster[pos] * dim;
            for (int m = 0; m < M; m++) {
                const float* cw = ix->codebooks + ((size_t)m * ix->pqK + code[m]) * dsub;
                for (int j = 0; j < dsub; j++) recon[m * dsub + j] = ce[m * dsub + j] + cw[j];
            }
            return (double)sqeuclid(q, recon, dim);
        }
    }
    return (double)sqeuclid(q, ix->vectors + (size_t)pos * dim, dim);
}

/* Returns the result count, or -1 on an allocation failure. With rerank > 0
 * the candidates are cut to the `rerank` best by the reference's PQ distance
 * and reordered by the exact FP32 distance to their stored vectors (the
 * GPU's exact-rerank mode, restated on the CPU; the reference has no such
 * mode). */
static int search_one(const oracle_index* ix, const float* q, int k, int nprobe, int fallback, int rerank,
                      int64_t* ids_out, double* dist_out, int* used_fallback,
                      int32_t* probe_out /* nullable, [nprobe] */) {
    int dim = ix->dim, nlist = ix->nlist;
    struct probe* pr = (struct probe*)malloc(sizeof(struct probe) * (nlist > 0 ? nlist : 1));
    for (int c = 0; c < nlist; c++) {
        pr[c].d = (double)sqeuclid(q, ix->coarse + (size_t)c * dim, dim);
        pr[c].c = c;
    }
    qsort(pr, nlist, sizeof(struct probe), cmp_probe);
    int np = nprobe < nlist ? nprobe : nlist;
    if (probe_out) for (int i = 0; i < np; i++) probe_out[i] = pr[i].c;
    int64_t total = 0;
    for (int i = 0; i < np; i++) total += ix->list_off[pr[i].c + 1] - ix->list_off[pr[i].c];
    int fb = 0;
    if (total < k && fallback) { fb = 1; total = ix->list_off[nlist]; }
    struct cand* cs = (struct cand*)malloc(sizeof(struct cand) * (total > 0 ? total : 1));
    float* recon = (float*)malloc(sizeof(float) * dim);
    int64_t nc = 0;
    if (!fb) {
        for (int i = 0; i < np; i++) {
            int c = pr[i].c;
            for (int64_t p = ix->list_off[c]; p < ix->list_off[c + 1]; p++, nc++) {
                cs[nc].d = entry_rank(ix, q, p, recon); cs[nc].pos = p; cs[nc].seq = nc;
            }
        }
    } else {
        /* The reference walks its list map in Go map order, which is random;
         * this restatement walks the lists in ascending cluster order. */
        for (int64_t p = 0; p < total; p++, nc++) {
            cs[nc].d = entry_rank(ix, q, p, recon); cs[nc].pos = p; cs[nc].seq = nc;
        }
    }
    qsort(cs, nc, sizeof(struct cand), cmp_cand);
    if (rerank > 0) {
        if (nc > rerank) nc = rerank;
        for (int64_t i = 0; i < nc; i++) cs[i].d = (double)sqeuclid(q, ix->vectors + (size_t)cs[i].pos * dim, dim);
        qsort(cs, nc, sizeof(struct cand), cmp_cand);
    }
    int kk = k < nc ? k : (int)nc;
    for (int i = 0; i < kk; i++) {
        ids_out[i] = ix->ids[cs[i].pos];
        dist_out[i] = sqrt(cs[i].d);
    }
    if (used_fallback) *used_fallback = fb;
    free(pr); free(cs); free(recon);
    return kk;
}

struct search_ctx {
    const oracle_index* ix; const float* q; const int32_t* k; const int32_t* nprobe; int fallback; int rerank;
    int kmax; int64_t* ids; double* dist; int32_t* nout; int32_t* fb;
};
static void search_range(void* p, int64_t b, int64_t e) {
    struct search_ctx* c = (struct search_ctx*)p;
    for (int64_t i = b; i < e; i++) {
        int ufb = 0;
        c->nout[i] = search_one(c->ix, c->q + (size_t)i * c->ix->dim, c->k[i], c->nprobe[i], c->fallback,
                                c->rerank, c->ids + (size_t)i * c->kmax, c->dist + (size_t)i * c->kmax, &ufb,
                                NULL);
        if (c->fb) c->fb[i] = ufb;
    }
}

void hann_oracle_search_batch_rerank(int dim, int M, int pqK, int nlist, const float* coarse, const float* codebooks,
                                     const int64_t* list_off, const int64_t* ids, const float* vectors,
                                     const int32_t* codes, const uint8_t* has_codes, const int32_t* entry_cluster,
                                     const float* queries, int64_t nq, const int32_t* k, const int32_t* nprobe,
                                     int fallback, int rerank, int kmax, int64_t* ids_out, double* dist_out,
                                     int32_t* n_out, int32_t* fallback_out, int nthreads);

/* Batch of independent Search calls, fanned out over nthreads like the
 * reference's query pool (example/run_datasets.go:84-120). Output rows have
 * stride kmax. */
void hann_oracle_search_batch(int dim, int M, int pqK, int nlist, const float* coarse, const float* codebooks,
                              const int64_t* list_off, const int64_t* ids, const float* vectors,
                              const int32_t* codes, const uint8_t* has_codes, const int32_t* entry_cluster,
                              const float* queries, int64_t nq, const int32_t* k, const int32_t* nprobe,
                              int fallback, int kmax, int64_t* ids_out, double* dist_out, int32_t* n_out,
                              int32_t* fallback_out, int nthreads) {
    hann_oracle_search_batch_rerank(dim, M, pqK, nlist, coarse, codebooks, list_off, ids, vectors, codes, has_codes,
                                    entry_cluster, queries, nq, k, nprobe, fallback, 0, kmax, ids_out, dist_out,
                                    n_out, fallback_out, nthreads);
}

/* The same with the exact rerank of search_one (rerank 0 = the reference's
 * Search). */
void hann_oracle_search_batch_rerank(int dim, int M, int pqK, int nlist, const float* coarse, const float* codebooks,
                                     const int64_t* list_off, const int64_t* ids, const float* vectors,
                                     const int32_t* codes, const uint8_t* has_codes, const int32_t* entry_cluster,
                                     const float* queries, int64_t nq, const int32_t* k, const int32_t* nprobe,
                                     int fallback, int rerank, int kmax, int64_t* ids_out, double* dist_out,
                                     int32_t* n_out, int32_t* fallback_out, int nthreads) {
    oracle_index ix = {dim, M, pqK, nlist, coarse, codebooks, list_off, ids, vectors, codes, has_codes,
                       entry_cluster};
    struct search_ctx c = {&ix, queries, k, nprobe, fallback, rerank, kmax, ids_out, dist_out, n_out, fallback_out};
    parallel_for(nq, nthreads, search_range, &c);
}

/* The probe order of one query (nearestCentroids, pqivf/index.go:184-206),
 * ties broken by the lower cluster index. */
void hann_oracle_probe(int dim, int nlist, const float* coarse, const float* q, int nprobe, int32_t* out) {
    struct probe* pr = (struct probe*)malloc(sizeof(struct probe) * (nlist > 0 ? nlist : 1));
    for (int c = 0; c < nlist; c++) {
        pr[c].d = (double)sqeuclid(q, coarse + (size_t)c * dim, dim);
        pr[c].c = c;
    }
    qsort(pr, nlist, sizeof(struct probe), cmp_probe);
    int np = nprobe < nlist ? nprobe : nlist;
    for (int i = 0; i < np; i++) out[i] = pr[i].c;
    free(pr);
}

/* ---------------------------------------------------------------------- */
/* testutil.BruteForceKNN (internal/testutil/data.go:66-93) for a batch of
 * queries over a flat base whose row numbers are the ids: every distance as
 * the tier's batch kernel returns it (FP32 widened to double; an empty
 * vector has distance 0, core/distance.go:23-25), sorted by (distance, id),
 * the first k kept; slots past n get id -1 and distance +inf. */
struct knn_item { double d; int64_t id; };
static int cmp_knn(const void* x, const void* y) {
    const struct knn_item* a = (const struct knn_item*)x;
    const struct knn_item* b = (const struct knn_item*)y;
    if (a->d < b->d) return -1;
    if (a->d > b->d) return 1;
    return (a->id > b->id) - (a->id < b->id);
}
struct knn_ctx { int metric; const float* q; const float* base; int64_t n; int dim; int k; int64_t* ids; double* dist; };
static void knn_range(void* p, int64_t b, int64_t e) {
    struct knn_ctx* c = (struct knn_ctx*)p;
    struct knn_item* it = (struct knn_item*)malloc(sizeof(struct knn_item) * (size_t)(c->n > 0 ? c->n : 1));
    double* dd = (double*)malloc(sizeof(double) * (size_t)(c->n > 0 ? c->n : 1));
    for (int64_t qi = b; qi < e; qi++) {
        if (c->dim > 0) hann_oracle_batch(c->metric, c->q + (size_t)qi * c->dim, c->base, (size_t)c->dim, (size_t)c->n, dd);
        for (int64_t i = 0; i < c->n; i++) {
            it[i].d = c->dim > 0 ? dd[i] : 0.0;
            it[i].id = i;
        }
        qsort(it, (size_t)c->n, sizeof(struct knn_item), cmp_knn);
        for (int j = 0; j < c->k; j++) {
            c->ids[qi * c->k + j] = j < c->n ? it[j].id : -1;
            c->dist[qi * c->k + j] = j < c->n ? it[j].d : INFINITY;
        }
    }
    free(it);
    free(dd);
}
void hann_oracle_knn(int metric, const float* q, int64_t nq, const float* base, int64_t n, int dim, int k,
                     int64_t* ids, double* dist, int nthreads) {
    struct knn_ctx c = {metric, q, base, n, dim, k, ids, dist};
    parallel_for(nq, nthreads, knn_range, &c);
}
