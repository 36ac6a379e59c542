// index.cu -- the PQIVF index behind the C ABI (include/hann_gb300.h).
//
// Host-side state mirrors the reference's pqivf.Index (pqivf/index.go:36-54):
// pending vectors before Train, the id -> cluster map, per-list id order, the
// ClusterCounts map and the list-map key set. Everything the kernels read
// lives in HBM in structure-of-arrays form, one row per stored vector:
//   codes  [rows][code_stride] uint8   PQ codes (M bytes, padded to 4)
//   term   [rows] f32                  ||r||^2 + 2<c, r> of the decoded residual
//   vectors[rows][dim] f32             raw vectors (exact rerank, re-Train)
//   row_id [rows] i64, row_cluster [rows] i32
// Rows of one inverted list are contiguous; every list starts on a multiple
// of 32 rows and keeps spare capacity so Adds append in place.
#include <cuda_fp16.h>
#include <chrono>

#include "index_internal.h"
#include "hann_gb300_diag.h"

std::string& hann_thread_error() {
    static thread_local std::string e;
    return e;
}


// Capacity for a list that must hold `len` rows.
// Slots for a list of len rows: a quarter more, plus 32.
static int64_t list_capacity(int64_t len) { return round_up(len + len / 4 + 32, 32); }

// ---------------------------------------------------------------------------
// Device layout management.

// Lays the lists out afresh with capacities caps[], moving the live rows.
// With move_rows false it only allocates (the caller fills the rows).
// Deleted (tombstoned) slots are dropped while the live rows move, so a
// relayout also compacts the lists. The rows move on the device, list by
// list; the host only renumbers the lists that held tombstones. The previous
// arrays are kept as the next relayout's destination, so a relayout of an
// index that does not grow allocates nothing.
// Free rows kept at the end of the arena after a full relayout, for lists
// that outgrow their capacity to move into (an eighth of the rows, at least
// 4,096).
static int64_t arena_slack(int64_t packed) { return round_up(std::max<int64_t>(packed / 8, 4096), 32); }

static int relayout(hann_pqivf* h, const std::vector<int64_t>& caps, bool move_rows = true) {
    const int dim = h->o.dimension;
    std::vector<int64_t> start(h->nlist);
    int64_t packed = 0;
    for (int l = 0; l < h->nlist; l++) {
        start[l] = packed;
        packed += round_up(caps[l], 32);
    }
    const int64_t total = packed + arena_slack(packed);
    if (total >= (int64_t)1 << 31) return h->fail(HANN_E_UNSUPPORTED, "more than 2^31 stored rows");
    CK(h->s_vectors.reserve((size_t)total * dim));
    CK(h->s_term.reserve((size_t)total));
    CK(h->s_row_id.reserve((size_t)total));
    CK(h->s_row_cluster.reserve((size_t)total));
    CK(h->s_codes.reserve((size_t)total * h->code_stride));
    // scan codes: each list's region rounded up to whole groups of rows
    const bool sw = scan_adc_supported(h->o.num_subquantizers);
    std::vector<int64_t> swstart(h->nlist);
    int64_t swtotal = 0, swcap = 0;
    if (sw) {
        const int G = scan_group_rows(h->o.num_subquantizers);
        for (int l = 0; l < h->nlist; l++) {
            swstart[l] = swtotal;
            swtotal += round_up(round_up(caps[l], 32), G);
        }
        swcap = swtotal + round_up(arena_slack(packed), G);
        CK(h->s_scanc.reserve((size_t)swcap * scan_codes_per_row(h->o.num_subquantizers)));
    }
    if (move_rows && h->rows_cap > 0) {
        std::vector<int64_t> src(h->nlist);
        std::vector<int32_t> len(h->nlist), cmp(h->nlist);
        for (int l = 0; l < h->nlist; l++) {
            src[l] = h->h_start[l];
            len[l] = (int32_t)h->list_ids[l].size();
            cmp[l] = h->live_count[l] != (int64_t)h->list_ids[l].size();
            if (!cmp[l]) continue;
            int64_t w = 0;
            for (size_t j = 0; j < h->list_ids[l].size(); j++) {
                if (!h->list_alive[l][j]) continue;
                h->list_ids[l][w++] = h->list_ids[l][j];
            }
            h->list_ids[l].resize(w);
            h->list_alive[l].assign(w, 1);
        }
        h->dead_rows = 0;
        DBuf<int64_t> dsrc, ddst;
        DBuf<int32_t> dlen, dcmp;
        CK(upload(dsrc, src.data(), src.size(), h->stream));
        CK(upload(ddst, start.data(), start.size(), h->stream));
        CK(upload(dlen, len.data(), len.size(), h->stream));
        CK(upload(dcmp, cmp.data(), cmp.size(), h->stream));
        CK(launch_relayout_lists(h->nlist, dsrc.p, dlen.p, ddst.p, dcmp.p, dim, h->code_stride / 4, h->d_vectors.p,
                                 h->s_vectors.p, h->d_codes.p, h->s_codes.p, h->d_term.p, h->s_term.p,
                                 h->d_row_id.p, h->s_row_id.p, h->d_row_cluster.p, h->s_row_cluster.p, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    h->d_vectors.swap(h->s_vectors);
    h->d_term.swap(h->s_term);
    h->d_row_id.swap(h->s_row_id);
    h->d_row_cluster.swap(h->s_row_cluster);
    h->d_codes.swap(h->s_codes);
    if (sw) h->d_scanc.swap(h->s_scanc);
    h->scanc_dirty = true;  // rebuilt by upload_lens, which every caller runs next
    h->h_start = start;
    h->h_cap.assign(h->nlist, 0);
    for (int l = 0; l < h->nlist; l++) h->h_cap[l] = round_up(caps[l], 32);
    h->rows_cap = total;
    h->arena_end = packed;
    h->hole_rows = 0;
    h->sw_end = swtotal;
    h->sw_cap = swcap;
    h->full_relayouts++;
    CK(upload(h->d_start, h->h_start.data(), h->h_start.size(), h->stream));
    if (sw) {
        h->h_swstart = swstart;
        CK(upload(h->d_swstart, h->h_swstart.data(), h->h_swstart.size(), h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

// Moves the given lists (all slots, tombstones too, in place order) to the
// arena's free tail with the given capacities, leaving their old slots as
// holes, and rebuilds their scan codes there. Sets *done; does nothing when
// the tail is too small or the holes would pass a quarter of the arena (the
// caller then relayouts everything). The moved rows keep their positions in
// their lists, so the host bookkeeping only changes the lists' starts.
static int grow_lists(hann_pqivf* h, const std::vector<int>& lists, const std::vector<int64_t>& caps, bool* done) {
    *done = false;
    const int n = (int)lists.size();
    if (n == 0 || h->rows_cap == 0) return HANN_OK;
    const bool sw = scan_adc_supported(h->o.num_subquantizers);
    const int G = scan_group_rows(h->o.num_subquantizers);
    int64_t need = 0, need_sw = 0, freed = 0;
    for (int i = 0; i < n; i++) {
        need += round_up(caps[i], 32);
        need_sw += round_up(round_up(caps[i], 32), G);
        freed += h->h_cap[lists[i]];
    }
    if (h->arena_end + need > h->rows_cap || (sw && h->sw_end + need_sw > h->sw_cap)) return HANN_OK;
    if ((h->hole_rows + freed) * 4 > h->rows_cap) return HANN_OK;
    std::vector<int64_t> src(n), dst(n), swd(n);
    std::vector<int32_t> len(n), cmp(n, 0);
    int64_t at = h->arena_end, swat = h->sw_end;
    for (int i = 0; i < n; i++) {
        const int l = lists[i];
        src[i] = h->h_start[l];
        len[i] = (int32_t)h->list_ids[l].size();
        dst[i] = at;
        swd[i] = swat;
        at += round_up(caps[i], 32);
        swat += round_up(round_up(caps[i], 32), G);
    }
    MutationScratch& m = h->mut;
    CK(upload(m.mv_src, src.data(), src.size(), h->stream));
    CK(upload(m.mv_dst, dst.data(), dst.size(), h->stream));
    CK(upload(m.mv_sw, swd.data(), swd.size(), h->stream));
    CK(upload(m.mv_len, len.data(), len.size(), h->stream));
    CK(upload(m.mv_cmp, cmp.data(), cmp.size(), h->stream));
    // source and destination slots are disjoint parts of the same arrays
    CK(launch_relayout_lists(n, m.mv_src.p, m.mv_len.p, m.mv_dst.p, m.mv_cmp.p, h->o.dimension, h->code_stride / 4,
                             h->d_vectors.p, h->d_vectors.p, h->d_codes.p, h->d_codes.p, h->d_term.p, h->d_term.p,
                             h->d_row_id.p, h->d_row_id.p, h->d_row_cluster.p, h->d_row_cluster.p, h->stream));
    if (sw)
        CK(launch_scan_codes_lists(h->d_codes.p, h->code_stride, h->o.num_subquantizers, m.mv_dst.p, m.mv_len.p,
                                   m.mv_sw.p, n, h->d_scanc.p, h->stream));
    for (int i = 0; i < n; i++) {
        const int l = lists[i];
        h->h_start[l] = dst[i];
        h->h_cap[l] = round_up(caps[i], 32);
        if (sw) h->h_swstart[l] = swd[i];
    }
    h->arena_end = at;
    h->sw_end = swat;
    h->hole_rows += freed;
    h->list_moves += n;
    CK(upload(h->d_start, h->h_start.data(), h->h_start.size(), h->stream));
    if (sw) CK(upload(h->d_swstart, h->h_swstart.data(), h->h_swstart.size(), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *done = true;
    return HANN_OK;
}

static int upload_lens(hann_pqivf* h) {
    std::vector<int32_t> len(h->nlist), live(h->nlist);
    int64_t mx = 0;
    for (int l = 0; l < h->nlist; l++) {
        len[l] = (int32_t)h->list_ids[l].size();
        live[l] = (int32_t)h->live_count[l];
        mx = std::max<int64_t>(mx, len[l]);
    }
    h->max_list_slots = mx;
    CK(upload(h->d_len, len.data(), len.size(), h->stream));
    CK(upload(h->d_live, live.data(), live.size(), h->stream));
    if (h->scanc_dirty && h->rows_cap > 0) {
        CK(launch_scan_codes_lists(h->d_codes.p, h->code_stride, h->o.num_subquantizers, h->d_start.p, h->d_len.p,
                                   h->d_swstart.p, h->nlist, h->d_scanc.p, h->stream));
        h->scanc_dirty = false;
    }
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

// FP16 codebooks for the list-major scan and the constants of its error
// bound: over every residual r the codebooks can reconstruct, max ||r|| and
// max ||r - r~|| (r~ the FP16 rounding) are at most the square roots of the
// sums over subquantizers of the largest codeword norm and rounding error;
// |term| = | ||r||^2 + 2 <c, r> | <= rmax^2 + 2 max||c|| rmax.
static int prepare_lms(hann_pqivf* h) {
    const int M = h->o.num_subquantizers, dim = h->o.dimension;
    h->lms_ok = !h->o.plain_fp32 && h->nlist > 0 && h->pqk_eff > 0 && lms_supported(dim, M, h->pqk_eff);
    if (!h->lms_ok) return HANN_OK;
    const size_t ncb = (size_t)M * h->pqk_eff * h->dsub;
    std::vector<uint16_t> cb16(ncb);
    double r2 = 0.0, d2 = 0.0;
    for (int m = 0; m < M; m++) {
        double mx = 0.0, md = 0.0;
        for (int j = 0; j < h->pqk_eff; j++) {
            double n2 = 0.0, e2 = 0.0;
            for (int e = 0; e < h->dsub; e++) {
                const size_t i = ((size_t)m * h->pqk_eff + j) * h->dsub + e;
                const float v = h->h_codebooks[i];
                const __half hv = __float2half_rn(v);
                cb16[i] = __half_as_ushort(hv);
                const double d = (double)v - (double)__half2float(hv);
                n2 += (double)v * v;
                e2 += d * d;
            }
            mx = std::max(mx, n2);
            md = std::max(md, e2);
        }
        r2 += mx;
        d2 += md;
    }
    double cmax = 0.0;
    for (int l = 0; l < h->nlist; l++) {
        double n2 = 0.0;
        for (int e = 0; e < dim; e++) {
            const double v = h->h_coarse[(size_t)l * dim + e];
            n2 += v * v;
        }
        cmax = std::max(cmax, n2);
    }
    const double rmax = std::sqrt(r2) * 1.0001, rd = std::sqrt(d2) * 1.0001;
    cmax = std::sqrt(cmax) * 1.0001;
    h->lms_bound.rmax = (float)rmax;
    h->lms_bound.rd = (float)rd;
    h->lms_bound.tmax = (float)((rmax * rmax + 2.0 * cmax * rmax) * 1.0001);
    h->lms_bound.kpad = (dim + 15) / 16 * 16;
    if (!std::isfinite(h->lms_bound.tmax) || rmax > 6.0e4) {
        // FP16 cannot hold these codewords: the table scan serves every batch
        h->lms_ok = false;
        return HANN_OK;
    }
    CK(upload(h->d_cb16, cb16.data(), cb16.size(), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

// Centred codebooks for the FP16 lookup tables (kernels_scan.cu): each
// codeword minus its subquantizer's mean, in the table-build layout
// [pqK][M][dsub]; the means; each subquantizer's largest centred codeword
// norm (rounded up); and the bounds max ||r|| <= sqrt(sum_m max_j
// ||c_mj||^2) and |term| <= rmax^2 + 2 max ||c|| rmax that size the screen's
// allowance for FP32 roundings.
static int prepare_adc(hann_pqivf* h) {
    const int M = h->o.num_subquantizers, K = h->pqk_eff, ds = h->dsub, dim = h->o.dimension;
    if (!scan_adc_supported(M) || K <= 0 || h->nlist <= 0) return HANN_OK;
    std::vector<float> cbc((size_t)K * M * ds), mu((size_t)dim, 0.0f), rm(M);
    double r2 = 0.0;
    for (int m = 0; m < M; m++) {
        const float* cb = h->h_codebooks.data() + (size_t)m * K * ds;
        for (int e = 0; e < ds; e++) {
            double a = 0.0;
            for (int j = 0; j < K; j++) a += cb[(size_t)j * ds + e];
            mu[(size_t)m * ds + e] = (float)(a / K);
        }
        double cmx = 0.0, mx = 0.0;
        for (int j = 0; j < K; j++) {
            double n2 = 0.0, c2 = 0.0;
            for (int e = 0; e < ds; e++) {
                const float v = cb[(size_t)j * ds + e];
                const float c = v - mu[(size_t)m * ds + e];
                cbc[((size_t)j * M + m) * ds + e] = c;
                n2 += (double)v * v;
                c2 += (double)c * c;
            }
            mx = std::max(mx, n2);
            cmx = std::max(cmx, c2);
        }
        rm[m] = (float)(std::sqrt(cmx) * 1.0001);
        r2 += mx;
    }
    double cmax = 0.0;
    for (int l = 0; l < h->nlist; l++) {
        double n2 = 0.0;
        for (int e = 0; e < dim; e++) {
            const double v = h->h_coarse[(size_t)l * dim + e];
            n2 += v * v;
        }
        cmax = std::max(cmax, n2);
    }
    const double rfull = std::sqrt(r2) * 1.0001;
    cmax = std::sqrt(cmax) * 1.0001;
    h->adc_rfull = (float)rfull;
    h->adc_tbound = (float)((rfull * rfull + 2.0 * cmax * rfull) * 1.0001);
    CK(upload(h->d_adc_cb, cbc.data(), cbc.size(), h->stream));
    CK(upload(h->d_adc_mu, mu.data(), mu.size(), h->stream));
    CK(upload(h->d_adc_rm, rm.data(), rm.size(), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}

// BF16 centroids, their FP32 squared norms and the largest norm, for the
// tensor-core preselection (dimensions up to 128).
static int prepare_coarse(hann_pqivf* h) {
    {
        int rc = prepare_lms(h);
        if (rc) return rc;
        rc = prepare_adc(h);
        if (rc) return rc;
    }
    if (h->nlist > 0 && h->pqk_eff > 0) {
        const size_t ncb = (size_t)h->o.num_subquantizers * h->pqk_eff * h->dsub;
        CK(h->d_codebooks_t.reserve(ncb));
        CK(launch_transpose_codebooks(h->d_codebooks.p, h->o.num_subquantizers, h->pqk_eff, h->dsub,
                                      h->d_codebooks_t.p, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    h->tc = !h->o.plain_fp32 && h->o.dimension <= 128 && h->nlist > 0;
    if (!h->tc) return HANN_OK;
    h->kp = gemm_kpad(h->o.dimension);
    CK(h->d_coarse_bf16.reserve((size_t)h->nlist * h->kp));
    CK(h->d_coarse_norm.reserve((size_t)h->nlist));
    CK(h->d_cmax.reserve(2));
    DBuf<float> cres;
    CK(cres.reserve((size_t)h->nlist));
    CK(h->d_err.reserve(1));
    CK(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), h->stream));
    CK(launch_to_bf16(h->d_coarse.p, h->nlist, h->o.dimension, h->kp, h->d_coarse_bf16.p, h->d_coarse_norm.p,
                      cres.p, h->stream));
    CK(launch_norm_maxes(h->d_coarse_norm.p, cres.p, h->nlist, h->d_cmax.p, h->stream));
    CK(h->d_coarse_terms.reserve((size_t)h->nlist));
    CK(launch_sq_terms(h->d_coarse_norm.p, h->nlist, h->d_coarse_terms.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return HANN_OK;
}


// Exact nearest centroid (reference-order FP32, lowest index on a tie) of
// every row of x: BF16 tensor-core preselection of 8 candidates per row, an
// exact rescore of the candidates, and the exact tiled kernel for the rows
// whose candidate band overflows (kernels_rescore.cu).
static int assign_rows(hann_pqivf* h, AssignScratch& sc, const float* x, int64_t n, int dim, const float* cent,
                       int k, int32_t* out_idx) {
    cudaStream_t s = h->stream;
    if (n <= 0) return HANN_OK;
    if (dim > 128 || h->o.plain_fp32) {
        DBuf<unsigned long long> keys;
        CK(keys.reserve((size_t)n));
        CK(launch_assign_exact(x, n, dim, cent, k, out_idx, nullptr, keys.p, s));
        return HANN_OK;
    }
    const int kp = gemm_kpad(dim);
    if (!sc.x_ready) {
        CK(sc.xbf.reserve((size_t)n * kp));
        CK(sc.xn2.reserve((size_t)n));
        CK(sc.xres.reserve((size_t)n));
        CK(launch_to_bf16(x, n, dim, kp, sc.xbf.p, sc.xn2.p, sc.xres.p, s));
        CK(sc.cand_idx.reserve((size_t)n * gemm_topc()));
        CK(sc.cand_val.reserve((size_t)n * gemm_topc()));
        CK(sc.ovf_rows.reserve((size_t)n));
        CK(sc.counters.reserve(2));
        CK(sc.cmax.reserve(2));
        sc.x_ready = true;
    }
    CK(sc.cbf.reserve((size_t)k * kp));
    CK(sc.cn2.reserve((size_t)k));
    CK(sc.cres.reserve((size_t)k));
    CK(launch_to_bf16(cent, k, dim, kp, sc.cbf.p, sc.cn2.p, sc.cres.p, s));
    CK(launch_norm_maxes(sc.cn2.p, sc.cres.p, k, sc.cmax.p, s));
    CK(cudaMemsetAsync(sc.counters.p, 0, 2 * sizeof(int), s));
    CK(sc.d2.reserve((size_t)n));
    // Warm: every row's nearest centroid is among those whose screened score
    // lies under a bound from the row's previous centroid (launch_warm_bound),
    // so the filter form of the GEMM keeps just those and an exact rescore
    // picks among them; the top-8 screen otherwise.
    constexpr int WARM_CAP = 32;
    const bool warm = sc.warm_ok && sc.warm && !sc.warm_skip && sc.warm_k == k && sc.warm_n == n &&
                      sc.warm_cent == cent;
    if (warm) {
        CK(sc.shift.reserve((size_t)k));
        CK(sc.cterm.reserve((size_t)k));
        CK(sc.rthr.reserve((size_t)n));
        CK(sc.fcnt.reserve((size_t)n));
        CK(sc.fcand.reserve((size_t)n * WARM_CAP));
        CK(sc.fcand_s.reserve((size_t)n * WARM_CAP));
        CK(launch_centroid_shift(cent, sc.cent_old.p, k, dim, sc.shift.p, s));
        CK(launch_warm_bound(sc.d2.p, out_idx, sc.shift.p, sc.xn2.p, sc.xres.p, sc.cmax.p, kp, n, sc.rthr.p, s));
        CK(launch_sq_terms(sc.cn2.p, k, sc.cterm.p, s));
        CK(cudaMemsetAsync(sc.fcnt.p, 0, sizeof(int32_t) * (size_t)n, s));
        CK(launch_gemm_filter(sc.xbf.p, n, sc.cbf.p, k, kp, 0, k, sc.cterm.p, 0, sc.rthr.p, WARM_CAP, sc.fcnt.p,
                              sc.fcand.p, sc.fcand_s.p, sc.counters.p + 1, s, false));
        CK(launch_rescore_filtered(x, n, dim, cent, sc.fcnt.p, sc.fcand.p, WARM_CAP, out_idx, sc.d2.p,
                                   sc.ovf_rows.p, sc.counters.p, s));
    } else {
        CK(launch_gemm_top8(sc.xbf.p, n, sc.cbf.p, k, kp, sc.cn2.p, sc.cand_idx.p, sc.cand_val.p, sc.counters.p + 1,
                            s));
        CK(launch_rescore_top8(x, sc.xn2.p, sc.xres.p, n, dim, kp, cent, k, sc.cmax.p, sc.cand_idx.p,
                               sc.cand_val.p, out_idx, sc.d2.p, sc.ovf_rows.p, sc.counters.p, s));
    }
    int hc[2] = {0, 0};
    CK(cudaMemcpyAsync(hc, sc.counters.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (hc[1]) return h->fail(HANN_E_CUDA, "tensor-core distance kernel timed out waiting on its pipeline");
    const int64_t novf = hc[0];
    if (novf > 0) {
        CK(sc.ovf_x.reserve((size_t)novf * dim));
        CK(sc.ovf_idx.reserve((size_t)novf));
        CK(sc.ovf_d2.reserve((size_t)novf));
        DBuf<unsigned long long> keys;
        CK(keys.reserve((size_t)novf));
        CK(launch_copy_words(x, sc.ovf_rows.p, sc.ovf_x.p, nullptr, novf, dim, s));
        CK(launch_assign_exact(sc.ovf_x.p, novf, dim, cent, k, sc.ovf_idx.p, sc.ovf_d2.p, keys.p, s));
        CK(launch_copy_words(sc.ovf_idx.p, nullptr, out_idx, sc.ovf_rows.p, novf, 1, s));
        CK(launch_copy_words(sc.ovf_d2.p, nullptr, sc.d2.p, sc.ovf_rows.p, novf, 1, s));
        CK(cudaStreamSynchronize(s));
    }
    h->warm_assignments += warm ? 1 : 0;
    h->warm_overflow_rows += warm ? novf : 0;
    if (sc.warm_ok) {
        // the next assignment's bounds start from these centroids; after a
        // warm assignment that overflowed on more than 1 row in 20 (the
        // centroids still move far) the next one takes the top-8 screen
        CK(sc.cent_old.reserve((size_t)k * dim));
        CK(cudaMemcpyAsync(sc.cent_old.p, cent, sizeof(float) * (size_t)k * dim, cudaMemcpyDeviceToDevice, s));
        sc.warm = true;
        sc.warm_skip = warm && novf * 20 > n;
        sc.warm_k = k;
        sc.warm_n = n;
        sc.warm_cent = cent;
    }
    return HANN_OK;
}

// Adding n vectors (ids ascending, host memory) to a trained index
// (assignLocked, pqivf/index.go:245-260) runs in two phases. add_prepare
// computes every vector's nearest list, codes and term into the handle's
// mutation scratch and changes nothing; it reports whether some list would
// overflow its capacity (a relayout). add_commit then appends the rows in
// place -- a concurrent search sees each list either before or after the
// append -- or relayouts first when needed.
int add_prepare(hann_pqivf* h, const int64_t* ids, const float* vecs, int64_t n) {
    MutationScratch& m = h->mut;
    m.held = false;
    m.n = n;
    m.grow = false;
    if (n <= 0) return HANN_OK;
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    CK(upload(m.x, vecs, (size_t)n * dim, h->stream));
    CK(m.asg.reserve((size_t)n));
    CK(m.term.reserve((size_t)n));
    CK(m.codes.reserve((size_t)n * h->code_stride));
    m.asc.x_ready = false;
    int rc = assign_rows(h, m.asc, m.x.p, n, dim, h->d_coarse.p, h->nlist, m.asg.p);
    if (rc) return rc;
    CK(launch_encode(m.x.p, nullptr, m.asg.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, h->pqk_eff, m.codes.p,
                     h->code_stride, m.term.p, h->stream));
    m.hasg.resize((size_t)n);
    CK(cudaMemcpyAsync(m.hasg.data(), m.asg.p, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    m.add.assign(h->nlist, 0);
    for (int64_t i = 0; i < n; i++) m.add[m.hasg[i]]++;
    for (int l = 0; l < h->nlist; l++)
        if ((int64_t)h->list_ids[l].size() + m.add[l] > h->h_cap[l]) m.grow = true;
    return HANN_OK;
}

int add_commit(hann_pqivf* h, const int64_t* ids) {
    MutationScratch& m = h->mut;
    const int64_t n = m.n;
    if (n <= 0) return HANN_OK;
    const int dim = h->o.dimension;
    if (m.grow) {
        // lists over capacity move to the arena's tail with twice their
        // rows of room, when it has space
        std::vector<int> gl;
        std::vector<int64_t> gc;
        for (int l = 0; l < h->nlist; l++) {
            const int64_t need = (int64_t)h->list_ids[l].size() + m.add[l];
            if (need <= h->h_cap[l]) continue;
            gl.push_back(l);
            gc.push_back(std::max<int64_t>(list_capacity(2 * (h->live_count[l] + m.add[l])), round_up(need, 32)));
        }
        bool moved = false;
        int grc = grow_lists(h, gl, gc, &moved);
        if (grc) return grc;
        if (moved) m.grow = false;
    }
    if (m.grow) {
        // otherwise one relayout of every list, which also drops every tombstone
        std::vector<int64_t> caps(h->nlist);
        // every list gets its headroom back; lists that overflowed double
        for (int l = 0; l < h->nlist; l++) {
            const int64_t live = h->live_count[l] + m.add[l];
            const int64_t need = (int64_t)h->list_ids[l].size() + m.add[l];
            caps[l] = std::max(h->h_cap[l], need > h->h_cap[l] ? list_capacity(2 * live) : list_capacity(live));
        }
        int rc = relayout(h, caps);
        if (rc) return rc;
        m.grow = false;
    }
    std::vector<int64_t> dst((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const int c = m.hasg[i];
        dst[i] = h->h_start[c] + (int64_t)h->list_ids[c].size();
        h->list_ids[c].push_back(ids[i]);
        h->list_alive[c].push_back(1);
        h->live_count[c]++;
        h->id_cluster.set(ids[i], c);
        h->cluster_counts[c]++;
        h->list_key[c] = 1;
    }
    CK(upload(m.dst, dst.data(), dst.size(), h->stream));
    CK(upload(m.ids, ids, (size_t)n, h->stream));
    CK(launch_copy_words(m.x.p, nullptr, h->d_vectors.p, m.dst.p, n, dim, h->stream));
    CK(launch_copy_words(m.codes.p, nullptr, h->d_codes.p, m.dst.p, n, h->code_stride / 4, h->stream));
    CK(launch_copy_words(m.ids.p, nullptr, h->d_row_id.p, m.dst.p, n, 2, h->stream));
    CK(launch_copy_words(m.asg.p, nullptr, h->d_row_cluster.p, m.dst.p, n, 1, h->stream));
    CK(launch_scan_codes_rows(h->d_codes.p, h->code_stride, h->o.num_subquantizers, h->d_start.p, h->d_swstart.p,
                              m.dst.p, m.asg.p, n, h->d_scanc.p, h->stream));
    // the term last: a row becomes selectable only once it is complete
    CK(launch_copy_words(m.term.p, nullptr, h->d_term.p, m.dst.p, n, 1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return upload_lens(h);
}

static int assign_batch(hann_pqivf* h, const int64_t* ids, const float* vecs, int64_t n) {
    int rc = add_prepare(h, ids, vecs, n);
    if (rc) return rc;
    return add_commit(h, ids);
}

// Removes the given (already validated, trained-side) ids (deleteLocked,
// pqivf/index.go:313-345). A removed row becomes a tombstone: its term is set
// to +inf, so no scan can select it, and its id to -1; the live rows keep
// their places, so the lists keep their order and concurrent readers never
// see a row move. A relayout compacts the tombstones away once they exceed a
// quarter of the slots.
static int remove_rows(hann_pqivf* h, const std::vector<int64_t>& ids) {
    h->mut.held = false;
    if (ids.empty()) return HANN_OK;
    std::vector<int64_t> rows;
    for (int64_t id : ids) {
        const int32_t* lp = h->id_cluster.find(id);
        if (!lp) continue;
        const int l = *lp;
        auto& lst = h->list_ids[l];
        for (size_t j = 0; j < lst.size(); j++) {
            if (h->list_alive[l][j] && lst[j] == id) {
                h->list_alive[l][j] = 0;
                rows.push_back(h->h_start[l] + (int64_t)j);
                break;
            }
        }
        h->live_count[l]--;
        h->cluster_counts[l]--;
        h->dead_rows++;
        h->id_cluster.erase(id);
    }
    if (!rows.empty()) {
        CK(upload(h->mut.rows, rows.data(), rows.size(), h->stream));
        CK(launch_tombstone(h->mut.rows.p, (int64_t)rows.size(), h->d_term.p, h->d_row_id.p, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    if (compaction_due(h, 0)) {
        const std::vector<int64_t> caps = h->h_cap;
        int rc = relayout(h, caps);
        if (rc) return rc;
    }
    return upload_lens(h);
}

// Whether deleting `extra` more live rows would trigger the compacting
// relayout (tombstones above a quarter of the slots).
bool compaction_due(const hann_pqivf* h, int64_t extra) {
    int64_t slots = 0;
    for (int l = 0; l < h->nlist; l++) slots += (int64_t)h->list_ids[l].size();
    return (h->dead_rows + extra) * 4 > slots;
}

// ---------------------------------------------------------------------------
// Train (pqivf/index.go:451-605) on the device.

struct SeedSource {
    const int64_t* coarse_init = nullptr;
    const int64_t* pq_init = nullptr;
    const int64_t* reseed = nullptr;
    int64_t n_reseed = 0;
    int64_t reseed_used = 0;
    // warm start (Retrain): k-means from the index's own centroids and
    // codebooks (device arrays) for warm_iters iterations
    const float* warm_coarse = nullptr;
    const float* warm_codebooks = nullptr;
    int warm_iters = 0;
};

static int64_t draw_reseed(hann_pqivf* h, SeedSource& src, int64_t n, bool& ok) {
    ok = true;
    if (src.reseed) {
        if (src.reseed_used >= src.n_reseed) {
            ok = false;
            return 0;
        }
        const int64_t v = src.reseed[src.reseed_used++];
        if (v < 0 || v >= n) ok = false;
        return v;
    }
    return h->rng.intn(n);
}

// Lloyd iterations over rows of x (n x dim) into cent (k x dim), as runKMeans
// (pqivf/index.go:795-847): init rows given, FP64 sums, FP32 mean, empty
// clusters reseeded from `reseed` in cluster order.
static int kmeans_device(hann_pqivf* h, const float* x, int64_t ld, int off, int64_t n, int dim, int k, int iters,
                         const std::vector<int64_t>& init, SeedSource& seeds, float* cent, int32_t* asg_buf,
                         bool sub_mode, const float* sub_full, int M, int m, AssignScratch* sc,
                         const float* init_cent = nullptr) {
    // sub_mode: x is the full residual matrix [n][M*dim]; k-means runs on
    // columns [m*dim, (m+1)*dim) and cent is codebook m ([k][dim]).
    // init_cent: start from these centroids instead of the init rows.
    DBuf<int64_t> dsrc;
    DBuf<double> sums;
    DBuf<int64_t> counts;
    if (init_cent) {
        CK(cudaMemcpyAsync(cent, init_cent, sizeof(float) * (size_t)k * dim, cudaMemcpyDeviceToDevice, h->stream));
    } else {
        CK(upload(dsrc, init.data(), init.size(), h->stream));
        CK(launch_gather_cols(x, ld, off, dsrc.p, nullptr, k, dim, cent, dim, h->stream));
    }
    CK(sums.reserve((size_t)k * dim * (sub_mode ? M : 1)));
    CK(counts.reserve((size_t)k * (sub_mode ? M : 1)));
    std::vector<int64_t> hcounts(k);
    for (int it = 0; it < iters; it++) {
        if (!sub_mode) {
            int rc = assign_rows(h, *sc, x, n, dim, cent, k, asg_buf);
            if (rc) return rc;
            CK(cudaMemsetAsync(sums.p, 0, (size_t)k * dim * sizeof(double), h->stream));
            CK(cudaMemsetAsync(counts.p, 0, (size_t)k * sizeof(int64_t), h->stream));
            CK(launch_kmeans_accumulate(x, n, dim, asg_buf, sums.p, counts.p, h->stream));
            CK(launch_kmeans_finalize(sums.p, counts.p, k, dim, cent, h->stream));
            CK(cudaMemcpyAsync(hcounts.data(), counts.p, (size_t)k * sizeof(int64_t), cudaMemcpyDeviceToHost,
                               h->stream));
        } else {
            // cent points at codebook m inside the [M][k][dim] codebook array.
            const float* cb_all = cent - (int64_t)m * k * dim;
            CK(cudaMemsetAsync(sums.p + (size_t)m * k * dim, 0, (size_t)k * dim * sizeof(double), h->stream));
            CK(cudaMemsetAsync(counts.p + (size_t)m * k, 0, (size_t)k * sizeof(int64_t), h->stream));
            if (pq_assign_accumulate_supported(dim, k)) {
                CK(launch_pq_assign_accumulate(sub_full, n, M, dim, cb_all, k, m, asg_buf, sums.p + (size_t)m * k * dim,
                                               counts.p + (size_t)m * k, h->stream));
            } else {
                CK(launch_pq_assign(sub_full, n, M, dim, cb_all, k, m, m + 1, asg_buf, h->stream));
                CK(launch_pq_accumulate(sub_full, n, M, dim, asg_buf, k, m, m + 1, sums.p, counts.p, h->stream));
            }
            CK(launch_kmeans_finalize(sums.p + (size_t)m * k * dim, counts.p + (size_t)m * k, k, dim, cent,
                                      h->stream));
            CK(cudaMemcpyAsync(hcounts.data(), counts.p + (size_t)m * k, (size_t)k * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        std::vector<int64_t> rs;
        std::vector<int32_t> rd;
        for (int c = 0; c < k; c++) {
            if (hcounts[c] == 0) {
                bool ok;
                const int64_t r = draw_reseed(h, seeds, n, ok);
                if (!ok) return h->fail(HANN_E_INVALID, "reseed index stream exhausted or out of range");
                rs.push_back(r);
                rd.push_back(c);
            }
        }
        if (!rs.empty()) {
            DBuf<int64_t> drs;
            DBuf<int32_t> drd;
            CK(upload(drs, rs.data(), rs.size(), h->stream));
            CK(upload(drd, rd.data(), rd.size(), h->stream));
            CK(launch_gather_cols(x, ld, off, drs.p, drd.p, (int64_t)rs.size(), dim, cent, dim, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
    }
    return HANN_OK;
}

static double ms_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

static int train_impl(hann_pqivf* h, SeedSource seeds) {
    h->mut.held = false;
    auto t_phase = std::chrono::steady_clock::now();
    for (double& v : h->train_phase_ms) v = 0;
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    // Consolidate every vector, clustered and pending, in ascending id order.
    // Source of each vector: its row in the device lists (>= 0), or -(slot + 1)
    // for slot `slot` of the pending array, which is uploaded whole.
    std::vector<std::pair<int64_t, int64_t>> all;  // (id, source)
    all.reserve(h->id_cluster.size() + h->pending.size());
    for (int l = 0; l < h->nlist; l++)
        for (size_t j = 0; j < h->list_ids[l].size(); j++)
            if (h->list_alive[l][j]) all.emplace_back(h->list_ids[l][j], h->h_start[l] + (int64_t)j);
    const PendingStore& pend = h->pending;
    for (size_t i = 0; i < pend.slot_id.size(); i++)
        if (pend.slot_live[i]) all.emplace_back(pend.slot_id[i], -(int64_t)i - 1);
    const int64_t n = (int64_t)all.size();
    if (n < h->o.coarse_k)
        return h->fail(HANN_E_STATE, "not enough vectors (%lld) to train coarse quantizer with %d clusters",
                       (long long)n, h->o.coarse_k);
    if (n >= (int64_t)1 << 31) return h->fail(HANN_E_UNSUPPORTED, "more than 2^31 vectors");
    if (!std::is_sorted(all.begin(), all.end())) std::sort(all.begin(), all.end());
    std::vector<int64_t> ids(n), src(n);
    bool direct = pend.dim == dim && (int64_t)pend.slot_id.size() == n;  // every vector pending, slots in id order
    for (int64_t i = 0; i < n; i++) {
        ids[i] = all[i].first;
        src[i] = all[i].second;
        direct = direct && src[i] == -i - 1;
    }
    std::vector<std::pair<int64_t, int64_t>>().swap(all);
    DBuf<float> X;
    CK(X.reserve((size_t)n * dim));
    if (direct) {
        CK(cudaMemcpyAsync(X.p, pend.vec.data(), sizeof(float) * (size_t)n * dim, cudaMemcpyHostToDevice,
                           h->stream));
    } else {
        DBuf<float> dstage;
        DBuf<int64_t> dsrc;
        if (!pend.vec.empty()) CK(upload(dstage, pend.vec.data(), pend.vec.size(), h->stream));
        CK(upload(dsrc, src.data(), src.size(), h->stream));
        CK(launch_gather2(h->d_vectors.p ? h->d_vectors.p : X.p, dstage.p, dsrc.p, n, dim, X.p, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    h->train_phase_ms[0] = ms_since(t_phase);
    t_phase = std::chrono::steady_clock::now();

    // Coarse k-means (runKMeans(allVectors, coarseK, iters)).
    const int k = (int)std::min<int64_t>(h->o.coarse_k, n);
    const bool warm = seeds.warm_coarse != nullptr;
    if (warm && k != h->nlist)
        return h->fail(HANN_E_STATE, "retrain needs the trained list count (%d); %lld vectors give %d", h->nlist,
                       (long long)n, k);
    std::vector<int64_t> init;
    if (warm) {
    } else if (seeds.coarse_init) {
        init.assign(seeds.coarse_init, seeds.coarse_init + k);
        for (int64_t v : init)
            if (v < 0 || v >= n) return h->fail(HANN_E_INVALID, "coarse init index out of range");
    } else {
        init = h->rng.perm_prefix(n, k);
    }
    DBuf<float> C;
    DBuf<int32_t> asg;
    CK(C.reserve((size_t)k * dim));
    CK(asg.reserve((size_t)n));
    AssignScratch asc;
    asc.warm_ok = true;  // iterations after the first, and the final assignment, may take the warm filter
    int rc = kmeans_device(h, X.p, dim, 0, n, dim, k, warm ? seeds.warm_iters : h->o.kmeans_iters, init, seeds, C.p,
                           asg.p, false, nullptr, 0, 0, &asc, seeds.warm_coarse);
    if (rc) return rc;
    // Final assignment and inverted lists in ascending (cluster, id) order.
    rc = assign_rows(h, asc, X.p, n, dim, C.p, k, asg.p);
    if (rc) return rc;
    std::vector<int32_t> hasg(n);
    CK(cudaMemcpyAsync(hasg.data(), asg.p, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->train_phase_ms[1] = ms_since(t_phase);
    t_phase = std::chrono::steady_clock::now();
    std::vector<int64_t> cnt(k, 0);
    for (int64_t i = 0; i < n; i++) cnt[hasg[i]]++;
    std::vector<int64_t> off(k + 1, 0);
    for (int c = 0; c < k; c++) off[c + 1] = off[c] + cnt[c];
    std::vector<int64_t> order(n);  // list-order position -> X row
    {
        std::vector<int64_t> fill(off.begin(), off.end() - 1);
        for (int64_t i = 0; i < n; i++) order[fill[hasg[i]]++] = i;
    }
    std::vector<int32_t> ord_cluster(n);
    for (int64_t j = 0; j < n; j++) ord_cluster[j] = hasg[order[j]];

    // Residuals in list order feed the subquantizer k-means.
    DBuf<int64_t> dorder;
    DBuf<int32_t> dordc;
    DBuf<float> Rm;
    CK(upload(dorder, order.data(), order.size(), h->stream));
    CK(upload(dordc, ord_cluster.data(), ord_cluster.size(), h->stream));
    CK(Rm.reserve((size_t)n * dim));
    CK(launch_residuals(X.p, dorder.p, dordc.p, n, dim, C.p, Rm.p, h->stream));
    const int kpq = (int)std::min<int64_t>(h->o.pq_k, n);
    const int ds = dim / M;
    if (warm && kpq != h->pqk_eff)
        return h->fail(HANN_E_STATE, "retrain needs the trained codebook size (%d); %lld vectors give %d", h->pqk_eff,
                       (long long)n, kpq);
    DBuf<float> CB;
    CK(CB.reserve((size_t)M * kpq * ds));
    DBuf<int32_t> pqa;
    CK(pqa.reserve((size_t)n * M));
    for (int m = 0; m < M; m++) {
        std::vector<int64_t> pinit;
        if (warm) {
        } else if (seeds.pq_init) {
            pinit.assign(seeds.pq_init + (int64_t)m * h->o.pq_k, seeds.pq_init + (int64_t)m * h->o.pq_k + kpq);
            for (int64_t v : pinit)
                if (v < 0 || v >= n) return h->fail(HANN_E_INVALID, "subquantizer init index out of range");
        } else {
            pinit = h->rng.perm_prefix(n, kpq);
        }
        rc = kmeans_device(h, Rm.p, dim, m * ds, n, ds, kpq, warm ? seeds.warm_iters : h->o.kmeans_iters, pinit,
                           seeds, CB.p + (size_t)m * kpq * ds, pqa.p, true, Rm.p, M, m, nullptr,
                           warm ? seeds.warm_codebooks + (size_t)m * kpq * ds : nullptr);
        if (rc) return rc;
    }
    Rm.reset();
    h->train_phase_ms[2] = ms_since(t_phase);
    t_phase = std::chrono::steady_clock::now();

    // New layout and state.
    h->nlist = k;
    h->pqk_eff = kpq;
    h->list_ids.assign(k, {});
    h->list_key.assign(k, 0);
    h->cluster_counts.assign(k, 0);
    h->id_cluster.clear();
    h->id_cluster.reserve((size_t)n);
    for (int c = 0; c < k; c++) h->list_ids[c].reserve((size_t)cnt[c]);
    for (int64_t j = 0; j < n; j++) {
        const int c = ord_cluster[j];
        h->list_ids[c].push_back(ids[order[j]]);
        h->id_cluster.set(ids[order[j]], c);
    }
    h->list_alive.assign(k, {});
    h->live_count.assign(k, 0);
    for (int c = 0; c < k; c++) {
        h->list_alive[c].assign(h->list_ids[c].size(), 1);
        h->live_count[c] = (int64_t)h->list_ids[c].size();
    }
    h->dead_rows = 0;
    for (int c = 0; c < k; c++) {
        h->cluster_counts[c] = cnt[c];
        h->list_key[c] = cnt[c] > 0;
    }
    h->d_coarse.swap(C);
    h->d_codebooks.swap(CB);
    h->d_vectors.reset();
    h->d_term.reset();
    h->d_row_id.reset();
    h->d_row_cluster.reset();
    h->d_codes.reset();
    h->rows_cap = 0;
    std::vector<int64_t> caps(k);
    for (int c = 0; c < k; c++) caps[c] = list_capacity(cnt[c]);
    rc = relayout(h, caps, false);
    if (rc) return rc;
    std::vector<int64_t> dst(n), rid(n);
    std::vector<int32_t> rcl(n);
    {
        std::vector<int64_t> fill(k, 0);
        for (int64_t j = 0; j < n; j++) {
            const int c = ord_cluster[j];
            dst[j] = h->h_start[c] + fill[c]++;
            rid[j] = ids[order[j]];
            rcl[j] = c;
        }
    }
    DBuf<int64_t> ddst, drid;
    DBuf<int32_t> drcl;
    CK(upload(ddst, dst.data(), dst.size(), h->stream));
    CK(upload(drid, rid.data(), rid.size(), h->stream));
    CK(upload(drcl, rcl.data(), rcl.size(), h->stream));
    CK(launch_copy_words(X.p, dorder.p, h->d_vectors.p, ddst.p, n, dim, h->stream));
    CK(launch_copy_words(drid.p, nullptr, h->d_row_id.p, ddst.p, n, 2, h->stream));
    CK(launch_copy_words(drcl.p, nullptr, h->d_row_cluster.p, ddst.p, n, 1, h->stream));
    CK(launch_encode(h->d_vectors.p, ddst.p, h->d_row_cluster.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, kpq,
                     h->d_codes.p, h->code_stride, h->d_term.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->h_coarse.resize((size_t)k * dim);
    h->h_codebooks.resize((size_t)M * kpq * ds);
    CK(cudaMemcpy(h->h_coarse.data(), h->d_coarse.p, h->h_coarse.size() * sizeof(float), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->h_codebooks.data(), h->d_codebooks.p, h->h_codebooks.size() * sizeof(float),
                  cudaMemcpyDeviceToHost));
    h->pending.clear();
    h->trained = true;
    rc = prepare_coarse(h);
    if (rc) return rc;
    rc = upload_lens(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    h->train_phase_ms[3] = ms_since(t_phase);
    return HANN_OK;
}

// ---------------------------------------------------------------------------
// Search.

int rerank_depth(const hann_pqivf* h, int kmax, int mode) { return rerank_depth_for(kmax, mode, h->o.rerank); }

// Runs the device search for nq queries already in d_q; k/nprobe per query
// in device arrays d_k/d_np. Outputs to device buffers.
constexpr int SCREEN_MIN_LISTS = 2048;  // below this the full score matrix is cheaper
constexpr int PROBE_CAP = 4096;         // screened-probe candidates per query and chunk
constexpr int PROBE_FIRST = 256;        // first centroid chunk at least (every list enters the band)
// Largest candidate dump of the table scan (a larger chunk of queries selects
// inside the scan blocks instead)
constexpr size_t SCAN_DUMP_MAX = (size_t)1 << 30;


// Every scratch buffer run_search needs for nq queries (in chunks of at most
// 2^28 / nlist), reserved up front; a server calls it once per slot at start
// so no batch ever reaches the allocator.
bool lms_use(const hann_pqivf* h, int64_t nq, int np_max);
int reserve_lms_scratch(hann_pqivf* h, SearchScratch& sc, int64_t chunk, int np_max);

int reserve_search_scratch(hann_pqivf* h, SearchScratch& sc, int64_t nq, int np_max, int kmax, int mode) {
    const int R = rerank_depth(h, kmax, mode);
    np_max = std::min(np_max, h->nlist);
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nq, ((int64_t)1 << 28) / std::max(1, h->nlist)));
    CK(sc.D.reserve((size_t)chunk * h->nlist));
    if (h->tc) {
        CK(sc.qbf.reserve((size_t)chunk * h->kp));
        CK(sc.qn2.reserve((size_t)chunk));
        CK(sc.qres.reserve((size_t)chunk));
    }
    CK(sc.probe_ids.reserve((size_t)chunk * np_max));
    CK(sc.probe_d.reserve((size_t)chunk * np_max));
    CK(sc.fb.reserve((size_t)chunk));
    CK(sc.cand_row.reserve((size_t)chunk * R));
    CK(sc.cand_d.reserve((size_t)chunk * R));
    CK(sc.cand_seq.reserve((size_t)chunk * R));
    CK(sc.fbcount.reserve(1));
    CK(sc.scut.reserve((size_t)chunk));
    CK(sc.seps.reserve((size_t)chunk));
    CK(sc.credo.reserve((size_t)chunk + 1));
    if (!sc.dump_off && scan_adc_supported(h->o.num_subquantizers) &&
        (size_t)chunk * scan_dump_bytes(R) <= SCAN_DUMP_MAX)
        CK(sc.dump.reserve((size_t)chunk * scan_dump_bytes(R)));
    if (h->tc && h->nlist >= SCREEN_MIN_LISTS) {
        const int lcap = std::max(1024, 2 * np_max);
        CK(sc.pe2.reserve((size_t)chunk));
        CK(sc.pasl.reserve((size_t)chunk));
        CK(sc.pthr.reserve((size_t)chunk));
        CK(sc.pcnt.reserve((size_t)chunk));
        CK(sc.plcount.reserve((size_t)chunk));
        CK(sc.pneed.reserve((size_t)chunk));
        CK(sc.ptodo.reserve((size_t)chunk + 1));
        CK(sc.pcand_id.reserve((size_t)chunk * PROBE_CAP));
        CK(sc.pcand_s.reserve((size_t)chunk * PROBE_CAP));
        CK(sc.pband.reserve((size_t)chunk * lcap));
        CK(sc.qorder.reserve((size_t)chunk));
        CK(sc.order_scratch.reserve((size_t)h->nlist));
    }
    if (lms_use(h, chunk, np_max)) return reserve_lms_scratch(h, sc, chunk, np_max);
    return HANN_OK;
}

// ---------------------------------------------------------------------------
// The list-major scan (kernels_lms.cu) of one chunk of queries whose probe
// lists are in sc.probe_ids / probe_d / fb: work queue, chunked scan with
// band merges, candidates for the rerank; queries it cannot serve exactly
// are listed in sc.lredo (count at lredo[nc]) for the table scan.

static int sm_count(int dev) {
    static int cached[64] = {};
    if (dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cached[dev] = v;
    }
    return cached[dev];
}

static LmsChunks lms_chunks(const LmsConfig& cfg, int np_max) {
    LmsChunks ch{};
    ch.n = 0;
    ch.bound[0] = 0;
    int b = std::min(np_max, std::max(1, cfg.first));
    while (true) {
        ch.bound[++ch.n] = b;
        if (b >= np_max) break;
        if (ch.n == LMS_MAX_CHUNKS - 1) {
            ch.bound[++ch.n] = np_max;
            break;
        }
        b = std::min<int64_t>(np_max, (int64_t)b * std::max(2, cfg.growth));
    }
    return ch;
}

static int lms_cap(const hann_pqivf* h) {
    // the dense first chunk holds every row of its lists; otherwise the
    // threshold keeps the appends far below one list's length
    const int64_t first = h->lms.seed ? h->max_list_slots : std::max<int64_t>(1, h->lms.first) * h->max_list_slots;
    return (int)std::min<int64_t>(8192, std::max<int64_t>(h->lms.seed ? 4096 : 2048, round_up(first, 256)));
}
constexpr int LMS_LCAP = 2048;  // band list per query: the large warp form of the band merge

// Whether a batch takes the list-major scan: on the index's state and the
// batch size only, never on the other queries' k or nprobe, so that a
// query's result does not depend on its batch. (Every rerank depth this
// build accepts, at most 480, fits the band list.)
bool lms_use(const hann_pqivf* h, int64_t nq, int np_max) {
    return h->lms_ok && h->lms.enabled && nq >= h->lms.min_queries && np_max >= std::max(1, h->lms.min_nprobe);
}
static_assert(LMS_LCAP / 2 >= 480, "band lists must hold the largest rerank depth");

static int lms_item_cap(const hann_pqivf* h, int64_t nq, int np_max, const LmsChunks& ch) {
    int wmax = 0;
    for (int c = 0; c < ch.n; c++) wmax = std::max(wmax, ch.bound[c + 1] - ch.bound[c]);
    const int64_t pairs = nq * (int64_t)wmax;
    const int64_t groups = pairs / LMS_NQ + std::min<int64_t>(h->nlist, pairs);
    const int64_t ranges = h->max_list_slots / std::max(1, h->lms.rows_max) + 1;
    return (int)std::min<int64_t>(INT32_MAX / 2, groups * ranges + 1);
}

int reserve_lms_scratch(hann_pqivf* h, SearchScratch& sc, int64_t chunk, int np_max) {
    const LmsChunks ch = lms_chunks(h->lms, np_max);
    const int cap = lms_cap(h);
    const int icap = lms_item_cap(h, chunk, np_max, ch);
    CK(sc.q16.reserve((size_t)chunk * 128));
    CK(sc.le2.reserve((size_t)chunk));
    CK(sc.leps.reserve((size_t)chunk));
    CK(sc.lones.reserve((size_t)chunk));
    CK(sc.lzeros.reserve((size_t)chunk));
    CK(sc.lasl.reserve((size_t)chunk));
    CK(sc.lthr.reserve((size_t)chunk));
    CK(sc.lcnt.reserve((size_t)chunk));
    CK(sc.llcount.reserve((size_t)chunk));
    CK(sc.lneed.reserve((size_t)chunk));
    CK(sc.lbandk.reserve((size_t)chunk));
    CK(sc.ltodo.reserve((size_t)chunk + 1));
    CK(sc.lredo.reserve((size_t)chunk + 1));
    CK(sc.lcand_id.reserve((size_t)chunk * cap));
    CK(sc.lcand_s.reserve((size_t)chunk * cap));
    CK(sc.lband.reserve((size_t)chunk * LMS_LCAP));
    CK(sc.lcounts.reserve((size_t)ch.n * h->nlist));
    CK(sc.lcursor.reserve((size_t)ch.n * h->nlist));
    CK(sc.ltotal.reserve(2));
    CK(sc.lpair_q.reserve((size_t)chunk * np_max));
    CK(sc.lpair_base.reserve((size_t)chunk * np_max));
    CK(sc.lpair_off.reserve((size_t)chunk * np_max));
    CK(sc.litems.reserve((size_t)ch.n * icap));
    CK(sc.ln_items.reserve((size_t)ch.n));
    CK(sc.litem_counter.reserve(1));
    CK(sc.lstats.reserve(2));
    return HANN_OK;
}

static int run_lms(hann_pqivf* h, SearchScratch& sc, const float* qp, int64_t nc, const int32_t* d_k,
                   const int32_t* d_np, int np_max, int kmax, int mode, int R, cudaStream_t s) {
    const LmsChunks ch = lms_chunks(h->lms, np_max);
    const int cap = lms_cap(h);
    const int icap = lms_item_cap(h, nc, np_max, ch);
    const int M = h->o.num_subquantizers;
    const bool seed = h->lms.seed != 0;
    CK(launch_lms_prep(qp, nc, h->o.dimension, sc.probe_ids.p, sc.probe_d.p, d_np, np_max, sc.fb.p, h->d_len.p,
                       seed ? 0 : ch.bound[1], h->lms.min_nprobe, h->lms_bound, mode, d_k, h->o.rerank, sc.lbandk.p,
                       sc.leps.p, sc.q16.p,
                       sc.le2.p, sc.lasl.p, sc.lcnt.p, sc.llcount.p, sc.lthr.p, sc.lneed.p, s));
    if (seed) {
        // the table scan of each query's nearest list (no brute-force
        // fallback: those queries go to the table scan anyway) sets the
        // first thresholds
        ScanParams ps = h->scan_params();
        ps.mode = mode;
        ps.kq = d_k;
        ps.adc_table = 0;  // the thresholds must bound exact distances: FP32 tables
        CK(launch_fill_i32(sc.lones.p, nc, 1, s));
        CK(cudaMemsetAsync(sc.lzeros.p, 0, sizeof(int32_t) * (size_t)nc, s));
        CK(launch_scan(ps, qp, nc, sc.probe_ids.p, sc.probe_d.p, sc.lones.p, np_max, sc.lzeros.p, R, sc.cand_row.p,
                       sc.cand_d.p, sc.cand_seq.p, nullptr, s));
        CK(launch_lms_seed(nc, R, sc.cand_d.p, sc.lbandk.p, sc.leps.p, sc.le2.p, sc.lasl.p, sc.lthr.p, s));
        h->launches += 3;
    }
    CK(launch_lms_queue(sc.probe_ids.p, sc.probe_d.p, d_np, nc, np_max, sc.lneed.p, ch, h->nlist, h->d_len.p,
                        h->d_start.p, h->lms.rows_max, icap, sc.lcounts.p, sc.lcursor.p, sc.ltotal.p, sc.litems.p, sc.ln_items.p,
                        sc.lpair_q.p, sc.lpair_base.p, sc.lpair_off.p, s));
    LmsParams lp{};
    lp.codes = h->d_codes.p;
    lp.code_stride = h->code_stride;
    lp.term = h->d_term.p;
    lp.list_start = h->d_start.p;
    lp.cb16 = h->d_cb16.p;
    lp.M = M;
    lp.dsub = h->dsub;
    lp.pqK = h->pqk_eff;
    lp.dim = h->o.dimension;
    lp.q16 = sc.q16.p;
    lp.item_counter = sc.litem_counter.p;
    lp.item_cap = icap;
    lp.pair_q = sc.lpair_q.p;
    lp.pair_base = sc.lpair_base.p;
    lp.pair_off = sc.lpair_off.p;
    lp.thr = sc.lthr.p;
    lp.cnt = sc.lcnt.p;
    lp.cand_id = sc.lcand_id.p;
    lp.cand_s = sc.lcand_s.p;
    lp.cap = cap;
    lp.stats = h->profile ? h->s_rows.p : nullptr;
    lp.err = h->d_err.p;
    const int grid = sm_count(h->o.device) * std::max(1, h->lms.ctas_per_sm);
    const int bandk_max = mode == 0 ? kmax : R;
    for (int c = 0; c < ch.n; c++) {
        lp.items = sc.litems.p + (int64_t)c * icap;
        lp.n_items = sc.ln_items.p + c;
        lp.dense = !seed && c == 0 ? 1 : 0;
        CK(launch_lms_scan(lp, grid, s));
        // k >= 33 selects the band merge's large warp form (2,048 keys a row)
        CK(launch_knn_merge_band((int)nc, std::max(bandk_max, 64), sc.lbandk.p, cap, LMS_LCAP, sc.lcnt.p,
                                 sc.lcand_id.p, sc.lcand_s.p, sc.le2.p, sc.lasl.p, sc.lband.p, sc.llcount.p,
                                 sc.lthr.p, sc.lneed.p, sc.ltodo.p, s));
    }
    CK(launch_lms_finish(nc, mode, R, LMS_LCAP, d_k, h->o.rerank, sc.lband.p, sc.llcount.p, sc.lneed.p,
                         sc.probe_ids.p, d_np, np_max, h->d_row_cluster.p, sc.ltotal.p + 1, sc.cand_row.p,
                         sc.cand_seq.p, sc.lredo.p, s));
    h->launches += 8 + 5 * ch.n;
    return HANN_OK;
}

int run_search(hann_pqivf* h, SearchScratch& sc, const float* d_q, int64_t nq, const int32_t* d_k,
                      const int32_t* d_np, int np_max, int kmax, int mode, int64_t* d_ids, double* d_dist,
                      int32_t* d_nout, cudaStream_t s, unsigned long long* fb_counter) {
    unsigned long long* fbc = fb_counter ? fb_counter : sc.fbcount.p;
    const int R = rerank_depth(h, kmax, mode);
    if (R > 480) return h->fail(HANN_E_UNSUPPORTED, "k (%d) above this build's limit of 448", kmax);
    np_max = std::min(np_max, h->nlist);
    if (np_max > 4096) return h->fail(HANN_E_UNSUPPORTED, "more than 4096 probed lists per query");
    ScanParams p = h->scan_params();
    p.mode = mode;
    p.rerank_fixed = h->o.rerank;
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nq, ((int64_t)1 << 28) / std::max(1, h->nlist)));
    int rrc = reserve_search_scratch(h, sc, nq, np_max, kmax, mode);
    if (rrc) return rrc;
    if (sc.dump.p && sc.dump.n >= (size_t)chunk * scan_dump_bytes(R)) p.dump = sc.dump.p;
    const int scan_launches = p.dump ? 2 : 1;  // the table scan and, with a dump, its selection
    auto mark = [&](int stage, bool begin) -> cudaError_t {
        if (!h->profile) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        if (begin) h->ev[stage].push_back({e, nullptr});
        else h->ev[stage].back().second = e;
        return cudaEventRecord(e, s);
    };
    // Screened probe: the BF16 GEMM walks the centroids in chunks, each
    // making the walked prefix eight times longer, and keeps per query only
    // the lists whose screened score can still reach its np-th (the band
    // merge of the batched k-NN, kernels_knn.cu); probe_final rescores the
    // band exactly. Same lists and distances as probe_select_band on the
    // full score matrix.
    const bool screened = h->tc && h->nlist >= SCREEN_MIN_LISTS;
    const int lcap = std::max(1024, 2 * np_max);
    const bool lms = lms_use(h, chunk, np_max);
    // The list scan and the rerank of queries [q0, q0 + nc) whose probe lists
    // are ready: the list-major tensor-core scan, then the table scan for the
    // queries it leaves (brute-force fallbacks and overflowing bands); or the
    // table scan alone (qorder: the L2-friendly block order).
    // Parity mode with FP16 tables: the rerank proves each query's top k
    // from the scan's cut and lists the queries it cannot prove, which are
    // scanned and reranked again with FP32 tables.
    const bool check = mode == 0 && p.adc_table && p.scanc && scan_adc_supported(h->o.num_subquantizers);
    auto scan_rerank = [&](int64_t q0, int64_t nc, const float* qp, const int32_t* qorder) -> int {
        p.kq = d_k + q0;
        ScanParams pt = p;  // the table scan: every query, or those the list-major scan leaves
        pt.qorder = qorder;
        pt.qcount = nullptr;
        unsigned long long* rows = h->profile ? h->s_rows.p : nullptr;
        CK(mark(2, true));
        if (lms && nc >= h->lms.min_queries) {
            const int lrc = run_lms(h, sc, qp, nc, d_k + q0, d_np + q0, np_max, kmax, mode, R, s);
            if (lrc) return lrc;
            CK(mark(2, false));
            CK(mark(3, true));
            ScanParams pl = p;
            pl.qorder = nullptr;
            CK(launch_rerank(pl, qp, nc, sc.cand_row.p, sc.cand_seq.p, R, d_k + q0, kmax, mode, d_ids + q0 * kmax,
                             d_dist + q0 * kmax, d_nout + q0, s));
            pt.qorder = sc.lredo.p;
            pt.qcount = sc.lredo.p + nc;
            rows = nullptr;
            h->launches += 1;
        }
        if (check) {
            pt.scan_cut = sc.scut.p;
            pt.scan_eps = sc.seps.p;
            pt.redo = sc.credo.p;
            pt.redo_count = sc.credo.p + nc;
            CK(cudaMemsetAsync(sc.credo.p + nc, 0, sizeof(int32_t), s));
        }
        CK(launch_scan(pt, qp, nc, sc.probe_ids.p, sc.probe_d.p, d_np + q0, np_max, sc.fb.p, R, sc.cand_row.p,
                       sc.cand_d.p, sc.cand_seq.p, rows, s));
        if (!pt.qcount) {
            CK(mark(2, false));
            CK(mark(3, true));
        }
        CK(launch_rerank(pt, qp, nc, sc.cand_row.p, sc.cand_seq.p, R, d_k + q0, kmax, mode, d_ids + q0 * kmax,
                         d_dist + q0 * kmax, d_nout + q0, s));
        h->launches += scan_launches + 1;
        if (check) {
            ScanParams pf = p;
            pf.adc_table = 0;
            pf.qorder = sc.credo.p;
            pf.qcount = sc.credo.p + nc;
            CK(launch_scan(pf, qp, nc, sc.probe_ids.p, sc.probe_d.p, d_np + q0, np_max, sc.fb.p, R, sc.cand_row.p,
                           sc.cand_d.p, sc.cand_seq.p, nullptr, s));
            CK(launch_rerank(pf, qp, nc, sc.cand_row.p, sc.cand_seq.p, R, d_k + q0, kmax, mode, d_ids + q0 * kmax,
                             d_dist + q0 * kmax, d_nout + q0, s));
            h->launches += scan_launches + 1;
        }
        CK(mark(3, false));
        return HANN_OK;
    };
    for (int64_t q0 = 0; q0 < nq; q0 += chunk) {
        const int64_t nc = std::min(chunk, nq - q0);
        const float* qp = d_q + q0 * h->o.dimension;
        if (screened) {
            CK(mark(0, true));
            CK(launch_to_bf16(qp, nc, h->o.dimension, h->kp, sc.qbf.p, sc.qn2.p, sc.qres.p, s));
            CK(launch_knn_query_band(sc.qn2.p, sc.qres.p, nc, h->kp, 0,
                                     reinterpret_cast<const unsigned int*>(h->d_cmax.p), sc.pe2.p, sc.pasl.p, s));
            CK(cudaMemsetAsync(sc.pcnt.p, 0, sizeof(int32_t) * nc, s));
            CK(cudaMemsetAsync(sc.plcount.p, 0, sizeof(int32_t) * nc, s));
            CK(cudaMemsetAsync(sc.pneed.p, 0, sizeof(int32_t) * nc, s));
            CK(launch_fill_f32(sc.pthr.p, nc, INFINITY, s));
            int launches = 3;
            const int first = std::min(h->nlist,
                                       std::min(PROBE_CAP, std::max(PROBE_FIRST, (int)round_up(2 * (int64_t)np_max, 256))));
            for (int b = 0, w = first; b < h->nlist; w = 7 * b) {
                const int e = std::min(h->nlist, b + w);
                CK(launch_gemm_filter(sc.qbf.p, nc, h->d_coarse_bf16.p, h->nlist, h->kp, b, e,
                                      h->d_coarse_terms.p, 0, sc.pthr.p, PROBE_CAP, sc.pcnt.p, sc.pcand_id.p,
                                      sc.pcand_s.p, h->d_err.p, s, b == 0));
                CK(launch_knn_merge_band((int)nc, np_max, d_np + q0, PROBE_CAP, lcap, sc.pcnt.p, sc.pcand_id.p,
                                         sc.pcand_s.p, sc.pe2.p, sc.pasl.p, sc.pband.p, sc.plcount.p, sc.pthr.p,
                                         sc.pneed.p, sc.ptodo.p, s));
                launches += 3;  // the filter GEMM, the warp merge and the block merge
                b = e;
            }
            CK(mark(0, false));
            CK(mark(1, true));
            CK(launch_probe_final(qp, nc, h->o.dimension, h->d_coarse.p, h->nlist, d_np + q0, np_max, d_k + q0,
                                  h->d_live.p, h->o.fallback ? 1 : 0, lcap, sc.pband.p, sc.plcount.p, sc.pneed.p,
                                  sc.D.p, sc.probe_ids.p, sc.probe_d.p, sc.fb.p, fbc, sc.ptodo.p, s));
            CK(launch_probe_order(sc.probe_ids.p, nc, np_max, h->nlist, sc.order_scratch.p, sc.qorder.p, s));
            CK(mark(1, false));
            const int rc = scan_rerank(q0, nc, qp, sc.qorder.p);
            if (rc) return rc;
            h->launches += launches + 5;  // + probe final (2), query order (3)
            continue;
        }
        CK(mark(0, true));
        if (h->tc) {
            CK(launch_to_bf16(qp, nc, h->o.dimension, h->kp, sc.qbf.p, sc.qn2.p, sc.qres.p, s));
            CK(launch_gemm_scores(sc.qbf.p, nc, h->d_coarse_bf16.p, h->nlist, h->kp, h->d_coarse_norm.p, sc.D.p,
                                  h->d_err.p, s));
        } else {
            CK(launch_dist_matrix(qp, nc, h->o.dimension, h->d_coarse.p, h->nlist, sc.D.p, s));
        }
        CK(mark(0, false));
        CK(mark(1, true));
        if (h->tc) {
            CK(launch_probe_select_band(sc.D.p, qp, sc.qn2.p, sc.qres.p, nc, h->o.dimension, h->kp, h->d_coarse.p,
                                        h->d_cmax.p,
                                        h->nlist, d_np + q0, np_max, d_k + q0, h->d_live.p, h->o.fallback ? 1 : 0,
                                        sc.probe_ids.p, sc.probe_d.p, sc.fb.p, fbc, s));
        } else {
            CK(launch_probe_select(sc.D.p, nc, h->nlist, d_np + q0, np_max, d_k + q0, h->d_live.p,
                                   h->o.fallback ? 1 : 0, sc.probe_ids.p, sc.probe_d.p, sc.fb.p, fbc, s));
        }
        CK(mark(1, false));
        const int rc = scan_rerank(q0, nc, qp, nullptr);
        if (rc) return rc;
        h->launches += h->tc ? 3 : 2;
    }
    return HANN_OK;
}

int check_searchable(hann_pqivf* h) {
    if (!h->trained)
        return h->fail(HANN_E_STATE, "PQIVF index is not trained. Call Train() after adding data before searching");
    bool any = false;
    for (uint8_t b : h->list_key) any |= b != 0;
    if (!any) return h->fail(HANN_E_STATE, "index is empty");
    return HANN_OK;
}

static int read_fallbacks(hann_pqivf* h, SearchScratch& sc, cudaStream_t s) {
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, sc.fbcount.p, sizeof(v), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->fallback_searches += (int64_t)v;
    return HANN_OK;
}

// ---------------------------------------------------------------------------
// C ABI.

extern "C" {

void hann_pqivf_options_init(hann_pqivf_options* o, int32_t dimension) {
    std::memset(o, 0, sizeof(*o));
    o->dimension = dimension;
    o->coarse_k = 16;
    o->pq_k = 16;
    o->kmeans_iters = 10;
    o->candidate_clusters = 3;
    o->fallback = 1;
    o->seed = 0x68616e6eull;
    o->device = 0;
    o->rerank = 0;
    int m = 1;
    for (int c : {8, 4, 2})
        if (dimension > 0 && dimension % c == 0) {
            m = c;
            break;
        }
    o->num_subquantizers = m;
}

int hann_pqivf_new(const hann_pqivf_options* opts, hann_pqivf** out) {
    char buf[256];
    auto bad = [&](int code) {
        hann_thread_error() = buf;
        return code;
    };
    if (!opts || !out) {
        snprintf(buf, sizeof(buf), "null argument");
        return bad(HANN_E_INVALID);
    }
    const hann_pqivf_options& o = *opts;
    if (o.dimension <= 0) {
        snprintf(buf, sizeof(buf), "dimension (%d) must be positive", o.dimension);
        return bad(HANN_E_INVALID);
    }
    if (o.coarse_k <= 0) {
        snprintf(buf, sizeof(buf), "coarseK (%d) must be positive", o.coarse_k);
        return bad(HANN_E_INVALID);
    }
    if (o.pq_k <= 0) {
        snprintf(buf, sizeof(buf), "pqK (%d) must be positive", o.pq_k);
        return bad(HANN_E_INVALID);
    }
    if (o.kmeans_iters <= 0) {
        snprintf(buf, sizeof(buf), "kMeansIters (%d) must be positive", o.kmeans_iters);
        return bad(HANN_E_INVALID);
    }
    if (o.num_subquantizers <= 0) {
        snprintf(buf, sizeof(buf), "numSubquantizers (%d) must be positive", o.num_subquantizers);
        return bad(HANN_E_INVALID);
    }
    if (o.dimension % o.num_subquantizers != 0) {
        snprintf(buf, sizeof(buf), "dimension (%d) must be divisible by numSubquantizers (%d)", o.dimension,
                 o.num_subquantizers);
        return bad(HANN_E_INVALID);
    }
    if (o.pq_k > 256) {
        snprintf(buf, sizeof(buf), "pqK (%d) above 256: this build stores one-byte codes", o.pq_k);
        return bad(HANN_E_UNSUPPORTED);
    }
    hann_pqivf* h = new (std::nothrow) hann_pqivf();
    if (!h) {
        snprintf(buf, sizeof(buf), "out of host memory");
        return bad(HANN_E_NOMEM);
    }
    h->o = o;
    h->dsub = o.dimension / o.num_subquantizers;
    h->code_stride = (int)round_up(o.num_subquantizers, 4);
    h->rng.seed(o.seed);
    cudaError_t e = cudaSetDevice(o.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = h->main.fbcount.reserve(1);
    if (e == cudaSuccess) e = h->s_rows.reserve(2);
    if (e == cudaSuccess) e = cudaMemset(h->s_rows.p, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = h->d_fb_dev.reserve(1);
    if (e == cudaSuccess) e = cudaMemset(h->d_fb_dev.p, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = h->d_adc_redo.reserve(1);
    if (e == cudaSuccess) e = cudaMemset(h->d_adc_redo.p, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->dev_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        snprintf(buf, sizeof(buf), "CUDA initialisation failed: %s", cudaGetErrorString(e));
        delete h;
        return bad(HANN_E_CUDA);
    }
    *out = h;
    return HANN_OK;
}

void hann_pqivf_free(hann_pqivf* h) {
    if (!h) return;
    cudaSetDevice(h->o.device);
    wait_device_searches(h);
    if (h->dev_ev) cudaEventDestroy(h->dev_ev);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    delete h;
}

const char* hann_pqivf_last_error(const hann_pqivf*) { return hann_thread_error().c_str(); }

int hann_pqivf_bulk_add(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && (!ids || !vectors))) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    return bulk_add_locked(h, ids, vectors, n);
}

}  // extern "C"

int bulk_add_locked(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n, bool allow_relayout,
                    bool* needs_relayout) {
    if (needs_relayout) *needs_relayout = false;
    const int dim = h->o.dimension;
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    if (!std::is_sorted(ids, ids + n))
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
    // First failing position in ascending id order; everything before it is
    // applied, as the reference's loop does (pqivf/index.go:276-296).
    int64_t f = n;
    int code = HANN_OK;
    std::string msg;
    for (int64_t i = 0; i < n; i++) {
        const int64_t id = ids[order[i]];
        const bool dup_prev = i > 0 && ids[order[i - 1]] == id;
        if (h->id_cluster.count(id) || (dup_prev && h->trained)) {
            f = i;
            code = HANN_E_EXISTS;
            msg = "id " + std::to_string(id) + " already exists in a cluster";
            break;
        }
        if (h->pending.count(id) || dup_prev) {
            f = i;
            code = HANN_E_EXISTS;
            msg = "id " + std::to_string(id) + " already exists in pending vectors";
            break;
        }
    }
    if (!h->trained) {
        h->pending.reserve_more((size_t)f, dim);
        for (int64_t i = 0; i < f; i++) {
            const int64_t r = order[i];
            h->pending.put(ids[r], vectors + r * dim, dim);
        }
    } else if (f > 0) {
        std::vector<int64_t> sid(f);
        std::vector<float> sv((size_t)f * dim);
        for (int64_t i = 0; i < f; i++) {
            sid[i] = ids[order[i]];
            std::memcpy(&sv[(size_t)i * dim], vectors + order[i] * dim, sizeof(float) * dim);
        }
        // A call that stopped for a relayout left these same rows prepared
        // (nothing else changes the index before the caller comes back).
        MutationScratch& m = h->mut;
        int rc = HANN_OK;
        if (!(allow_relayout && m.held && m.held_ids == sid)) {
            rc = add_prepare(h, sid.data(), sv.data(), f);
            if (rc) return rc;
        }
        m.held = false;
        if (m.grow && !allow_relayout) {
            m.held = true;
            m.held_ids = sid;
            if (needs_relayout) *needs_relayout = true;
            return HANN_OK;
        }
        rc = add_commit(h, sid.data());
        if (rc) return rc;
    }
    if (code) return h->fail(code, "%s", msg.c_str());
    return HANN_OK;
}

extern "C" {

int hann_pqivf_add(hann_pqivf* h, int64_t id, const float* vector) { return hann_pqivf_bulk_add(h, &id, vector, 1); }

// Deletes in the given order; `strict` stops at the first unknown id.
static int delete_ids(hann_pqivf* h, std::vector<int64_t> ids, bool strict) {
    std::vector<int64_t> trained_side;
    std::unordered_set<int64_t> seen;
    for (int64_t id : ids) {
        if (h->pending.erase(id)) continue;
        if (!h->id_cluster.count(id) || seen.count(id)) {
            if (strict) {
                int rc = remove_rows(h, trained_side);
                if (rc) return rc;
                return h->fail(HANN_E_NOT_FOUND, "id %lld not found", (long long)id);
            }
            continue;
        }
        seen.insert(id);
        trained_side.push_back(id);
    }
    return remove_rows(h, trained_side);
}

int hann_pqivf_delete(hann_pqivf* h, int64_t id) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    return delete_ids(h, {id}, true);
}

int hann_pqivf_bulk_delete(hann_pqivf* h, const int64_t* ids, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && !ids)) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    return bulk_delete_locked(h, ids, n);
}

}  // extern "C"

int bulk_delete_locked(hann_pqivf* h, const int64_t* ids, int64_t n, bool allow_relayout, bool* needs_relayout) {
    if (needs_relayout) *needs_relayout = false;
    std::vector<int64_t> v(ids, ids + n);
    std::sort(v.begin(), v.end());
    if (!allow_relayout) {
        std::unordered_set<int64_t> live;
        for (int64_t id : v)
            if (h->id_cluster.count(id)) live.insert(id);
        if (compaction_due(h, (int64_t)live.size())) {
            if (needs_relayout) *needs_relayout = true;
            return HANN_OK;
        }
    }
    return delete_ids(h, v, false);
}

extern "C" {

int hann_pqivf_bulk_update(hann_pqivf* h, const int64_t* ids, const float* vectors, int64_t n) {
    if (!h) return HANN_E_INVALID;
    if (n < 0 || (n > 0 && (!ids || !vectors))) return h->fail(HANN_E_INVALID, "invalid arguments");
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    const int dim = h->o.dimension;
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    if (!std::is_sorted(ids, ids + n))
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
    // Delete-then-add per id in ascending order; the first id that is not
    // present stops the batch (pqivf/index.go:435-442).
    int64_t f = n;
    for (int64_t i = 0; i < n; i++) {
        const int64_t id = ids[order[i]];
        const bool present = h->pending.count(id) || h->id_cluster.count(id);
        const bool dup_prev = i > 0 && ids[order[i - 1]] == id;
        if (!present && !dup_prev) {
            f = i;
            break;
        }
    }
    // Apply the updates before f. A repeated id updates twice, the last wins.
    std::vector<int64_t> del;
    for (int64_t i = 0; i < f; i++) del.push_back(ids[order[i]]);
    std::vector<int64_t> last_pos;
    for (int64_t i = 0; i < f; i++)
        if (i + 1 == f || ids[order[i + 1]] != ids[order[i]]) last_pos.push_back(order[i]);
    int rc = delete_ids(h, del, false);
    if (rc) return rc;
    if (!h->trained) {
        for (int64_t r : last_pos) h->pending.put(ids[r], vectors + r * dim, dim);
    } else if (!last_pos.empty()) {
        std::vector<int64_t> sid;
        std::vector<float> sv;
        for (int64_t r : last_pos) {
            sid.push_back(ids[r]);
            sv.insert(sv.end(), vectors + r * dim, vectors + (r + 1) * dim);
        }
        rc = assign_batch(h, sid.data(), sv.data(), (int64_t)sid.size());
        if (rc) return rc;
    }
    if (f < n) return h->fail(HANN_E_NOT_FOUND, "id %lld not found", (long long)ids[order[f]]);
    return HANN_OK;
}

int hann_pqivf_update(hann_pqivf* h, int64_t id, const float* vector) {
    return hann_pqivf_bulk_update(h, &id, vector, 1);
}

int hann_pqivf_train_seeded(hann_pqivf* h, const int64_t* coarse_init, const int64_t* pq_init, const int64_t* reseed,
                            int64_t n_reseed) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    SeedSource s;
    s.coarse_init = coarse_init;
    s.pq_init = pq_init;
    s.reseed = reseed;
    s.n_reseed = n_reseed;
    return train_impl(h, s);
}

int hann_pqivf_train(hann_pqivf* h) { return hann_pqivf_train_seeded(h, nullptr, nullptr, nullptr, 0); }

int hann_pqivf_retrain(hann_pqivf* h, int32_t iters) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    if (iters < 0) return h->fail(HANN_E_INVALID, "retrain iterations must not be negative");
    if (!h->trained || h->nlist == 0)
        return h->fail(HANN_E_STATE, "PQIVF index is not trained. Call Train() before Retrain()");
    SeedSource s;
    s.warm_coarse = h->d_coarse.p;
    s.warm_codebooks = h->d_codebooks.p;
    s.warm_iters = iters;
    return train_impl(h, s);
}

int hann_pqivf_search_batch(hann_pqivf* h, const float* queries, int64_t nq, const int32_t* k, const int32_t* nprobe,
                            int32_t kmax, int32_t mode, int64_t* ids, double* distances, int32_t* n_out) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (nq < 0 || (nq > 0 && (!queries || !k || !ids || !distances || !n_out)))
        return h->fail(HANN_E_INVALID, "invalid arguments");
    for (int64_t i = 0; i < nq; i++)
        if (k[i] <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    for (int64_t i = 0; i < nq; i++)
        if (k[i] > kmax) return h->fail(HANN_E_INVALID, "k (%d) above kmax (%d)", k[i], kmax);
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq == 0) return HANN_OK;
    std::vector<int32_t> np(nq);
    int np_max = 1;
    for (int64_t i = 0; i < nq; i++) {
        np[i] = nprobe ? nprobe[i] : h->o.candidate_clusters;
        if (np[i] <= 0) return h->fail(HANN_E_INVALID, "nprobe must be positive");
        np[i] = std::min(np[i], h->nlist);
        np_max = std::max(np_max, np[i]);
    }
    cudaStream_t s = h->stream;
    SearchScratch& sc = h->main;
    CK(upload(sc.q, queries, (size_t)nq * h->o.dimension, s));
    CK(upload(sc.k, k, (size_t)nq, s));
    CK(upload(sc.np, np.data(), (size_t)nq, s));
    CK(sc.ids.reserve((size_t)nq * kmax));
    CK(sc.dist.reserve((size_t)nq * kmax));
    CK(sc.nout.reserve((size_t)nq));
    CK(sc.fbcount.reserve(1));
    CK(cudaMemsetAsync(sc.fbcount.p, 0, sizeof(unsigned long long), s));
    rc = run_search(h, sc, sc.q.p, nq, sc.k.p, sc.np.p, np_max, kmax, mode, sc.ids.p, sc.dist.p, sc.nout.p, s);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ids, sc.ids.p, (size_t)nq * kmax * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(distances, sc.dist.p, (size_t)nq * kmax * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(n_out, sc.nout.p, (size_t)nq * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    return read_fallbacks(h, sc, s);
}

int hann_pqivf_search(hann_pqivf* h, const float* query, int32_t k, int64_t* ids, double* distances,
                      int32_t* n_out) {
    if (!h) return HANN_E_INVALID;
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    return hann_pqivf_search_batch(h, query, 1, &k, nullptr, k, 0, ids, distances, n_out);
}

int hann_pqivf_search_batch_device(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k, int32_t nprobe,
                                   int32_t mode, int64_t* d_ids, double* d_distances, int32_t* d_n_out,
                                   void* stream) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (nprobe <= 0) nprobe = h->o.candidate_clusters;
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq <= 0) return HANN_OK;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const int np = std::min<int>(nprobe, h->nlist);
    SearchScratch& sc = h->main;
    // k and nprobe filled on the device: the call enqueues everything on s
    // and returns without waiting, so back-to-back calls keep the GPU busy
    CK(sc.k.reserve((size_t)nq));
    CK(sc.np.reserve((size_t)nq));
    CK(sc.fbcount.reserve(1));
    CK(launch_fill_i32(sc.k.p, nq, k, s));
    CK(launch_fill_i32(sc.np.p, nq, np, s));
    h->launches += 2;
    rc = run_search(h, sc, d_queries, nq, sc.k.p, sc.np.p, np, k, mode, d_ids, d_distances, d_n_out, s,
                    h->d_fb_dev.p);
    if (rc) return rc;
    CK(note_device_search(h, s));
    return HANN_OK;
}

int hann_pqivf_arena_stats(void* hv, int64_t* out) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    out[0] = h->rows_cap;
    out[1] = h->arena_end;
    out[2] = h->hole_rows;
    out[3] = h->list_moves;
    out[4] = h->full_relayouts;
    return HANN_OK;
}

int hann_pqivf_set_candidate_clusters(hann_pqivf* h, int32_t n) {
    if (!h) return HANN_E_INVALID;
    if (n <= 0) return h->fail(HANN_E_INVALID, "candidate clusters must be positive");
    std::unique_lock<std::mutex> w(h->wmu);
    std::unique_lock<std::shared_mutex> g(h->mu);
    h->o.candidate_clusters = n;
    return HANN_OK;
}

int hann_pqivf_set_adc_tables(hann_pqivf* h, int32_t kind) {
    if (!h) return HANN_E_INVALID;
    if (kind < HANN_ADC_FP32 || kind > HANN_ADC_FIXED16) return h->fail(HANN_E_INVALID, "unknown lookup-table kind %d", kind);
    std::unique_lock<std::mutex> w(h->wmu);
    std::unique_lock<std::shared_mutex> g(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    h->adc_table = kind;
    return HANN_OK;
}

int hann_pqivf_set_plain_fp32(hann_pqivf* h, int32_t on) {
    if (!h) return HANN_E_INVALID;
    std::unique_lock<std::mutex> w(h->wmu);
    std::unique_lock<std::shared_mutex> g(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    h->o.plain_fp32 = on ? 1 : 0;
    if (!h->trained) return HANN_OK;
    return prepare_coarse(h);
}

int hann_pqivf_set_profiling(hann_pqivf* h, int32_t on) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> rl(h->run_mu);
    h->profile = on != 0;
    return HANN_OK;
}

int hann_pqivf_stage_times(hann_pqivf* h, double* ms4, int64_t* launches, int64_t* rows_scanned) {
    if (!h) return HANN_E_INVALID;
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    for (int st = 0; st < 4; st++) {
        double tot = 0.0;
        for (auto& pr : h->ev[st]) {
            if (pr.second) {
                CK(cudaEventSynchronize(pr.second));
                float ms = 0.0f;
                CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
                tot += ms;
                cudaEventDestroy(pr.second);
            }
            cudaEventDestroy(pr.first);
        }
        h->ev[st].clear();
        if (ms4) ms4[st] = tot;
    }
    const int64_t nl = h->launches.exchange(0);
    if (launches) *launches = nl;
    unsigned long long rows[2] = {0, 0};
    CK(cudaMemcpy(rows, h->s_rows.p, sizeof(rows), cudaMemcpyDeviceToHost));
    CK(cudaMemset(h->s_rows.p, 0, sizeof(rows)));
    if (rows_scanned) *rows_scanned = (int64_t)rows[0];
    h->rows_decoded = (int64_t)rows[1];
    return HANN_OK;
}

int hann_pqivf_autotune_scan(hann_pqivf* h, const float* queries, int64_t nq, int32_t k, int32_t mode,
                             int32_t* chosen8, double* ms_table, double* ms_list) {
    if (!h) return HANN_E_INVALID;
    if (nq <= 0 || !queries) return h->fail(HANN_E_INVALID, "invalid arguments");
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    int rc = check_searchable(h);
    if (rc) return rc;
    cudaStream_t s = h->stream;
    DBuf<float> dq;
    DBuf<int32_t> dk, dnp, dn;
    DBuf<int64_t> di;
    DBuf<double> dd;
    CK(upload(dq, queries, (size_t)nq * h->o.dimension, s));
    CK(dk.reserve((size_t)nq));
    CK(dnp.reserve((size_t)nq));
    CK(dn.reserve((size_t)nq));
    CK(di.reserve((size_t)nq * k));
    CK(dd.reserve((size_t)nq * k));
    CK(launch_fill_i32(dk.p, nq, k, s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const LmsConfig saved = h->lms;
    // the median of three timed runs after a warm one, in ms
    auto time_search = [&](int np) -> double {
        if (launch_fill_i32(dnp.p, nq, np, s) != cudaSuccess) return -1.0;
        float best[3] = {0, 0, 0};
        for (int r = 0; r < 4; r++) {
            if (cudaEventRecord(e0, s) != cudaSuccess) return -1.0;
            if (run_search(h, h->main, dq.p, nq, dk.p, dnp.p, np, k, mode, di.p, dd.p, dn.p, s) != HANN_OK)
                return -1.0;
            if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return -1.0;
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) best[r - 1] = ms;
        }
        std::sort(best, best + 3);
        return best[1];
    };
    // list-major candidates: chunk growth and the rows of a list per work item
    // (the list-split threshold); the first chunk takes each query's nearest list
    const int grid[][3] = {{1, 32, 512}, {1, 8, 512}, {1, 32, 1024}, {1, 8, 256}};
    const int ngrid = (int)(sizeof(grid) / sizeof(grid[0]));
    const int ladder[] = {8, 16, 32, 64, 128, 256};
    const int nl = (int)(sizeof(ladder) / sizeof(ladder[0]));
    double tab[6], lm[6][4];
    int used = 0;
    bool fail = false;
    for (int i = 0; i < nl && !fail; i++) {
        const int np = std::min(ladder[i], h->nlist);
        if (i > 0 && np == std::min(ladder[i - 1], h->nlist)) break;
        used = i + 1;
        h->lms = saved;
        h->lms.enabled = 0;
        tab[i] = time_search(np);
        for (int g = 0; g < ngrid; g++) {
            h->lms = saved;
            h->lms.enabled = h->lms_ok ? 1 : 0;
            h->lms.min_nprobe = 1;
            h->lms.min_queries = 1;
            h->lms.seed = 0;
            h->lms.first = grid[g][0];
            h->lms.growth = grid[g][1];
            h->lms.rows_max = grid[g][2];
            lm[i][g] = h->lms_ok ? time_search(np) : 1e30;
        }
        fail = tab[i] < 0.0;
        for (int g = 0; g < ngrid; g++) fail |= lm[i][g] < 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->lms = saved;
    if (fail) return h->fail(HANN_E_CUDA, "a tuning search failed");
    // the list-major form with the smallest total over the ladder, then the
    // crossover: the smallest ladder value from which it is faster at every
    // larger value
    int bg = 0;
    double bsum = 1e300;
    for (int g = 0; g < ngrid; g++) {
        double sum = 0.0;
        for (int i = 0; i < used; i++) sum += lm[i][g];
        if (sum < bsum) {
            bsum = sum;
            bg = g;
        }
    }
    int cross = h->nlist + 1;  // never
    for (int i = used - 1; i >= 0; i--) {
        if (lm[i][bg] < tab[i]) cross = std::min(ladder[i], h->nlist);
        else break;
    }
    h->lms.enabled = h->lms_ok ? 1 : 0;
    h->lms.min_queries = 1;
    h->lms.seed = 0;
    h->lms.first = grid[bg][0];
    h->lms.growth = grid[bg][1];
    h->lms.rows_max = grid[bg][2];
    h->lms.min_nprobe = cross;
    if (chosen8) {
        chosen8[0] = h->lms.enabled;
        chosen8[1] = h->lms.min_queries;
        chosen8[2] = h->lms.first;
        chosen8[3] = h->lms.growth;
        chosen8[4] = h->lms.rows_max;
        chosen8[5] = h->lms.ctas_per_sm;
        chosen8[6] = h->lms.seed;
        chosen8[7] = h->lms.min_nprobe;
    }
    for (int i = 0; i < nl; i++) {
        if (ms_table) ms_table[i] = i < used ? tab[i] : -1.0;
        if (ms_list) ms_list[i] = i < used ? lm[i][bg] : -1.0;
    }
    return HANN_OK;
}

int hann_pqivf_rows_decoded(void* hv, int64_t* out) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h || !out) return HANN_E_INVALID;
    std::lock_guard<std::mutex> rl(h->run_mu);
    *out = h->rows_decoded;
    return HANN_OK;
}

int hann_pqivf_train_stats(void* hv, int64_t* out2) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h || !out2) return HANN_E_INVALID;
    std::unique_lock<std::mutex> w(h->wmu);
    out2[0] = h->warm_assignments;
    out2[1] = h->warm_overflow_rows;
    return HANN_OK;
}

int hann_pqivf_train_phases(void* hv, double* out4) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h || !out4) return HANN_E_INVALID;
    std::unique_lock<std::mutex> w(h->wmu);
    for (int i = 0; i < 4; i++) out4[i] = h->train_phase_ms[i];
    return HANN_OK;
}

int hann_pqivf_adc_redos(void* hv, int64_t* out) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h || !out) return HANN_E_INVALID;
    std::unique_lock<std::mutex> w(h->wmu);
    std::unique_lock<std::shared_mutex> g(h->mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, h->d_adc_redo.p, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *out = (int64_t)v;
    return HANN_OK;
}

int hann_pqivf_scan_options(void* hv, const int32_t* set8, int32_t* get8) {
    hann_pqivf* h = static_cast<hann_pqivf*>(hv);
    if (!h) return HANN_E_INVALID;
    std::unique_lock<std::mutex> w(h->wmu);
    std::unique_lock<std::shared_mutex> g(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    if (set8) {
        const int32_t* set7 = set8;
        if (set7[1] < 1 || set7[2] < 1 || set7[3] < 2 || set7[4] < 1 || set7[5] < 1 || set7[5] > 2 || set8[7] < 1)
            return h->fail(HANN_E_INVALID, "invalid list-scan options");
        h->lms.min_nprobe = set8[7];
        h->lms.enabled = set7[0] ? 1 : 0;
        h->lms.min_queries = set7[1];
        h->lms.first = set7[2];
        h->lms.growth = set7[3];
        h->lms.rows_max = set7[4];
        h->lms.ctas_per_sm = set7[5];
        h->lms.seed = set7[6] ? 1 : 0;
    }
    if (get8) {
        int32_t* get7 = get8;
        get8[7] = h->lms.min_nprobe;
        get7[0] = h->lms.enabled;
        get7[1] = h->lms.min_queries;
        get7[2] = h->lms.first;
        get7[3] = h->lms.growth;
        get7[4] = h->lms.rows_max;
        get7[5] = h->lms.ctas_per_sm;
        get7[6] = h->lms.seed;
    }
    return HANN_OK;
}

int hann_pqivf_list_lengths(hann_pqivf* h, int64_t* out, int32_t capacity, int32_t* n_out) {
    if (!h || !n_out || (capacity > 0 && !out)) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    *n_out = h->nlist;
    if (h->nlist > capacity)
        return h->fail(HANN_E_CHANGED, "the index has %d lists, the buffer holds %d", h->nlist, (int)capacity);
    for (int l = 0; l < h->nlist; l++) out[l] = h->live_count[l];
    return HANN_OK;
}

int hann_pqivf_stats(hann_pqivf* h, hann_pqivf_index_stats* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    // Fallbacks of device-buffer searches are counted on the device: wait for
    // those enqueued so far, then add the device count.
    unsigned long long dev_fb = 0;
    {
        std::lock_guard<std::mutex> rl(h->run_mu);
        cudaSetDevice(h->o.device);
        CK(wait_device_searches(h));
        CK(cudaMemcpyAsync(&dev_fb, h->d_fb_dev.p, sizeof(dev_fb), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    out->count = (int64_t)h->pending.size() + h->total_rows();
    out->dimension = h->o.dimension;
    out->fallback_searches = h->fallback_searches.load() + (int64_t)dev_fb;
    out->trained = h->trained ? 1 : 0;
    out->nlist = h->nlist;
    out->rows_capacity = h->rows_cap;
    return HANN_OK;
}

int hann_pqivf_tune_candidate_clusters(hann_pqivf* h, const float* queries, int64_t nq, int32_t k,
                                       double target_recall, const int32_t* ladder, int32_t n_ladder, int32_t mode,
                                       const int64_t* ground_truth, int32_t apply, int32_t* chosen,
                                       int32_t* tried_out, double* recall_out, int32_t* n_tried) {
    if (!h) return HANN_E_INVALID;
    if (nq <= 0 || !queries || !chosen) return h->fail(HANN_E_INVALID, "invalid arguments");
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    if (ladder && n_ladder <= 0) return h->fail(HANN_E_INVALID, "empty nprobe ladder");
    const int dim = h->o.dimension;
    int nlist = 0;
    std::vector<int64_t> gt;
    {
        std::shared_lock<std::shared_mutex> lk(h->mu);
        int rc = check_searchable(h);
        if (rc) return rc;
        nlist = h->nlist;
        if (ground_truth) {
            gt.assign(ground_truth, ground_truth + nq * k);
        } else {
            // Exact k-NN over the stored (live) vectors on the device: gather
            // them into one flat base, then the batched k-NN's tensor-core
            // screen with exact rescoring.
            std::lock_guard<std::mutex> rl(h->run_mu);
            cudaSetDevice(h->o.device);
            std::vector<int64_t> rows, ids;
            for (int l = 0; l < h->nlist; l++)
                for (size_t j = 0; j < h->list_ids[l].size(); j++)
                    if (h->list_alive[l][j]) {
                        rows.push_back(h->h_start[l] + (int64_t)j);
                        ids.push_back(h->list_ids[l][j]);
                    }
            const int64_t n = (int64_t)rows.size();
            DBuf<int64_t> d_rows;
            DBuf<float> base;
            CK(upload(d_rows, rows.data(), rows.size(), h->stream));
            CK(base.reserve((size_t)n * dim));
            CK(launch_copy_words(h->d_vectors.p, d_rows.p, base.p, nullptr, n, dim, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            hann_knn* kh = knn_new_from_device(base.p, n, dim, h->stream);
            if (!kh) return h->fail(HANN_E_CUDA, "could not build the exact k-NN of the stored vectors");
            std::vector<int64_t> r((size_t)nq * k);
            std::vector<double> d((size_t)nq * k);
            rc = hann_knn_search(kh, HANN_METRIC_SQEUCLID, queries, nq, k, HANN_KNN_AUTO, r.data(), d.data());
            std::string msg = rc ? std::string(hann_knn_last_error(kh)) : std::string();
            hann_knn_free(kh);
            if (rc) return h->fail(rc, "exact k-NN for the recall target: %s", msg.c_str());
            gt.resize(r.size());
            for (size_t i = 0; i < r.size(); i++) gt[i] = r[i] >= 0 ? ids[(size_t)r[i]] : -1;
        }
    }
    std::vector<int32_t> lad;
    if (ladder) {
        lad.assign(ladder, ladder + n_ladder);
    } else {
        for (int p = 1; p <= 4096; p *= 2)
            if (p <= nlist) lad.push_back(p);
        if (lad.empty() || lad.back() != std::min(nlist, 4096)) lad.push_back(std::min(nlist, 4096));
    }
    for (int32_t p : lad)
        if (p <= 0) return h->fail(HANN_E_INVALID, "nprobe must be positive");
    int64_t tot = 0;
    for (int64_t v : gt) tot += v >= 0;
    std::vector<int32_t> kk((size_t)nq, k), npv((size_t)nq);
    std::vector<int64_t> ids((size_t)nq * k);
    std::vector<double> dist((size_t)nq * k);
    std::vector<int32_t> nout((size_t)nq);
    int32_t pick = lad.back(), ntried = 0;
    for (size_t li = 0; li < lad.size(); li++) {
        std::fill(npv.begin(), npv.end(), lad[li]);
        int rc = hann_pqivf_search_batch(h, queries, nq, kk.data(), npv.data(), k, mode, ids.data(), dist.data(),
                                         nout.data());
        if (rc) return rc;
        int64_t hits = 0;
        for (int64_t i = 0; i < nq; i++) {
            const int64_t* g = gt.data() + i * k;
            for (int j = 0; j < nout[(size_t)i]; j++) {
                const int64_t id = ids[(size_t)(i * k + j)];
                for (int t = 0; t < k; t++)
                    if (g[t] >= 0 && g[t] == id) {
                        hits++;
                        break;
                    }
            }
        }
        const double rec = tot ? (double)hits / (double)tot : 1.0;
        if (tried_out) tried_out[ntried] = lad[li];
        if (recall_out) recall_out[ntried] = rec;
        ntried++;
        if (rec >= target_recall) {
            pick = lad[li];
            break;
        }
    }
    *chosen = pick;
    if (n_tried) *n_tried = ntried;
    if (apply) return hann_pqivf_set_candidate_clusters(h, pick);
    return HANN_OK;
}

}  // extern "C"

// The handle's layout; the caller holds h->mu.
static void layout_locked(const hann_pqivf* h, hann_pqivf_layout* out) {
    out->dimension = h->o.dimension;
    out->coarse_k = h->o.coarse_k;
    out->num_subquantizers = h->o.num_subquantizers;
    out->pq_k = h->o.pq_k;
    out->kmeans_iters = h->o.kmeans_iters;
    out->candidate_clusters = h->o.candidate_clusters;
    out->fallback = h->o.fallback;
    out->trained = h->trained;
    out->nlist = h->nlist;
    out->pq_k_eff = h->pqk_eff;
    out->n_rows = h->total_rows();
    out->n_pending = (int64_t)h->pending.size();
}

extern "C" {

int hann_pqivf_export_layout(hann_pqivf* h, hann_pqivf_layout* out) {
    if (!h || !out) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    layout_locked(h, out);
    return HANN_OK;
}

int hann_pqivf_export(hann_pqivf* h, const hann_pqivf_layout* layout, float* coarse, float* codebooks,
                      int64_t* list_len, uint8_t* list_key, int64_t* cluster_counts, int64_t* ids, float* vectors,
                      int32_t* codes, int64_t* pending_ids, float* pending_vectors) {
    if (!h || !layout) return HANN_E_INVALID;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    // The arrays were sized from `layout`; a mutation since then would make
    // the copies below overrun them.
    hann_pqivf_layout now;
    layout_locked(h, &now);
    if (now.dimension != layout->dimension || now.num_subquantizers != layout->num_subquantizers ||
        now.nlist != layout->nlist || now.pq_k_eff != layout->pq_k_eff || now.n_rows != layout->n_rows ||
        now.n_pending != layout->n_pending)
        return h->fail(HANN_E_CHANGED, "the index changed since its layout was read; read the layout again");
    cudaSetDevice(h->o.device);
    const int dim = h->o.dimension, M = h->o.num_subquantizers;
    if (h->nlist > 0) {
        std::memcpy(coarse, h->h_coarse.data(), h->h_coarse.size() * sizeof(float));
        std::memcpy(codebooks, h->h_codebooks.data(), h->h_codebooks.size() * sizeof(float));
    }
    int64_t r = 0;
    std::vector<uint8_t> cbuf;
    std::vector<float> vbuf;
    for (int l = 0; l < h->nlist; l++) {
        const int64_t len = (int64_t)h->list_ids[l].size();
        list_len[l] = h->live_count[l];
        list_key[l] = h->list_key[l];
        cluster_counts[l] = h->cluster_counts[l];
        if (len == 0) continue;
        vbuf.resize((size_t)len * dim);
        CK(cudaMemcpy(vbuf.data(), h->d_vectors.p + h->h_start[l] * dim, (size_t)len * dim * sizeof(float),
                      cudaMemcpyDeviceToHost));
        cbuf.resize((size_t)len * h->code_stride);
        CK(cudaMemcpy(cbuf.data(), h->d_codes.p + h->h_start[l] * h->code_stride, cbuf.size(),
                      cudaMemcpyDeviceToHost));
        for (int64_t j = 0; j < len; j++) {
            if (!h->list_alive[l][j]) continue;
            ids[r] = h->list_ids[l][j];
            std::memcpy(vectors + r * dim, &vbuf[(size_t)j * dim], sizeof(float) * dim);
            for (int m = 0; m < M; m++) codes[r * M + m] = cbuf[(size_t)j * h->code_stride + m];
            r++;
        }
    }
    // Pending vectors in ascending id order.
    const std::vector<int64_t> pid = h->pending.sorted_ids();
    for (size_t i = 0; i < pid.size(); i++) {
        pending_ids[i] = pid[i];
        std::memcpy(pending_vectors + i * dim, h->pending.find(pid[i]), sizeof(float) * dim);
    }
    return HANN_OK;
}

int hann_pqivf_import(hann_pqivf* h, const hann_pqivf_layout* L, const float* coarse, const float* codebooks,
                      const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                      const int64_t* ids, const float* vectors, const int32_t* codes, const uint8_t* has_codes,
                      const int64_t* pending_ids, const float* pending_vectors) {
    if (!h || !L) return HANN_E_INVALID;
    std::lock_guard<std::mutex> wl(h->wmu);
    std::unique_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    CK(wait_device_searches(h));
    return import_locked(h, L, coarse, codebooks, list_len, list_key, cluster_counts, ids, vectors, codes, nullptr,
                         has_codes, pending_ids, pending_vectors);
}

}  // extern "C"

// The import behind hann_pqivf_import and the snapshot loader (all locks
// held). Codes come as the reference's ints (codes32, with has_codes) or as
// bytes (codes8, M per row); codes out of range are recomputed from the
// vectors.
int import_locked(hann_pqivf* h, const hann_pqivf_layout* L, const float* coarse, const float* codebooks,
                  const int64_t* list_len, const uint8_t* list_key, const int64_t* cluster_counts,
                  const int64_t* ids, const float* vectors, const int32_t* codes32, const uint8_t* codes8,
                  const uint8_t* has_codes, const int64_t* pending_ids, const float* pending_vectors) {
    h->mut.held = false;
    // GobDecode's parameter checks (pqivf/index.go:1035-1045).
    if (L->dimension <= 0) return h->fail(HANN_E_INVALID, "serialized index has invalid dimension %d", L->dimension);
    if (L->num_subquantizers <= 0 || L->dimension % L->num_subquantizers != 0)
        return h->fail(HANN_E_INVALID, "serialized index has invalid subquantizer count %d for dimension %d",
                       L->num_subquantizers, L->dimension);
    if (L->coarse_k <= 0 || L->pq_k <= 0 || L->kmeans_iters <= 0)
        return h->fail(HANN_E_INVALID,
                       "serialized index has invalid training parameters: coarseK %d, pqK %d, kMeansIters %d",
                       L->coarse_k, L->pq_k, L->kmeans_iters);
    if (L->pq_k_eff > 256 || L->pq_k > 256)
        return h->fail(HANN_E_UNSUPPORTED, "pqK above 256: this build stores one-byte codes");
    if (L->n_rows > 0 && (L->nlist <= 0 || L->pq_k_eff <= 0))
        return h->fail(HANN_E_UNSUPPORTED, "entries without centroids or codebooks");
    h->o.dimension = L->dimension;
    h->o.coarse_k = L->coarse_k;
    h->o.num_subquantizers = L->num_subquantizers;
    h->o.pq_k = L->pq_k;
    h->o.kmeans_iters = L->kmeans_iters;
    if (L->candidate_clusters > 0) h->o.candidate_clusters = L->candidate_clusters;
    h->o.fallback = L->fallback;
    h->dsub = L->dimension / L->num_subquantizers;
    h->code_stride = (int)round_up(L->num_subquantizers, 4);
    const int dim = L->dimension, M = L->num_subquantizers;
    h->trained = L->trained != 0;
    h->pending.clear();
    h->pending.reserve_more((size_t)L->n_pending, dim);
    for (int64_t i = 0; i < L->n_pending; i++) h->pending.put(pending_ids[i], pending_vectors + i * dim, dim);
    h->nlist = L->nlist;
    h->pqk_eff = L->pq_k_eff;
    h->h_coarse.assign(coarse, coarse + (size_t)L->nlist * dim);
    h->h_codebooks.assign(codebooks, codebooks + (size_t)M * L->pq_k_eff * h->dsub);
    h->list_ids.assign(h->nlist, {});
    h->list_alive.assign(h->nlist, {});
    h->live_count.assign(h->nlist, 0);
    h->dead_rows = 0;
    h->list_key.assign(h->nlist, 0);
    h->cluster_counts.assign(h->nlist, 0);
    h->id_cluster.clear();
    h->id_cluster.reserve((size_t)L->n_rows);
    int64_t r = 0;
    for (int l = 0; l < h->nlist; l++) {
        h->list_key[l] = list_key[l];
        h->cluster_counts[l] = cluster_counts[l];
        for (int64_t j = 0; j < list_len[l]; j++, r++) {
            h->list_ids[l].push_back(ids[r]);
            h->id_cluster.set(ids[r], l);
        }
        h->list_alive[l].assign(h->list_ids[l].size(), 1);
        h->live_count[l] = (int64_t)h->list_ids[l].size();
    }
    h->d_vectors.reset();
    h->d_term.reset();
    h->d_row_id.reset();
    h->d_row_cluster.reset();
    h->d_codes.reset();
    h->d_coarse.reset();
    h->d_codebooks.reset();
    h->rows_cap = 0;
    h->h_start.assign(h->nlist, 0);
    h->h_cap.assign(h->nlist, 0);
    if (h->nlist == 0) return HANN_OK;
    CK(upload(h->d_coarse, h->h_coarse.data(), h->h_coarse.size(), h->stream));
    CK(upload(h->d_codebooks, h->h_codebooks.data(), h->h_codebooks.size(), h->stream));
    {
        int prc = prepare_coarse(h);
        if (prc) return prc;
    }
    std::vector<int64_t> caps(h->nlist);
    for (int l = 0; l < h->nlist; l++) caps[l] = list_capacity(list_len[l]);
    int rc = relayout(h, caps, false);
    if (rc) return rc;
    const int64_t n = L->n_rows;
    if (n == 0) return upload_lens(h);
    std::vector<int64_t> dst(n), recode;
    std::vector<int32_t> rcl(n);
    std::vector<uint8_t> cbytes((size_t)n * h->code_stride, 0);
    r = 0;
    for (int l = 0; l < h->nlist; l++)
        for (int64_t j = 0; j < list_len[l]; j++, r++) {
            dst[r] = h->h_start[l] + j;
            rcl[r] = l;
            bool ok = has_codes == nullptr || has_codes[r];
            for (int m = 0; ok && m < M; m++) {
                const int32_t c = codes8 ? (int32_t)codes8[r * M + m] : codes32[r * M + m];
                if (c < 0 || c >= h->pqk_eff) ok = false;
                else cbytes[(size_t)r * h->code_stride + m] = (uint8_t)c;
            }
            if (!ok) recode.push_back(dst[r]);
        }
    DBuf<int64_t> ddst, did;
    DBuf<int32_t> drcl;
    DBuf<float> dvec;
    DBuf<uint8_t> dcodes;
    CK(upload(ddst, dst.data(), dst.size(), h->stream));
    CK(upload(did, ids, (size_t)n, h->stream));
    CK(upload(drcl, rcl.data(), rcl.size(), h->stream));
    CK(upload(dvec, vectors, (size_t)n * dim, h->stream));
    CK(upload(dcodes, cbytes.data(), cbytes.size(), h->stream));
    CK(launch_copy_words(dvec.p, nullptr, h->d_vectors.p, ddst.p, n, dim, h->stream));
    CK(launch_copy_words(did.p, nullptr, h->d_row_id.p, ddst.p, n, 2, h->stream));
    CK(launch_copy_words(drcl.p, nullptr, h->d_row_cluster.p, ddst.p, n, 1, h->stream));
    CK(launch_copy_words(dcodes.p, nullptr, h->d_codes.p, ddst.p, n, h->code_stride / 4, h->stream));
    CK(launch_term(h->d_codes.p, ddst.p, h->d_row_cluster.p, n, dim, h->d_coarse.p, h->d_codebooks.p, M, h->pqk_eff,
                   h->code_stride, h->d_term.p, h->stream));
    if (!recode.empty()) {
        DBuf<int64_t> drec;
        CK(upload(drec, recode.data(), recode.size(), h->stream));
        CK(launch_encode(h->d_vectors.p, drec.p, h->d_row_cluster.p, (int64_t)recode.size(), dim, h->d_coarse.p,
                         h->d_codebooks.p, M, h->pqk_eff, h->d_codes.p, h->code_stride, h->d_term.p, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return upload_lens(h);
}

extern "C" {

int hann_gpu_distance_batch(int32_t metric, const float* query, const float* flat, size_t dim, size_t n,
                            double* out) {
    if (metric < 0 || metric > 3) return HANN_E_INVALID;
    if (n == 0) return HANN_OK;
    if (dim == 0) {
        for (size_t i = 0; i < n; i++) out[i] = 0.0;
        return HANN_OK;
    }
    DBuf<float> dq, dx;
    DBuf<double> dout;
    if (upload(dq, query, dim, nullptr) != cudaSuccess || upload(dx, flat, dim * n, nullptr) != cudaSuccess ||
        dout.reserve(n) != cudaSuccess)
        return HANN_E_CUDA;
    if (launch_distance_rows(metric, dq.p, dx.p, (int)dim, (int64_t)n, dout.p, nullptr) != cudaSuccess)
        return HANN_E_CUDA;
    if (cudaMemcpy(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return HANN_E_CUDA;
    return HANN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batch search.
//
// Some callers cannot allocate device memory at the moment they search: a
// latency-bound serving thread must not stall on the device-wide
// synchronisation that cudaMalloc/cudaFree may imply; code that records its
// launches into a CUDA graph may not call the allocator while the stream is
// being captured; and a process that fixes its device-memory budget at start
// must not grow it per request. hann_pqivf_search_batch_device_noalloc serves
// them. It runs the same kernels as hann_pqivf_search_batch_device, but every
// scratch buffer of the search (coarse distance matrix, probe lists,
// fallback flags, candidates, per-query k and nprobe, the fallback counter)
// is carved out of one fixed device array of NOALLOC_ARENA_BYTES that every
// GPU which loads this library holds until the process exits. The index's
// own arrays were allocated when it was built; the call allocates nothing.

namespace {

constexpr size_t NOALLOC_ARENA_BYTES = (size_t)16 << 20;  // 16 MiB per device
constexpr int NOALLOC_MAX_DEVICES = 64;

// Host code must not take this symbol's address directly: on the host it is
// only a stand-in. The device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_arena[NOALLOC_ARENA_BYTES];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the arena on the current device `dev`, looked up once.
cudaError_t noalloc_arena(int dev, unsigned char** out) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
    return cudaSuccess;
}

__global__ void noalloc_fill_kernel(int32_t* a, int32_t va, int32_t* b, int32_t vb, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        a[i] = va;
        b[i] = vb;
    }
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

extern "C" int hann_pqivf_search_batch_device_noalloc(hann_pqivf* h, const float* d_queries, int64_t nq, int32_t k,
                                                      int32_t nprobe, int32_t mode, int64_t* d_ids,
                                                      double* d_distances, int32_t* d_n_out, void* stream) {
    if (!h) return HANN_E_INVALID;
    std::shared_lock<std::shared_mutex> lk(h->mu);
    std::lock_guard<std::mutex> rl(h->run_mu);
    cudaSetDevice(h->o.device);
    if (k <= 0) return h->fail(HANN_E_INVALID, "k must be positive");
    if (nprobe <= 0) nprobe = h->o.candidate_clusters;
    if (mode != 0 && mode != 1) return h->fail(HANN_E_INVALID, "mode must be 0 or 1");
    int rc = check_searchable(h);
    if (rc) return rc;
    if (nq <= 0) return HANN_OK;
    const int np = std::min<int>(nprobe, h->nlist);
    const int R = rerank_depth(h, k, mode);
    if (R > 480) return h->fail(HANN_E_UNSUPPORTED, "k (%d) above this build's limit of 448", k);
    if (np > 4096) return h->fail(HANN_E_UNSUPPORTED, "more than 4096 probed lists per query");
    // Every query needs at least 4 * nlist bytes of the arena (its row of
    // coarse distances): a larger batch is refused before the sizes below are
    // multiplied out, so a huge nq cannot wrap them past the check.
    const int64_t nq_cap = (int64_t)(NOALLOC_ARENA_BYTES / (sizeof(float) * (size_t)std::max(1, h->nlist)));
    if (nq > nq_cap)
        return h->fail(HANN_E_UNSUPPORTED,
                       "allocation-free search of %lld queries cannot fit its fixed %zu-byte arena (at most %lld "
                       "queries at nlist %d); split the batch",
                       (long long)nq, NOALLOC_ARENA_BYTES, (long long)nq_cap, h->nlist);
    // Scratch layout inside the arena, every region 256-byte aligned.
    const size_t b_D = align256((size_t)nq * h->nlist * sizeof(float));
    const size_t b_pid = align256((size_t)nq * np * sizeof(int32_t));
    const size_t b_pd = align256((size_t)nq * np * sizeof(float));
    const size_t b_q32 = align256((size_t)nq * sizeof(int32_t));
    const size_t b_cr = align256((size_t)nq * R * sizeof(int32_t));
    const size_t b_cd = align256((size_t)nq * R * sizeof(float));
    const size_t b_cs = align256((size_t)nq * R * sizeof(uint32_t));
    const size_t b_redo = align256((size_t)(nq + 1) * sizeof(int32_t));
    const size_t need = b_D + b_pid + b_pd + 5 * b_q32 + b_cr + b_cd + b_cs + b_redo;
    if (need > NOALLOC_ARENA_BYTES)
        return h->fail(HANN_E_UNSUPPORTED,
                       "allocation-free search of %lld queries needs %zu bytes of scratch, above its fixed %zu-byte "
                       "arena; split the batch (at most about %lld queries at nlist %d, nprobe %d, k %d)",
                       (long long)nq, need, NOALLOC_ARENA_BYTES,
                       (long long)(NOALLOC_ARENA_BYTES / (need / nq + 1)), h->nlist, np, k);
    unsigned char* base = nullptr;
    CK(noalloc_arena(h->o.device, &base));
    float* D = reinterpret_cast<float*>(base);
    int32_t* pid = reinterpret_cast<int32_t*>(base + b_D);
    float* pd = reinterpret_cast<float*>(base + b_D + b_pid);
    int32_t* fb = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd);
    int32_t* dk = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + b_q32);
    int32_t* dnp = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + 2 * b_q32);
    int32_t* crow = reinterpret_cast<int32_t*>(base + b_D + b_pid + b_pd + 3 * b_q32);
    float* cd = reinterpret_cast<float*>(base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr);
    uint32_t* cs = reinterpret_cast<uint32_t*>(base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr + b_cd);
    unsigned char* tail = base + b_D + b_pid + b_pd + 3 * b_q32 + b_cr + b_cd + b_cs;
    float* scut = reinterpret_cast<float*>(tail);
    float* seps = reinterpret_cast<float*>(tail + b_q32);
    int32_t* redo = reinterpret_cast<int32_t*>(tail + 2 * b_q32);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    // The arena keeps the previous call's contents: the per-query k and
    // nprobe are written first; every other region is fully written by the
    // kernel that produces it before it is read. Fallbacks are counted in the
    // handle's device counter (allocated with the handle), which Stats reads.
    noalloc_fill_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(dk, k, dnp, np, nq);
    CK(cudaGetLastError());
    ScanParams p = h->scan_params();
    p.kq = dk;
    p.mode = mode;
    p.rerank_fixed = h->o.rerank;
    CK(launch_dist_matrix(d_queries, nq, h->o.dimension, h->d_coarse.p, h->nlist, D, s));
    CK(launch_probe_select(D, nq, h->nlist, dnp, np, dk, h->d_live.p, h->o.fallback ? 1 : 0, pid, pd, fb,
                           h->d_fb_dev.p, s));
    // parity mode with FP16 tables: queries the rerank cannot prove from the
    // scan's cut are scanned again with FP32 tables (as in run_search)
    const bool check = mode == 0 && p.adc_table && p.scanc && scan_adc_supported(h->o.num_subquantizers);
    if (check) {
        p.scan_cut = scut;
        p.scan_eps = seps;
        p.redo = redo;
        p.redo_count = redo + nq;
        CK(cudaMemsetAsync(redo + nq, 0, sizeof(int32_t), s));
    }
    CK(launch_scan(p, d_queries, nq, pid, pd, dnp, np, fb, R, crow, cd, cs, nullptr, s));
    CK(launch_rerank(p, d_queries, nq, crow, cs, R, dk, k, mode, d_ids, d_distances, d_n_out, s));
    h->launches += 5;  // fill, distance matrix, probe select, scan, rerank
    if (check) {
        ScanParams pf = p;
        pf.adc_table = 0;
        pf.scan_cut = nullptr;
        pf.qorder = redo;
        pf.qcount = redo + nq;
        CK(launch_scan(pf, d_queries, nq, pid, pd, dnp, np, fb, R, crow, cd, cs, nullptr, s));
        CK(launch_rerank(pf, d_queries, nq, crow, cs, R, dk, k, mode, d_ids, d_distances, d_n_out, s));
        h->launches += 2;
    }
    CK(note_device_search(h, s));
    return HANN_OK;
}
