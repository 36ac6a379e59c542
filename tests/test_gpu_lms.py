"""The list-major tensor-core scan (kernels_lms.cu) against the oracle and
against the table scan on the same index.

Parity mode must give the reference's results (ids identical except inside
1e-5-relative ties of the reference distance, distances within 1e-5) for
every choice of chunks, rows per work item and blocks per SM, including
queries it hands to the table scan (brute-force fallbacks, bands that
overflow) and lists with deleted rows. In exact-rerank mode every returned
distance is the exact distance of the returned row and recall@10 against an
FP64 brute force is not below the table scan's."""
import os

import numpy as np
import pytest

import hann_gb300 as hg
import oracle
from tests.helpers import assert_same_results, gaussian_mixture, state_to_oracle

pytestmark = pytest.mark.gpu
NT = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def _setup(gpu):
    oracle.set_tier(oracle.TIER_NEON)


def unit_index(seed, n=30000, dim=96, centers=200, nlist=128, M=24, pqk=256, iters=4):
    rng = np.random.default_rng(seed)
    x, c = gaussian_mixture(rng, n, dim, centers, 0.5)
    x = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)
    q = c[rng.integers(0, centers, 600)] + 0.5 * rng.standard_normal((600, dim))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    idx = hg.New(dim, hg.WithCoarseK(nlist), hg.WithNumSubquantizers(M), hg.WithPQK(pqk), hg.WithKMeansIters(iters))
    idx.BulkAddArrays(np.arange(n, dtype=np.int64), x)
    idx.Train()
    idx.ScanOptions(min_nprobe=1)  # every query through the list-major scan
    return idx, x, q


@pytest.fixture(scope="module")
def bench_like():
    idx, x, q = unit_index(61)
    yield idx, x, q
    idx.close()


def test_list_major_scan_runs(bench_like):
    idx, _, q = bench_like
    opts = idx.ScanOptions()
    assert opts["list_major"] == 1 and opts["min_nprobe"] == 1
    idx.SetProfiling(True)
    idx.StageTimes()
    idx.SearchBatch(q[:200], 10, nprobe=8)
    idx.StageTimes()
    idx.SetProfiling(False)
    assert idx.RowsDecoded() > 0


@pytest.mark.parametrize("nprobe,k", [(1, 10), (8, 10), (24, 1), (24, 37), (128, 100)])
def test_parity_against_oracle(bench_like, nprobe, k):
    idx, _, q = bench_like
    ora = state_to_oracle(idx.export_state())
    g = idx.SearchBatch(q, k, nprobe=nprobe)
    o = ora.search(q, k, nprobe, nthreads=NT)
    assert_same_results(*g, *o[:3])


@pytest.mark.parametrize("opts", [
    dict(first_chunk=1, chunk_growth=2, rows_per_item=128, ctas_per_sm=1),
    dict(first_chunk=2, chunk_growth=4, rows_per_item=256, ctas_per_sm=2),
    dict(first_chunk=1, chunk_growth=64, rows_per_item=4096, ctas_per_sm=2),
    dict(seed_threshold=0, first_chunk=1, chunk_growth=8),
    dict(seed_threshold=1, first_chunk=4, chunk_growth=4),
    dict(min_nprobe=16),
])
def test_options_do_not_change_results(bench_like, opts):
    idx, _, q = bench_like
    ora = state_to_oracle(idx.export_state())
    before = idx.ScanOptions()
    try:
        idx.ScanOptions(**opts)
        for mode in (0, 1):
            g = idx.SearchBatch(q, 10, nprobe=16, mode=mode)
            if mode == 0:
                assert_same_results(*g, *ora.search(q, 10, 16, nthreads=NT)[:3])
            else:
                idx.ScanOptions(**before)
                t = idx.SearchBatch(q, 10, nprobe=16, mode=mode)
                idx.ScanOptions(**opts)
                assert (g[2] == t[2]).all()
    finally:
        idx.ScanOptions(**before)


def test_matches_table_scan(bench_like):
    """The same queries through the table scan: parity-mode results agree,
    and exact-rerank recall@10 against FP64 brute force is not lower."""
    idx, x, q = bench_like
    gt, _ = oracle.brute_force_knn_fp64(q, x, 10)
    lm = [idx.SearchBatch(q, 10, nprobe=16, mode=m) for m in (0, 1)]
    idx.ScanOptions(list_major=0)
    try:
        tb = [idx.SearchBatch(q, 10, nprobe=16, mode=m) for m in (0, 1)]
    finally:
        idx.ScanOptions(list_major=1)
    assert_same_results(*lm[0], *tb[0])

    def recall(ids):
        return np.mean([len(set(ids[i]) & set(gt[i])) / 10 for i in range(len(gt))])

    assert recall(lm[1][0]) >= recall(tb[1][0]) - 0.002
    # exact-rerank distances are the exact distances of the returned rows
    for i in range(0, len(q), 37):
        for j in range(lm[1][2][i]):
            want = np.sqrt(oracle.sqeuclid(q[i], x[lm[1][0][i, j]]))
            assert abs(lm[1][1][i, j] - want) <= 1e-6 * max(want, 1e-12)


def test_fallback_and_deleted_rows():
    """Deleted rows never come back; queries whose probed lists hold fewer
    than k rows take the brute-force fallback (through the table scan) with
    the reference's results."""
    idx, x, q = unit_index(62, n=8000, nlist=256, M=12, pqk=64)
    try:
        rng = np.random.default_rng(3)
        dead = rng.choice(len(x), 2000, replace=False)
        idx.BulkDelete(dead.tolist())
        ora = state_to_oracle(idx.export_state())
        for nprobe, k in ((1, 60), (4, 10), (32, 20)):
            g = idx.SearchBatch(q, k, nprobe=nprobe)
            o = ora.search(q, k, nprobe, nthreads=NT)
            assert_same_results(*g, *o[:3])
            assert not (set(g[0][g[0] >= 0].ravel().tolist()) & set(dead.tolist()))
    finally:
        idx.close()


@pytest.mark.parametrize("dim,M", [(16, 4), (32, 8), (64, 8), (128, 16), (40, 10), (8, 4)])
def test_shapes(dim, M):
    """Dimensions with K padding (not a multiple of 16), subquantizer widths
    of 2, 4 and 8, and the general decode path."""
    rng = np.random.default_rng(dim * 100 + M)
    x, c = gaussian_mixture(rng, 6000, dim, 30, 0.4)
    q = (c[rng.integers(0, 30, 300)] + 0.4 * rng.standard_normal((300, dim))).astype(np.float32)
    idx = hg.New(dim, hg.WithCoarseK(40), hg.WithNumSubquantizers(M), hg.WithPQK(32), hg.WithKMeansIters(3))
    try:
        idx.BulkAddArrays(np.arange(len(x), dtype=np.int64), x)
        idx.Train()
        idx.ScanOptions(min_nprobe=1)
        ora = state_to_oracle(idx.export_state())
        g = idx.SearchBatch(q, 10, nprobe=6)
        o = ora.search(q, 10, 6, nthreads=NT)
        assert_same_results(*g, *o[:3])
    finally:
        idx.close()


def test_uneven_k_and_nprobe(bench_like):
    """One batch with per-query k in [1, 100] and nprobe in [1, 128]: each
    query's result equals its result searched alone-sized (the oracle)."""
    idx, _, q = bench_like
    rng = np.random.default_rng(8)
    k = rng.integers(1, 101, len(q)).astype(np.int32)
    npb = np.exp(rng.uniform(0, np.log(128), len(q))).astype(np.int32)
    ora = state_to_oracle(idx.export_state())
    ids, dist, n = idx.SearchBatch(q, k, nprobe=npb)
    for i in range(0, len(q), 7):
        o = ora.search(q[i:i + 1], int(k[i]), int(npb[i]), nthreads=1)
        assert_same_results(ids[i:i + 1, :k[i]], dist[i:i + 1, :k[i]], n[i:i + 1], *o[:3])


def test_routing_by_nprobe(bench_like):
    """Queries probing fewer lists than min_nprobe take the table scan, the
    others the list-major scan, in one batch: every result is the
    reference's."""
    idx, _, q = bench_like
    before = idx.ScanOptions()
    try:
        idx.ScanOptions(min_nprobe=20)
        rng = np.random.default_rng(12)
        npb = rng.integers(1, 60, len(q)).astype(np.int32)
        ora = state_to_oracle(idx.export_state())
        ids, dist, n = idx.SearchBatch(q, 10, nprobe=npb)
        for i in range(0, len(q), 5):
            o = ora.search(q[i:i + 1], 10, int(npb[i]), nthreads=1)
            assert_same_results(ids[i:i + 1], dist[i:i + 1], n[i:i + 1], *o[:3])
    finally:
        idx.ScanOptions(**before)


def test_autotune_scan(bench_like):
    """The autotuner measures both scans on a sample, keeps one routing, and
    searches afterwards still give the reference's results."""
    idx, _, q = bench_like
    before = idx.ScanOptions()
    try:
        r = idx.AutotuneScan(q[:400], 10, mode=1)
        opts = r["options"]
        assert opts == idx.ScanOptions()
        assert opts["min_nprobe"] in (8, 16, 32, 64, 128, 129)
        assert set(r["ms_table_scan"]) == {8, 16, 32, 64, 128} == set(r["ms_list_major"])
        assert all(v > 0 for v in r["ms_table_scan"].values())
        ora = state_to_oracle(idx.export_state())
        for nprobe in (8, 128):
            assert_same_results(*idx.SearchBatch(q, 10, nprobe=nprobe), *ora.search(q, 10, nprobe, nthreads=NT)[:3])
    finally:
        idx.ScanOptions(**before)
