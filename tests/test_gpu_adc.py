"""16-bit (FP16 and fixed-point) against FP32 lookup tables in the table
scan (kernels_scan.cu).

The reference decodes every candidate to FP32 and takes its distance
(pqivf/index.go:909-923). Here the scan screens rows through per-query ADC
tables and the rerank computes the reference's distance. With 16-bit tables
parity mode must still give the reference's results: the rerank proves each
query's top k against the screen's error bound and sends the rest to an FP32
rescan, so the results equal the oracle's whatever the tables, and the
proof must succeed for nearly every query (else the 16-bit screen is not
doing its work). In exact-rerank mode recall@10 against an FP64 brute force
must not drop by more than 0.005."""
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


def table_index(seed, n=30000, dim=96, centers=200, nlist=128, M=24, pqk=256, iters=4, offset=0.0, nq=500):
    rng = np.random.default_rng(seed)
    x, c = gaussian_mixture(rng, n, dim, centers, 0.5)
    x = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)
    q = c[rng.integers(0, centers, nq)] + 0.5 * rng.standard_normal((nq, dim))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    x = (x + offset).astype(np.float32)
    q = (q + offset).astype(np.float32)
    idx = hg.New(dim, hg.WithCoarseK(nlist), hg.WithNumSubquantizers(M), hg.WithPQK(pqk), hg.WithKMeansIters(iters))
    idx.BulkAddArrays(np.arange(n, dtype=np.int64), x)
    idx.Train()
    idx.ScanOptions(list_major=0)  # every query through the table scan
    return idx, x, q


@pytest.fixture(scope="module")
def unit():
    idx, x, q = table_index(71)
    yield idx, x, q
    idx.close()


TABLES16 = ("fp16", "fixed16")


@pytest.mark.parametrize("kind", TABLES16)
@pytest.mark.parametrize("nprobe,k", [(1, 1), (8, 10), (24, 37), (64, 100)])
def test_parity_16bit_tables(unit, kind, nprobe, k):
    idx, _, q = unit
    ora = state_to_oracle(idx.export_state())
    idx.SetADCTables(kind)
    try:
        before = idx.ADCRedos()
        g = idx.SearchBatch(q, k, nprobe=nprobe, mode=0)
        redos = idx.ADCRedos() - before
    finally:
        idx.SetADCTables("fixed16")
    assert_same_results(*g, *ora.search(q, k, nprobe, nthreads=NT)[:3])
    # the screen proves almost every query's top k by itself
    assert redos <= 0.05 * len(q), redos


def test_fp32_tables_same_results(unit):
    idx, _, q = unit
    a = idx.SearchBatch(q, 10, nprobe=16, mode=0)
    idx.SetADCTables("fp32")
    try:
        before = idx.ADCRedos()
        b = idx.SearchBatch(q, 10, nprobe=16, mode=0)
        assert idx.ADCRedos() == before  # FP32 tables are never checked
    finally:
        idx.SetADCTables("fixed16")
    assert_same_results(*a, *b)
    with pytest.raises(ValueError):
        idx.SetADCTables("fp8")


@pytest.mark.parametrize("kind", TABLES16)
def test_exact_rerank_recall(unit, kind):
    idx, x, q = unit
    gt, _ = oracle.brute_force_knn_fp64(q, x, 10)
    idx.SetADCTables(kind)
    h = idx.SearchBatch(q, 10, nprobe=16, mode=1)
    idx.SetADCTables("fp32")
    try:
        f = idx.SearchBatch(q, 10, nprobe=16, mode=1)
    finally:
        idx.SetADCTables("fixed16")

    def recall(ids):
        return np.mean([len(set(ids[i]) & set(gt[i])) / 10 for i in range(len(gt))])

    assert recall(h[0]) >= recall(f[0]) - 0.005
    # every returned distance is the exact distance of the returned row
    for i in range(0, len(q), 41):
        for j in range(h[2][i]):
            want = np.sqrt(oracle.sqeuclid(q[i], x[h[0][i, j]]))
            assert abs(h[1][i, j] - want) <= 1e-6 * max(want, 1e-12)


@pytest.mark.parametrize("kind", TABLES16)
@pytest.mark.parametrize("dim,M", [(16, 4), (32, 8), (40, 10), (64, 16), (96, 12), (128, 32), (60, 20)])
def test_shapes(dim, M, kind):
    """Every padded table width (M rounded up to 8, 16, 24, 32)."""
    rng = np.random.default_rng(dim * 31 + M)
    x, c = gaussian_mixture(rng, 6000, dim, 30, 0.4)
    q = (c[rng.integers(0, 30, 300)] + 0.4 * rng.standard_normal((300, dim))).astype(np.float32)
    idx = hg.New(dim, hg.WithCoarseK(40), hg.WithNumSubquantizers(M), hg.WithPQK(64), hg.WithKMeansIters(3))
    try:
        idx.BulkAddArrays(np.arange(len(x), dtype=np.int64), x)
        idx.Train()
        idx.ScanOptions(list_major=0)
        idx.SetADCTables(kind)
        ora = state_to_oracle(idx.export_state())
        before = idx.ADCRedos()
        g = idx.SearchBatch(q, 10, nprobe=6)
        assert_same_results(*g, *ora.search(q, 10, 6, nthreads=NT)[:3])
        assert idx.ADCRedos() - before <= 0.05 * len(q)
    finally:
        idx.close()


@pytest.mark.parametrize("kind", TABLES16)
def test_large_offset_data(kind):
    """Vectors far from the origin (every coordinate + 100): the FP32
    allowance grows with the decomposition's magnitudes; results stay the
    reference's (the FP32 rescan takes what the screen cannot prove)."""
    idx, _, q = table_index(72, n=8000, dim=32, centers=40, nlist=32, M=8, pqk=64, offset=100.0, nq=200)
    try:
        idx.SetADCTables(kind)
        ora = state_to_oracle(idx.export_state())
        g = idx.SearchBatch(q, 10, nprobe=4, mode=0)
        assert_same_results(*g, *ora.search(q, 10, 4, nthreads=NT)[:3])
    finally:
        idx.close()


def test_fallback_and_deleted_rows():
    idx, x, q = table_index(73, n=8000, nlist=256, M=12, pqk=64)
    try:
        rng = np.random.default_rng(4)
        dead = rng.choice(len(x), 2000, replace=False)
        idx.BulkDelete(dead.tolist())
        ora = state_to_oracle(idx.export_state())
        for nprobe, k in ((1, 60), (4, 10), (32, 20)):
            g = idx.SearchBatch(q, k, nprobe=nprobe, mode=0)
            assert_same_results(*g, *ora.search(q, k, nprobe, nthreads=NT)[:3])
            assert not (set(g[0][g[0] >= 0].ravel().tolist()) & set(dead.tolist()))
    finally:
        idx.close()


def test_rows_added_after_training():
    """Rows placed by BulkAdd after training get their scan codes written in
    place (and lists that outgrow their room move): results stay the
    reference's."""
    idx, x, _ = table_index(74, n=6000, dim=32, centers=30, nlist=16, M=8, pqk=64)
    try:
        rng = np.random.default_rng(5)
        extra = (x[rng.integers(0, len(x), 5000)] + 0.01 * rng.standard_normal((5000, 32))).astype(np.float32)
        idx.BulkAddArrays(np.arange(len(x), len(x) + len(extra), dtype=np.int64), extra)
        q = extra[:200] + 0.02
        ora = state_to_oracle(idx.export_state())
        g = idx.SearchBatch(q, 10, nprobe=3, mode=0)
        assert_same_results(*g, *ora.search(q, 10, 3, nthreads=NT)[:3])
    finally:
        idx.close()
