"""GPU path vs the oracle: distances bit-exact, the reference's golden index,
training inertia, encoding, search results (parity bar: ids identical except
inside 1e-5-relative ties, distances within 1e-5 relative)."""
import io
import os

import numpy as np
import pytest

import hann_gb300 as hg
import oracle
from hann_gb300 import gob
from tests.helpers import REL, assert_same_results, gaussian_mixture, gob_to_oracle, state_to_oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "index_v1.gob")
NT = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def _setup(gpu):
    oracle.set_tier(oracle.TIER_NEON)


@pytest.mark.parametrize("metric", [0, 1, 2, 3])
def test_distance_batch_bit_exact(metric):
    rng = np.random.default_rng(metric)
    for dim in (1, 3, 4, 8, 16, 17, 31, 96, 128, 784):
        q = rng.standard_normal(dim).astype(np.float32)
        flat = rng.standard_normal((300, dim)).astype(np.float32)
        flat[0] = q
        if metric == 3:
            flat[1] = 0
        g = hg.distance_batch(metric, q, flat)
        o = oracle.batch(metric, q, flat)
        assert np.array_equal(g, o), (metric, dim, np.nonzero(g != o)[0][:5])


def _golden_index():
    idx = hg.New(8)
    idx.Load(io.BytesIO(open(GOLDEN, "rb").read()))
    return idx


def test_golden_load_stats_and_codes():
    idx = _golden_index()
    assert idx.Stats().Count == 29
    st = idx.export_state()
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    want = [e["Codes"] for c in sorted(ser["InvertedLists"]) for e in ser["InvertedLists"][c]]
    assert np.array_equal(st["codes"], np.asarray(want))


def test_golden_recode_matches_reference_codes():
    """Codes the GPU computes for the fixture's vectors equal the codes the
    reference stored (encodeWithCodebooks on the reference's CPU)."""
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    st = hg.gob_to_state(ser)
    want = st["codes"].copy()
    st["has_codes"] = np.zeros_like(st["has_codes"])
    st["codes"] = np.zeros_like(st["codes"])
    idx = hg.New(8)
    idx.import_state(st)
    assert np.array_equal(idx.export_state()["codes"], want)


def test_golden_search_parity():
    idx = _golden_index()
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    ora = gob_to_oracle(ser)
    rng = np.random.default_rng(8)
    q = (ora.vectors[rng.integers(0, ora.count, 40)] + 0.1 * rng.standard_normal((40, 8))).astype(np.float32)
    for k in (1, 5, 29, 40):
        g = idx.SearchBatch(q, k)
        o = ora.search(q, k, 3)
        assert_same_results(*g, *o[:3])
    # one-query Search, twice (golden_test.go:122-145)
    for _ in range(2):
        res = idx.Search(q[0], 5)
        o = ora.search(q[:1], 5, 3)
        assert [r.ID for r in res] == list(o[0][0][:5])


@pytest.fixture(scope="module")
def config1():
    """Plain PQIVF at 20,000 x 128: 64 centers ~ N(0,1), sigma 0.3; coarse 64,
    8 x 256 (16-d), 10 iterations, seeded init; 1,000 queries."""
    rng = np.random.default_rng(20240)
    n, dim = 20000, 128
    x, centers = gaussian_mixture(rng, n, dim, 64, 0.3)
    lab = rng.integers(0, 64, 1000)
    q = (centers[lab] + 0.3 * rng.standard_normal((1000, dim))).astype(np.float32)
    ids = np.arange(n, dtype=np.int64) * 7 + 3
    cinit = rng.permutation(n)[:64]
    pinit = np.stack([rng.permutation(n)[:256] for _ in range(8)])
    reseed = rng.integers(0, n, 10000)
    idx = hg.New(dim, hg.WithCoarseK(64), hg.WithNumSubquantizers(8), hg.WithPQK(256), hg.WithKMeansIters(10))
    idx.BulkAddArrays(ids, x)
    idx.TrainSeeded(cinit, pinit, reseed)
    ora, info = oracle.train(ids, x, 64, 8, 256, 10, cinit, pinit, reseed, nthreads=NT)
    return {"x": x, "q": q, "ids": ids, "idx": idx, "ora": ora, "info": info}


def test_train_inertia_within_half_percent(config1):
    c = config1
    st = c["idx"].export_state()
    order = np.argsort(c["ids"])
    x = c["x"][order]
    g_asg = oracle.assign(x, st["coarse"], NT)
    o_asg = c["info"]["assign"]
    gi = oracle.inertia_fp64(x, st["coarse"], g_asg)
    oi = oracle.inertia_fp64(x, c["ora"].coarse, o_asg)
    assert abs(gi - oi) <= 0.005 * oi, (gi, oi)
    # product quantizer: reconstruction error of each side's own encoding
    def pq_err(coarse, cbs, asg):
        codes = oracle.encode(x, asg, coarse, cbs, NT)
        M, K, ds = cbs.shape
        rec = coarse[asg] + np.concatenate([cbs[m][codes[:, m]] for m in range(M)], axis=1)
        d = x.astype(np.float64) - rec
        return float((d * d).sum())
    ge = pq_err(st["coarse"], st["codebooks"], g_asg)
    oe = pq_err(c["ora"].coarse, c["ora"].codebooks, o_asg)
    assert abs(ge - oe) <= 0.005 * oe, (ge, oe)


def test_assignment_and_codes_match_oracle(config1):
    """Given the GPU-trained centroids and codebooks, every entry's list and
    codes are the oracle's (ties within 1e-5 relative allowed)."""
    st = config1["idx"].export_state()
    ora = state_to_oracle(st)
    x = st["vectors"]
    cl = np.repeat(np.arange(st["layout"]["nlist"]), st["list_len"])
    assert np.array_equal(oracle.assign(x, st["coarse"], NT), cl)
    want = oracle.encode(x, cl, st["coarse"], st["codebooks"], NT)
    bad = np.argwhere(want != st["codes"])
    for r, m in bad:
        ds = x.shape[1] // st["codes"].shape[1]
        res = x[r, m * ds:(m + 1) * ds] - st["coarse"][cl[r], m * ds:(m + 1) * ds]
        a = oracle.sqeuclid(res, st["codebooks"][m][want[r, m]])
        b = oracle.sqeuclid(res, st["codebooks"][m][st["codes"][r, m]])
        assert abs(a - b) <= REL * max(a, 1e-12), (r, m, a, b)
    # lists hold ascending ids (pqivf/index_test.go:1072-1101)
    off = 0
    for n in st["list_len"]:
        assert (np.diff(st["ids"][off:off + n]) > 0).all()
        off += n


@pytest.mark.parametrize("nprobe", [3, 8, 64])
@pytest.mark.parametrize("k", [1, 10, 100])
def test_search_parity_config1(config1, nprobe, k):
    idx = config1["idx"]
    st = idx.export_state()
    ora = state_to_oracle(st)
    q = config1["q"][:300]
    g = idx.SearchBatch(q, k, nprobe=nprobe)
    o = ora.search(q, k, nprobe, nthreads=NT)
    assert_same_results(*g, *o[:3])


def test_recall_not_below_reference(config1):
    idx = config1["idx"]
    st = idx.export_state()
    ora = state_to_oracle(st)
    q = config1["q"]
    gt, _ = oracle.brute_force_knn_fp64(q, config1["x"], 10, base_ids=config1["ids"])
    g_ids, _, _ = idx.SearchBatch(q, 10, nprobe=8)
    o_ids = ora.search(q, 10, 8, nthreads=NT)[0]
    def recall(ids):
        return np.mean([len(set(ids[i]) & set(gt[i])) / 10 for i in range(len(gt))])
    assert recall(g_ids) >= recall(o_ids) - 1e-9
    # the exact-rerank mode only improves on the PQ distances
    e_ids, e_d, _ = idx.SearchBatch(q, 10, nprobe=8, mode=hg.MODE_EXACT_RERANK)
    assert recall(e_ids) >= recall(g_ids)


def test_exact_rerank_distances(config1):
    idx = config1["idx"]
    q = config1["q"][:50]
    ids, d, n = idx.SearchBatch(q, 10, nprobe=8, mode=hg.MODE_EXACT_RERANK)
    pos = {int(i): r for r, i in enumerate(config1["ids"])}
    for i in range(len(q)):
        for j in range(n[i]):
            want = np.sqrt(np.float64(oracle.sqeuclid(q[i], config1["x"][pos[int(ids[i, j])]])))
            assert d[i, j] == want
        assert (np.diff(d[i, :n[i]]) >= 0).all()


@pytest.mark.parametrize("M", [24, 12, 32, 6, 48, 16])
def test_search_parity_by_subquantizers(M):
    """Every scan-kernel shape (M = 24 as the 10M x 96 bench, M not dividing
    32, M = 32, the general M > 32 kernel) against the oracle, both in
    parity mode and with the exact rerank, on unit-norm 96-d data."""
    rng = np.random.default_rng(500 + M)
    x, centers = gaussian_mixture(rng, 12000, 96, 40, 0.35)
    x = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)
    q = centers[rng.integers(0, 40, 200)] + 0.35 * rng.standard_normal((200, 96))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    idx = hg.New(96, hg.WithCoarseK(48), hg.WithNumSubquantizers(M), hg.WithPQK(64), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(len(x), dtype=np.int64), x)
    idx.Train()
    ora = state_to_oracle(idx.export_state())
    for nprobe, k in ((4, 10), (13, 37)):
        g = idx.SearchBatch(q, k, nprobe=nprobe)
        o = ora.search(q, k, nprobe, nthreads=NT)
        assert_same_results(*g, *o[:3])
    # exact rerank: rows of the probed lists, exact distances, ascending
    ids, dist, n = idx.SearchBatch(q[:50], 10, nprobe=8, mode=1)
    st = idx.export_state()
    starts = np.concatenate([[0], np.cumsum(st["list_len"])])
    vec_of = dict(zip(st["ids"].tolist(), range(len(st["ids"]))))
    for i in range(50):
        rows = np.concatenate([np.arange(starts[l], starts[l + 1]) for l in ora.probe(q[i], 8)])
        allowed = set(st["ids"][rows].tolist())
        got = ids[i, :n[i]]
        assert set(got.tolist()) <= allowed
        assert (np.diff(dist[i, :n[i]]) >= 0).all()
        for j, id_ in enumerate(got):
            want = np.sqrt(oracle.sqeuclid(q[i], st["vectors"][vec_of[int(id_)]]))
            assert abs(dist[i, j] - want) <= 1e-6 * max(want, 1e-12)
