"""The oracle pinned against the reference's own known answers, its compiled
distance kernels, and its golden fixture (CPU only)."""
import math
import os

import numpy as np
import pytest

import oracle
from hann_gb300 import gob
from tests.helpers import gob_to_oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build()


# core/distance_test.go:14-86
KNOWN = [
    ([1, 2, 3, 4, 5, 6], [1, 2, 3, 4, 5, 6], 0, 0, 0, 0),
    ([1, 2, 3, 4, 5, 6], [6, 5, 4, 3, 2, 1], 70, math.sqrt(70), 18, 1 - 56.0 / 91.0),
    ([1, 0, 0, 1, 0, 1], [0, 1, 1, 0, 1, 0], 6, math.sqrt(6), 6, 1),
    ([-1, -2, -3, -4, -5, -6], [-6, -5, -4, -3, -2, -1], 70, math.sqrt(70), 18, 1 - 56.0 / 91.0),
    ([0, 0, 0, 0, 0, 0], [1, 2, 3, 4, 5, 6], 91, math.sqrt(91), 21, 1),
    ([1, 2, 3, 4, 5, 6], [1, 2, 3, 4, 5, 6.000001], 1e-12, 1e-6, 1e-6, 0),
]


@pytest.mark.parametrize("tier", [0, 1, 2, 3])
@pytest.mark.parametrize("case", KNOWN)
def test_known_answers(tier, case):
    a, b, sq, eu, l1, cos = case
    assert abs(oracle.sqeuclid(a, b, tier) - sq) < 1e-6
    assert abs(math.sqrt(oracle.sqeuclid(a, b, tier)) - eu) < 1e-6
    assert abs(oracle.manhattan(a, b, tier) - l1) < 1e-6
    assert abs(oracle.cosine(a, b, tier) - cos) < 1e-6


def test_empty_vectors():
    assert oracle.sqeuclid([], []) == 0.0
    assert oracle.manhattan([], []) == 0.0


@pytest.mark.parametrize("dim", [1, 25, 128, 784])
def test_fp64_differential(dim):
    # core/distance_test.go:159-239: every metric vs float64, tol 1e-3*max(1,|want|)
    rng = np.random.default_rng(dim)
    for _ in range(20):
        a = rng.standard_normal(dim).astype(np.float32)
        b = rng.standard_normal(dim).astype(np.float32)
        a64, b64 = a.astype(np.float64), b.astype(np.float64)
        want_sq = float(((a64 - b64) ** 2).sum())
        want_l1 = float(np.abs(a64 - b64).sum())
        na, nb = np.linalg.norm(a64), np.linalg.norm(b64)
        want_cos = 1 - float(np.clip(a64 @ b64 / (na * nb), -1, 1))
        for tier in range(4):
            assert abs(oracle.sqeuclid(a, b, tier) - want_sq) <= 1e-3 * max(1, abs(want_sq))
            assert abs(oracle.manhattan(a, b, tier) - want_l1) <= 1e-3 * max(1, abs(want_l1))
            assert abs(oracle.cosine(a, b, tier) - want_cos) <= 1e-3 * max(1, abs(want_cos))


def test_batch_matches_pairs():
    # core/metric_batch_test.go:34-72
    rng = np.random.default_rng(1)
    for dim in (25, 128, 784):
        for n in (1, 7, 64):
            q = rng.standard_normal(dim).astype(np.float32)
            flat = rng.standard_normal((n, dim)).astype(np.float32)
            out = oracle.batch(oracle.METRIC_SQEUCLID, q, flat)
            for i in range(n):
                assert out[i] == oracle.sqeuclid(q, flat[i])


needs_ref = pytest.mark.skipif(not os.path.exists(oracle.REF_PATH),
                               reason="reference kernels are compiled only where the reference tree exists")


@needs_ref
@pytest.mark.parametrize("tier", [0, 1, 2])
def test_bit_exact_vs_compiled_reference(tier):
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("x86 tiers")
    R = oracle.RefKernels()
    R.init(tier)
    rng = np.random.default_rng(tier)
    for dim in (1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 25, 31, 32, 33, 64, 96, 100, 127, 128, 129, 784):
        for _ in range(20):
            a = (rng.standard_normal(dim) * rng.uniform(0.1, 10)).astype(np.float32)
            b = rng.standard_normal(dim).astype(np.float32)
            for name, f in (("squared_euclidean", oracle.sqeuclid), ("manhattan", oracle.manhattan),
                            ("cosine_distance", oracle.cosine)):
                r, o = R.pair(name, a, b), f(a, b, tier)
                assert np.float32(r).tobytes() == np.float32(o).tobytes(), (tier, name, dim, r, o)


def test_assign_lowest_index_tie():
    # pqivf/index_test.go:1056-1069
    got = oracle.assign([[0, 0, 0, 0]], [[1, 2, 3, 4], [1, 2, 3, 4]])
    assert got[0] == 0


def _golden():
    return gob.decode_pqivf(open(os.path.join(GOLDEN, "index_v1.gob"), "rb").read())


@pytest.mark.parametrize("tier", [0, 1, 2, 3])
def test_golden_fixture_codes_and_clusters(tier):
    """The reference trained index_v1.gob: re-deriving every entry's cluster
    and PQ codes from its stored centroids and codebooks reproduces them."""
    oracle.set_tier(tier)
    try:
        ser = _golden()
        coarse = np.asarray(ser["CoarseCentroids"], np.float32)
        cbs = np.asarray(ser["Codebooks"], np.float32)
        ents = [e for c in sorted(ser["InvertedLists"]) for e in ser["InvertedLists"][c]]
        X = np.asarray([e["Vector"] for e in ents], np.float32)
        cl = np.asarray([e.get("Cluster", 0) for e in ents])
        codes = np.asarray([e["Codes"] for e in ents])
        assert (oracle.assign(X, coarse) == cl).all()
        assert (oracle.encode(X, cl, coarse, cbs) == codes).all()
    finally:
        oracle.set_tier(3)


def test_golden_fixture_counts():
    ser = _golden()
    import json
    exp = json.load(open(os.path.join(GOLDEN, "index_v1_expected.json")))
    n = sum(len(v) for v in ser["InvertedLists"].values()) + len(ser.get("PendingVectors") or {})
    assert n == exp["count"] == 29
    assert ser["Dimension"] == 8 and ser["CoarseK"] == 3 and ser["NumSubquantizers"] == 2
    assert ser["PqK"] == 4 and ser["KMeansIters"] == 5 and ser["Trained"]


def test_golden_search_stored_vectors():
    """Searching a stored vector of the golden index returns it at rank 0
    when its own reconstruction is nearest; results are sorted."""
    ser = _golden()
    ix = gob_to_oracle(ser)
    ids, dist, n, fb = ix.search(ix.vectors, 5, 3)
    assert (n == 5).all()
    assert (np.diff(dist, axis=1) >= 0).all()


def test_search_semantics_small():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((300, 8)).astype(np.float32)
    ids = np.arange(300) * 3 + 1
    init = rng.permutation(300)[:6]
    pinit = [rng.permutation(300)[:8] for _ in range(2)]
    ix, info = oracle.train(ids, x, 6, 2, 8, 4, init, pinit, reseed_idx=rng.integers(0, 300, 100))
    # lists in ascending id order (pqivf/index_test.go:1072-1101)
    for c in range(ix.nlist):
        li = ix.ids[ix.list_off[c]:ix.list_off[c + 1]]
        assert (np.diff(li) > 0).all()
    r_ids, r_d, r_n, fb = ix.search(x[:10], 5, 2)
    assert (r_n == 5).all()
    # brute-force fallback: k above the probed candidates
    r_ids, r_d, r_n, fb = ix.search(x[:3], 299, 1)
    assert fb.all() and (r_n == 299).all()


def test_neon_fast_path_equals_generic_tier():
    """The vectorisable NEON-order squared distance the oracle's search and
    k-means use equals the generic lane-by-lane restatement bit for bit."""
    oracle.set_tier(oracle.TIER_NEON)
    rng = np.random.default_rng(1)
    for n in (1, 3, 4, 15, 16, 17, 31, 32, 96, 128, 129, 784):
        a = (rng.normal(size=(300, n)) * rng.choice([1e-3, 1, 1e3], size=(300, 1))).astype(np.float32)
        b = rng.normal(size=n).astype(np.float32)
        generic = np.array([oracle.sqeuclid(a[i], b, tier=oracle.TIER_NEON) for i in range(300)], np.float32)
        assert np.array_equal(generic.astype(np.float64), oracle.batch(oracle.METRIC_SQEUCLID, b, a)), n


def test_exact_rerank_search_mode():
    """rerank=R keeps the R best candidates by PQ distance and orders them by
    the exact distance to their stored vectors: with R covering every
    candidate of the probed lists the result is the exact k-NN over those
    lists."""
    oracle.set_tier(oracle.TIER_NEON)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((400, 8)).astype(np.float32)
    ids = np.arange(400)
    ix, _ = oracle.train(ids, x, 4, 2, 8, 4, rng.permutation(400)[:4], [rng.permutation(400)[:8] for _ in range(2)],
                         reseed_idx=rng.integers(0, 400, 100))
    q = rng.standard_normal((20, 8)).astype(np.float32)
    r_ids, r_d, r_n, _ = ix.search(q, 5, 2, rerank=400)
    for i in range(len(q)):
        probed = oracle.OracleIndex.probe(ix, q[i], 2)
        rows = np.concatenate([np.arange(ix.list_off[c], ix.list_off[c + 1]) for c in probed])
        d = np.array([oracle.sqeuclid(q[i], ix.vectors[r]) for r in rows], np.float64)
        order = np.argsort(d, kind="stable")[:5]
        assert np.array_equal(r_ids[i, :5], ix.ids[rows[order]])
        np.testing.assert_allclose(r_d[i, :5], np.sqrt(d[order]), rtol=1e-12)
    # rerank of fewer candidates than k still returns the candidates it kept
    r_ids, r_d, r_n, _ = ix.search(q, 5, 2, rerank=3)
    assert (r_n == 3).all()
