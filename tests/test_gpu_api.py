"""The reference's interface semantics on the GPU index (pqivf/index_test.go):
errors, edge cases, fallback, mutations, persistence."""
import io

import numpy as np
import pytest

import hann_gb300 as hg
import oracle
from tests.helpers import assert_same_results, state_to_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup(gpu):
    oracle.set_tier(oracle.TIER_NEON)


def new_index(dim, coarse_k, m, pqk, iters, *more):
    return hg.New(dim, hg.WithCoarseK(coarse_k), hg.WithNumSubquantizers(m), hg.WithPQK(pqk),
                  hg.WithKMeansIters(iters), *more)


def test_new_validation():
    # pqivf/index_test.go:502-568
    for args in [(0,), (-1,)]:
        with pytest.raises(hg.HannError, match="dimension"):
            hg.New(*args)
    with pytest.raises(hg.HannError, match="coarseK"):
        hg.New(4, hg.WithCoarseK(0))
    with pytest.raises(hg.HannError, match="pqK"):
        hg.New(4, hg.WithPQK(0))
    with pytest.raises(hg.HannError, match="kMeansIters"):
        hg.New(4, hg.WithKMeansIters(0))
    with pytest.raises(hg.HannError, match="numSubquantizers"):
        hg.New(4, hg.WithNumSubquantizers(0))
    with pytest.raises(hg.HannError, match="divisible"):
        hg.New(6, hg.WithNumSubquantizers(4))


def test_edge_cases():
    # pqivf/index_test.go:371-453
    idx = new_index(4, 2, 2, 256, 5)
    with pytest.raises(hg.HannError):
        idx.Train()
    with pytest.raises(hg.HannError):
        idx.Search([1, 2, 3, 4], 1)
    idx.Add(1, [1, 1, 1, 1])
    with pytest.raises(hg.HannError, match="already exists"):
        idx.Add(1, [1, 1, 1, 1])
    with pytest.raises(hg.HannError):
        idx.Add(2, [1, 2, 3])
    with pytest.raises(hg.HannError):
        idx.Update(1, [1, 2, 3])
    with pytest.raises(hg.HannError):
        idx.Search([1, 2, 3], 1)
    with pytest.raises(hg.HannError, match="not enough vectors"):
        idx.Train()
    idx.BulkAdd({2: [2, 2, 2, 2], 3: [3, 3, 3, 3]})
    idx.Train()
    with pytest.raises(hg.HannError, match="k must be positive"):
        idx.Search([1, 1, 1, 1], 0)
    res = idx.Search([1, 1, 1, 1], 5)
    assert len(res) == 3
    assert res[0].ID == 1


def test_untrained_search_errors():
    idx = new_index(4, 2, 2, 2, 5)
    idx.Add(1, [1, 0, 0, 0])
    with pytest.raises(hg.HannError, match="not trained"):
        idx.Search([1, 0, 0, 0], 1)


def clustered_vectors():
    rng = np.random.default_rng(11)
    centers = np.array([[0, 0, 0, 0], [10, 10, 10, 10], [-10, 10, -10, 10], [10, -10, 10, -10]], np.float32)
    return {i: (centers[i % 4] + rng.normal(size=4)).astype(np.float32) for i in range(40)}


def test_candidate_clusters_and_fallback_off():
    # pqivf/index_test.go:570-641
    vecs = clustered_vectors()
    q = vecs[0]
    k = len(vecs)
    r = new_index(4, 4, 2, 4, 10, hg.WithCandidateClusters(1), hg.WithBruteForceFallback(False))
    r.BulkAdd(vecs)
    r.Train()
    got = r.Search(q, k)
    assert 0 < len(got) < k
    assert any(n.ID == 0 for n in got)
    assert r.Stats().FallbackSearches == 0
    f = new_index(4, 4, 2, 4, 10, hg.WithCandidateClusters(1))
    f.BulkAdd(vecs)
    f.Train()
    got = f.Search(q, k)
    assert len(got) == k
    assert f.Stats().FallbackSearches >= 1
    ora = state_to_oracle(f.export_state())
    o = ora.search(q[None, :], k, 1)
    assert_same_results(*f.SearchBatch(q[None, :], k, nprobe=1), *o[:3])


def test_fallback_counter():
    # pqivf/index_test.go:819-845
    pq = new_index(4, 8, 2, 2, 5)
    for i in range(40):
        pq.Add(i, [i, i + 1, i + 2, i + 3])
    pq.Train()
    assert pq.Stats().FallbackSearches == 0
    pq.Search([0, 1, 2, 3], 40)
    assert pq.Stats().FallbackSearches >= 1


def test_delete_all_then_search():
    # pqivf/index_test.go:847-892
    idx = new_index(4, 2, 2, 2, 5)
    vecs = {1: [1, 0, 0, 0], 2: [0, 1, 0, 0], 3: [0, 0, 1, 0], 4: [0, 0, 0, 1]}
    idx.BulkAdd(vecs)
    idx.Train()
    for i in vecs:
        idx.Delete(i)
    assert idx.Stats().Count == 0
    assert idx.Search([1, 0, 0, 0], 2) == []
    idx.Add(5, [1, 1, 0, 0])
    res = idx.Search([1, 1, 0, 0], 1)
    assert len(res) == 1 and res[0].ID == 5


def test_delete_unknown_and_bulk_semantics():
    # pqivf/index_test.go:679-710
    idx = new_index(4, 2, 2, 2, 5)
    idx.BulkAdd({1: [1, 0, 0, 0], 2: [0, 1, 0, 0], 3: [0, 0, 1, 0]})
    with pytest.raises(hg.HannError, match="not found"):
        idx.Delete(99)
    ids = [3, 99, 1]
    idx.BulkDelete(ids)
    assert ids == [3, 99, 1]
    assert idx.Stats().Count == 1
    with pytest.raises(hg.HannError, match="not found"):
        idx.BulkUpdate({2: [0, 0, 0, 1], 77: [1, 1, 1, 1]})
    with pytest.raises(hg.HannError, match="invalid vector for id"):
        idx.BulkUpdate({2: [0, 0, 0]})
    assert idx.Stats().Count == 1


def test_bulk_add_stops_at_first_failure():
    # pqivf/index_test.go:643-677: ids before the failing one stay added
    idx = new_index(4, 2, 2, 2, 5)
    idx.Add(5, [5, 5, 5, 5])
    with pytest.raises(hg.HannError, match="already exists"):
        idx.BulkAdd({1: [1, 1, 1, 1], 5: [0, 0, 0, 0], 9: [9, 9, 9, 9]})
    assert idx.Stats().Count == 2
    with pytest.raises(hg.HannError, match="does not match index dimension 4 for id 12"):
        idx.BulkAdd({11: [1, 1, 1, 1], 12: [1, 1]})
    assert idx.Stats().Count == 3


def test_mutations_after_train_match_oracle():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(2000, 16)).astype(np.float32)
    idx = new_index(16, 16, 4, 16, 5, hg.WithCandidateClusters(4))
    idx.BulkAddArrays(np.arange(2000), x)
    idx.Train()
    # adds (a list may grow past its capacity), deletes, updates
    extra = rng.normal(size=(3000, 16)).astype(np.float32)
    idx.BulkAddArrays(np.arange(5000, 8000), extra)
    idx.BulkDelete(list(range(0, 2000, 3)))
    idx.Delete(1)
    idx.Update(2, x[2] + 1)
    idx.BulkUpdate({5000: extra[0] * 2, 4: x[4] - 1})
    st = idx.export_state()
    live = set(range(2000)) - set(range(0, 2000, 3)) - {1}
    live |= set(range(5000, 8000))
    assert set(st["ids"].tolist()) == live
    assert idx.Stats().Count == len(live)
    # every stored row sits in its nearest list with its own codes
    cl = np.repeat(np.arange(st["layout"]["nlist"]), st["list_len"])
    assert np.array_equal(oracle.assign(st["vectors"], st["coarse"]), cl)
    assert np.array_equal(oracle.encode(st["vectors"], cl, st["coarse"], st["codebooks"]), st["codes"])
    ora = state_to_oracle(st)
    q = rng.normal(size=(100, 16)).astype(np.float32)
    assert_same_results(*idx.SearchBatch(q, 10), *ora.search(q, 10, 4)[:3])


def test_growing_lists_move_and_relayout():
    """Chunks of vectors near one centroid overflow that list again and
    again: it moves to the arena's free tail each time (its old slots become
    holes) until the holes call for a full relayout. After every chunk, with
    deletes between, the index answers like the oracle on its own state."""
    rng = np.random.default_rng(17)
    x = rng.normal(size=(3000, 16)).astype(np.float32)
    idx = new_index(16, 32, 4, 16, 4, hg.WithCandidateClusters(6))
    idx.BulkAddArrays(np.arange(3000), x)
    idx.Train()
    c0 = idx.export_state()["coarse"][5]
    q = np.concatenate([c0 + 0.05 * rng.normal(size=(40, 16)),
                        rng.normal(size=(40, 16))]).astype(np.float32)
    next_id = 10_000
    for rnd in range(12):
        chunk = (c0 + 0.05 * rng.normal(size=(150 * (rnd + 1), 16))).astype(np.float32)
        idx.BulkAddArrays(np.arange(next_id, next_id + len(chunk)), chunk)
        next_id += len(chunk)
        if rnd % 3 == 2:
            idx.BulkDelete(list(range(next_id - 100, next_id)))
        st = idx.export_state()
        cl = np.repeat(np.arange(st["layout"]["nlist"]), st["list_len"])
        assert np.array_equal(oracle.assign(st["vectors"], st["coarse"]), cl)
        ora = state_to_oracle(st)
        for mode in (0, 1):
            g = idx.SearchBatch(q, 10, mode=mode)
            if mode == 0:
                assert_same_results(*g, *ora.search(q, 10, 6)[:3])
            else:
                assert (g[2] == 10).all()
    assert idx.Stats().Count == 3000 + sum(150 * (r + 1) for r in range(12)) - 4 * 100
    ar = idx.ArenaStats()
    # the list moved into the slack, and at least once the holes (or the
    # slack running out) called for a full relayout after training's
    assert ar["list_moves"] >= 2 and ar["full_relayouts"] >= 2, ar


def test_save_load_round_trip():
    rng = np.random.default_rng(6)
    x = rng.normal(size=(1000, 8)).astype(np.float32)
    idx = new_index(8, 8, 2, 16, 5, hg.WithCandidateClusters(5))
    idx.BulkAddArrays(np.arange(1000), x)
    idx.Train()
    idx.Add(5000, x[0])
    buf = io.BytesIO()
    idx.Save(buf)
    other = hg.New(8)
    other.Load(io.BytesIO(buf.getvalue()))
    assert other.Stats().Count == 1001
    q = rng.normal(size=(50, 8)).astype(np.float32)
    a = idx.SearchBatch(q, 7)
    b = other.SearchBatch(q, 7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # candidate clusters travel with the file (pqivf/index_test.go:894-942)
    assert other.export_state()["layout"]["candidate_clusters"] == 5


def test_save_load_untrained_keeps_pending():
    idx = new_index(4, 2, 2, 2, 5)
    idx.BulkAdd({1: [1, 0, 0, 0], 2: [0, 1, 0, 0]})
    buf = io.BytesIO()
    idx.Save(buf)
    other = hg.New(4)
    other.Load(io.BytesIO(buf.getvalue()))
    assert other.Stats().Count == 2
    other.Add(3, [0, 0, 1, 0])
    other.Train()
    assert len(other.Search([1, 0, 0, 0], 3)) == 3


def test_search_batch_uneven_k_and_nprobe():
    rng = np.random.default_rng(9)
    x = rng.normal(size=(3000, 32)).astype(np.float32)
    idx = new_index(32, 32, 8, 32, 5)
    idx.BulkAddArrays(np.arange(3000), x)
    idx.Train()
    q = rng.normal(size=(64, 32)).astype(np.float32)
    k = rng.integers(1, 60, 64)
    npb = rng.integers(1, 33, 64)
    g = idx.SearchBatch(q, k, nprobe=npb)
    o = state_to_oracle(idx.export_state()).search(q, k, npb)
    assert_same_results(*g, *o[:3])
    # each row alone equals the row in the mix
    for i in (0, 17, 63):
        gi = idx.SearchBatch(q[i:i + 1], int(k[i]), nprobe=int(npb[i]))
        assert np.array_equal(gi[0][0, :gi[2][0]], g[0][i, :g[2][i]])


def test_gob_encode_decode_methods():
    """GobEncode / GobDecode on the index (pqivf/index.go:992-1084), and a
    struct holding only the five parameters decodes to an empty index that
    takes an Add (pqivf/index_test.go:771-795)."""
    from tests.helpers import flat_struct_stream

    rng = np.random.default_rng(9)
    x = rng.normal(size=(800, 8)).astype(np.float32)
    idx = new_index(8, 8, 2, 16, 5)
    idx.BulkAddArrays(np.arange(800), x)
    idx.Train()
    data = idx.GobEncode()
    other = hg.New(8)
    other.GobDecode(data)
    a, b = idx.export_state(), other.export_state()
    assert a["layout"] == b["layout"]
    for key in ("coarse", "codebooks", "list_len", "ids", "vectors", "codes"):
        assert np.array_equal(a[key], b[key]), key
    legacy = hg.New(4)
    legacy.GobDecode(flat_struct_stream([("Dimension", 4), ("CoarseK", 2), ("NumSubquantizers", 2), ("PqK", 4),
                                         ("KMeansIters", 5)]))
    legacy.Add(1, [1, 2, 3, 4])
    assert legacy.Stats().Count == 1
    with pytest.raises(hg.HannError):
        legacy.GobDecode(b"not a gob stream")
    assert legacy.Stats().Count == 1  # a failed decode changes nothing
