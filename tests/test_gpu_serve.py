"""Continuous-batching server: requests of uneven size, k and nprobe from
several threads, batched together on several streams; each result equals a
Search of the request's queries alone. Mutations run between batches."""
import threading

import numpy as np
import pytest

import hann_gb300 as hg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def index(gpu):
    rng = np.random.default_rng(77)
    x = rng.normal(size=(60000, 32)).astype(np.float32)
    idx = hg.New(32, hg.WithCoarseK(256), hg.WithNumSubquantizers(8), hg.WithPQK(256), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(60000), x)
    idx.Train()
    yield idx, x, rng
    idx.close()


@pytest.mark.parametrize("mode", [hg.MODE_PARITY, hg.MODE_EXACT_RERANK])
def test_each_result_equals_alone(index, mode):
    idx, x, rng = index
    reqs = []
    for _ in range(80):
        nq = int(rng.integers(1, 65))
        reqs.append((rng.normal(size=(nq, 32)).astype(np.float32), int(rng.integers(1, 51)),
                     int(rng.integers(1, 65))))
    out = [None] * len(reqs)
    with hg.Server(idx, slots=3, max_batch_queries=512, max_k=50, max_nprobe=64, mode=mode) as srv:
        def worker(lo, hi):
            tickets = [(i, srv.submit(reqs[i][0], reqs[i][1], reqs[i][2])) for i in range(lo, hi)]
            for i, t in tickets:
                out[i] = srv.wait(t)
        ths = [threading.Thread(target=worker, args=(i * 20, (i + 1) * 20)) for i in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        st = srv.stats()
    assert st["requests"] == len(reqs)
    assert st["batches"] < len(reqs)  # requests were batched together
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    for (q, k, npb), res in zip(reqs, out):
        ids, dist, n, lat = res
        a_ids, a_d, a_n = idx.SearchBatch(q, k, nprobe=npb, mode=mode)
        assert np.array_equal(n, a_n)
        for i in range(q.shape[0]):
            assert np.array_equal(ids[i, :n[i]], a_ids[i, :a_n[i]])
            assert np.array_equal(dist[i, :n[i]], a_d[i, :a_n[i]])


def test_mutations_between_batches(index):
    idx, x, rng = index
    newv = (x[:5] + 1e-3).astype(np.float32)
    with hg.Server(idx, slots=2, max_batch_queries=256, max_k=10, max_nprobe=16) as srv:
        t1 = srv.submit(newv, 1, 16)
        ta = srv.submit_add(np.arange(900000, 900005), newv)
        t2 = srv.submit(newv, 1, 16)
        td = srv.submit_delete([900000, 900001])
        t3 = srv.submit(newv, 1, 16)
        r1, _, r2, r3 = srv.wait(t1), srv.wait(ta), srv.wait(t2), srv.wait(t3)
        srv.wait(td)
        assert srv.stats()["mutations"] == 2
    # before the add: the originals; after it: the added copies (exact rerank
    # distance 0); after the delete: originals for the first two again
    assert (r2[0][:, 0] == np.arange(900000, 900005)).all()
    assert (r3[0][:2, 0] != np.arange(900000, 900002)).all()
    assert (r3[0][2:, 0] == np.arange(900002, 900005)).all()
    idx.BulkDelete(list(range(900000, 900005)))


def test_admission_by_memory_budget(index):
    idx, x, rng = index
    with pytest.raises(hg.HannError, match="memory budget"):
        hg.Server(idx, slots=2, max_batch_queries=4096, memory_budget=1 << 20)
    # a budget that admits about one 256-query batch per slot
    srv = hg.Server(idx, slots=2, max_batch_queries=256, max_k=10, max_nprobe=16, memory_budget=2 * (1 << 20))
    try:
        ts = [srv.submit(rng.normal(size=(64, 32)).astype(np.float32), 10, 16) for _ in range(12)]
        for t in ts:
            srv.wait(t)
        st = srv.stats()
        assert st["peak_admitted_bytes"] <= 2 * (1 << 20)
        assert st["requests"] == 12
    finally:
        srv.stop()
