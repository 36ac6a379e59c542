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
    """A search sees every mutation whose ticket was waited for before it
    was submitted."""
    idx, x, rng = index
    newv = (x[:5] + 1e-3).astype(np.float32)
    with hg.Server(idx, slots=2, max_batch_queries=256, max_k=10, max_nprobe=16) as srv:
        r1 = srv.wait(srv.submit(newv, 1, 16))
        srv.wait(srv.submit_add(np.arange(900000, 900005), newv))
        r2 = srv.wait(srv.submit(newv, 1, 16))
        srv.wait(srv.submit_delete([900000, 900001]))
        r3 = srv.wait(srv.submit(newv, 1, 16))
        assert srv.stats()["mutations"] == 2
    # before the add: the originals; after it: the added copies (exact rerank
    # distance 0); after the delete: originals for the first two again
    assert not np.isin(r1[0][:, 0], np.arange(900000, 900005)).any()
    assert (r2[0][:, 0] == np.arange(900000, 900005)).all()
    assert (r3[0][:2, 0] != np.arange(900000, 900002)).all()
    assert (r3[0][2:, 0] == np.arange(900002, 900005)).all()
    idx.BulkDelete(list(range(900000, 900005)))


def test_mutations_beside_running_batches(index):
    """Searches and mutations submitted without waiting all complete; every
    search returns full, sorted results; once all are waited for, a search
    sees every mutation."""
    idx, x, rng = index
    added = []
    with hg.Server(idx, slots=3, max_batch_queries=512, max_k=10, max_nprobe=16) as srv:
        tickets = []
        for i in range(40):
            q = rng.normal(size=(int(rng.integers(1, 64)), x.shape[1])).astype(np.float32)
            tickets.append((0, srv.submit(q, 10, 16)))
            if i % 5 == 0:
                ids = np.arange(950000 + 10 * i, 950000 + 10 * i + 10)
                v = (x[rng.integers(0, len(x), 10)] + 1e-3).astype(np.float32)
                added.append((ids, v))
                tickets.append((1, srv.submit_add(ids, v)))
            if i % 7 == 3 and added:
                tickets.append((2, srv.submit_delete(added[0][0][:3])))
        for kind, t in tickets:
            r = srv.wait(t)
            if kind == 0:
                ids, dist, n, _ = r
                assert (n == 10).all()
                assert (np.diff(dist, axis=1) >= 0).all()
        ids0, v0 = added[-1]
        r = srv.wait(srv.submit(v0, 1, 16))
        assert (r[0][:, 0] == ids0).all()
    # BulkDelete skips the ids already deleted (pqivf/index.go:365-367)
    idx.BulkDelete([int(i) for ids, _ in added for i in ids])


def test_admission_by_memory_budget(index):
    idx, x, rng = index
    with pytest.raises(hg.HannError, match="memory budget"):
        hg.Server(idx, slots=2, max_batch_queries=4096, memory_budget=1 << 20)
    # a budget that admits about one 256-query batch per slot (each query's
    # share includes the table scan's 24 KB candidate dump at k 10)
    budget = 16 << 20
    srv = hg.Server(idx, slots=2, max_batch_queries=256, max_k=10, max_nprobe=16, memory_budget=budget)
    try:
        ts = [srv.submit(rng.normal(size=(64, 32)).astype(np.float32), 10, 16) for _ in range(12)]
        for t in ts:
            srv.wait(t)
        st = srv.stats()
        assert st["peak_admitted_bytes"] <= budget
        assert st["requests"] == 12
    finally:
        srv.stop()


def test_priority_and_cancel(index):
    """A high-priority search returns the same results as a normal one; a
    cancelled search either had not started (its wait raises) or had (its
    wait returns its results)."""
    idx, x, rng = index
    q = rng.normal(size=(40, x.shape[1])).astype(np.float32)
    with hg.Server(idx, slots=1, max_batch_queries=64, max_k=10, max_nprobe=16) as srv:
        normal = [srv.submit(q, 10, 16) for _ in range(12)]
        hi = srv.submit(q, 10, 16, priority=1)
        victim = srv.submit(q, 10, 16)
        cancelled = srv.cancel(victim)
        r_hi = srv.wait(hi)
        r_n = srv.wait(normal[-1])
        np.testing.assert_array_equal(r_hi[0], r_n[0])
        np.testing.assert_array_equal(r_hi[1], r_n[1])
        if cancelled:
            with pytest.raises(hg.HannError, match="cancelled"):
                srv.wait(victim)
        else:
            assert (srv.wait(victim)[2] == 10).all()
        for t in normal[:-1]:
            srv.wait(t)
        with pytest.raises(hg.HannError):
            srv.cancel(123456789)


def test_wait_without_results(index):
    """A waiter that wants only the latency gets it without the copies; the
    next request's results are unaffected."""
    idx, x, rng = index
    q = rng.normal(size=(5, 32)).astype(np.float32)
    with hg.Server(idx, slots=2, max_batch_queries=64, max_k=10, max_nprobe=16) as srv:
        ids, dist, n, lat = srv.wait(srv.submit(q, 7, 8), results=False)
        assert ids is None and dist is None and n is None and lat > 0
        ids, dist, n, _ = srv.wait(srv.submit(q, 7, 8))
    want = idx.SearchBatch(q, 7, nprobe=8, mode=hg.MODE_EXACT_RERANK)
    np.testing.assert_array_equal(ids, want[0])


def test_native_replay(index):
    """The native load generator (hann_serve_replay): searches, an add and a
    delete submitted on an arrival schedule; each kept search result equals a
    Search of its queries alone, every request gets a latency and a
    lateness, and rows deleted before a search never come back."""
    idx, x, rng = index
    q = rng.normal(size=(300, 32)).astype(np.float32)
    reqs = np.zeros(60, dtype=hg.Server.REQUEST_DTYPE)
    rows, t, out = [], 0.0, 0
    del_ids = np.arange(100, 160, dtype=np.int64)
    plan = []
    for i in range(len(reqs)):
        t += float(rng.exponential(0.5))
        reqs[i]["at_ms"] = t
        if i == 20:
            reqs[i]["kind"], reqs[i]["first"], reqs[i]["count"] = 2, 0, len(del_ids)
            continue
        nq = int(rng.integers(1, 9))
        reqs[i]["kind"], reqs[i]["k"], reqs[i]["nprobe"] = 0, int(rng.integers(1, 21)), int(rng.integers(1, 33))
        reqs[i]["first"], reqs[i]["count"], reqs[i]["out_offset"] = len(rows), nq, out
        r = rng.integers(0, len(q), nq)
        plan.append((i, r, out))
        rows.extend(r.tolist())
        out += nq * int(reqs[i]["k"])
    with hg.Server(idx, slots=2, max_batch_queries=256, max_k=20, max_nprobe=32, mode=hg.MODE_EXACT_RERANK) as srv:
        lat, late, ids = srv.replay(reqs, q, np.array(rows), del_ids=del_ids, n_out_ids=out)
    assert (lat > 0).all() and (late >= 0).all() and late.max() < 50.0
    for i, r, off in plan:
        k = int(reqs[i]["k"])
        got = ids[off:off + len(r) * k].reshape(len(r), k)
        want, _, _ = idx.SearchBatch(q[r], k, nprobe=int(reqs[i]["nprobe"]), mode=hg.MODE_EXACT_RERANK)
        if i > 20:
            # queued after the delete: it ran on the index without those
            # rows, the state the search alone now sees (the searches before
            # it may or may not have seen the delete)
            assert not (set(got.ravel().tolist()) & set(del_ids.tolist()))
            np.testing.assert_array_equal(got, want)


def test_native_replay_refuses_bad_ranges(index):
    """A schedule naming a query row, an id range or an output slot outside
    its array is refused before anything is submitted."""
    idx, x, rng = index
    q = rng.normal(size=(10, 32)).astype(np.float32)
    with hg.Server(idx, slots=1, max_batch_queries=64, max_k=10, max_nprobe=8) as srv:
        for bad in ("row", "range", "out", "del"):
            reqs = np.zeros(1, dtype=hg.Server.REQUEST_DTYPE)
            reqs[0]["kind"], reqs[0]["k"], reqs[0]["nprobe"], reqs[0]["count"] = 0, 5, 4, 2
            rows = np.array([0, 1])
            n_out = 10
            reqs[0]["out_offset"] = 0
            if bad == "row":
                rows = np.array([0, 10])          # past the 10 query rows
            elif bad == "range":
                reqs[0]["first"] = 1              # rows [1, 3) of 2
            elif bad == "out":
                n_out = 9                         # 2 x 5 ids do not fit
            else:
                reqs[0]["kind"], reqs[0]["count"] = 2, 5  # 5 ids of an empty list
            with pytest.raises(hg.HannError) as e:
                srv.replay(reqs, q, rows, n_out_ids=n_out)
            assert e.value.code == hg.HANN_E_INVALID
        assert srv.stats()["requests"] == 0
