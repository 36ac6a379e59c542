"""Scenarios of concurrent use of one index handle (pqivf/concurrency_test.go,
internal/testutil/concurrent.go:19-118) and of failed updates that keep
their entries (pqivf/index_test.go:455-500). Python threads call the C ABI,
which releases the interpreter lock, so the handle's own locks order the
calls.

Run as a program (`python -m tests.concurrency_scenarios [name ...]`), one
JSON line per scenario as it ends; tests/test_zy_gpu_concurrency.py runs
it in a child process, so that a crash or a deadlock in one scenario fails
that test alone instead of ending the test session."""
import io
import json
import os
import random
import sys
import threading
import traceback

import numpy as np
import pytest

import hann_gb300 as hg
from tests.helpers import gaussian_mixture

DEADLINE_S = 30.0


def new_index(dim, coarse_k, m, pqk, iters, *more):
    return hg.New(dim, hg.WithCoarseK(coarse_k), hg.WithNumSubquantizers(m), hg.WithPQK(pqk),
                  hg.WithKMeansIters(iters), *more)


def make_vec(i):
    return [float(i + j) for j in range(6)]


def run_threads(fns, workers=16):
    """Runs the callables on `workers` daemon threads; raises the first
    failure, or fails when they do not finish by the deadline (a deadlock
    leaves only daemon threads behind)."""
    errors, lock = [], threading.Lock()
    it = iter(list(fns))

    def worker():
        while True:
            with lock:
                f = next(it, None)
            if f is None:
                return
            try:
                f()
            except BaseException as e:  # noqa: BLE001 - reported below
                with lock:
                    errors.append(e)
                return

    ts = [threading.Thread(target=worker, daemon=True) for _ in range(workers)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(DEADLINE_S)
    assert not any(t.is_alive() for t in ts), "concurrent calls did not finish: the handle deadlocked"
    if errors:
        raise errors[0]


def scenario_concurrent_adds():
    """TestPQIVF_ConcurrentOperations (concurrency_test.go:12-45)."""
    idx = new_index(6, 3, 2, 256, 10)
    run_threads([lambda i=i: idx.Add(i, make_vec(i)) for i in range(1000)])
    assert idx.Stats().Count == 1000


def scenario_concurrent_save_add():
    """TestPQIVF_ConcurrentSaveAdd (concurrency_test.go:47-95): Saves beside
    Adds finish, and every saved stream is a whole index."""
    idx = new_index(6, 3, 2, 256, 10)
    idx.BulkAddArrays(np.arange(2000), np.asarray([make_vec(i) for i in range(2000)], np.float32))
    saved = []

    def save():
        buf = io.BytesIO()
        idx.Save(buf)
        saved.append(buf.getvalue())

    fns = []
    for i in range(200):
        fns.append(save)
        fns.append(lambda i=i: idx.Add(10_000 + i, make_vec(10_000 + i)))
    run_threads(fns)
    assert idx.Stats().Count == 2200
    assert len(saved) == 200
    for data in saved[::20]:
        st = hg.gob_decode_state(data)
        assert st["layout"]["dimension"] == 6
        assert 2000 <= st["layout"]["n_pending"] <= 2200
        assert np.array_equal(st["pending_ids"][:2000], np.arange(2000))


def scenario_concurrent_update_search():
    """TestPQIVF_ConcurrentUpdateSearch (concurrency_test.go:97-141): the
    index stays trained, so every search succeeds while updates run."""
    idx = new_index(6, 3, 2, 256, 10, hg.WithSeed(42))
    idx.BulkAddArrays(np.arange(100), np.asarray([make_vec(i) for i in range(100)], np.float32))
    idx.Train()
    query = make_vec(50)
    found = []

    def search():
        found.append(len(idx.Search(query, 1)))

    fns = []
    for i in range(50):
        fns.append(lambda i=i: idx.Update(i, make_vec(i + 1000)))
        fns.append(search)
    run_threads(fns)
    assert found == [1] * 50
    assert idx.Stats().Count == 100


def scenario_atomic_update_vs_add():
    """TestPQIVF_AtomicUpdateVsAdd (concurrency_test.go:143-184): an Update
    of a live id never fails while Adds of the same id race with it, and
    every such Add fails."""
    idx = new_index(4, 2, 2, 4, 5)
    idx.Add(7, [1, 1, 1, 1])

    def updates():
        for i in range(500):
            idx.Update(7, [float(i), 2, 3, 4])

    def adds():
        for i in range(500):
            with pytest.raises(hg.HannError, match="already exists"):
                idx.Add(7, [9, 9, 9, 9])

    run_threads([updates, adds], workers=2)
    assert idx.Stats().Count == 1


def scenario_concurrent_stress():
    """TestPQIVF_ConcurrentStress: RunConcurrentOps(dim 16, 8 workers, 300
    operations each) over newIndex(16, 2, 2, 4, 5) seeded with 100 clustered
    vectors and trained (internal/testutil/concurrent.go:19-118)."""
    dim, workers, ops = 16, 8, 300
    idx = new_index(dim, 2, 2, 4, 5)
    seed, _ = gaussian_mixture(np.random.default_rng(1), 100, dim, 4, 0.3)
    idx.BulkAddArrays(np.arange(100), seed.astype(np.float32))
    idx.Train()
    live = [0] * workers

    def worker(w):
        rng = random.Random(w + 1)
        base = 1000 * (w + 1)
        present = set()
        for _ in range(ops):
            i = base + rng.randrange(32)
            action = rng.randrange(10)
            vec = [rng.uniform(-5, 5) for _ in range(dim)]
            if action < 4 and i not in present:
                idx.Add(i, vec)
                present.add(i)
            elif action < 6 and i in present:
                idx.Update(i, vec)
            elif action == 6 and i in present:
                idx.Delete(i)
                present.discard(i)
            elif action == 7:
                idx.Save(io.BytesIO())
            else:
                try:  # errors in transient states are tolerated, as the reference does
                    idx.Search(vec, 5)
                except hg.HannError:
                    pass
        live[w] = len(present)

    run_threads([lambda w=w: worker(w) for w in range(workers)], workers=workers)
    assert idx.Stats().Count == 100 + sum(live)


def scenario_update_failure_keeps_entry():
    """TestPQIVF_UpdateFailureKeepsEntry (index_test.go:455-476)."""
    idx = new_index(4, 2, 2, 256, 5)
    idx.Add(1, [1, 1, 1, 1])
    with pytest.raises(hg.HannError):
        idx.Update(1, [1, 2, 3])
    assert idx.Stats().Count == 1
    idx.Update(1, [2, 2, 2, 2])
    assert idx.Stats().Count == 1


def scenario_bulk_update_failure_keeps_entries():
    """TestPQIVF_BulkUpdateFailureKeepsEntries (index_test.go:478-500)."""
    idx = new_index(4, 2, 2, 256, 5)
    idx.BulkAdd({1: [1, 1, 1, 1], 2: [2, 2, 2, 2]})
    with pytest.raises(hg.HannError):
        idx.BulkUpdate({1: [3, 3, 3, 3], 2: [1, 2, 3]})
    assert idx.Stats().Count == 2


SCENARIOS = {name[len("scenario_"):]: fn for name, fn in sorted(globals().items()) if name.startswith("scenario_")}


def main(names):
    for name in names or sorted(SCENARIOS):
        try:
            SCENARIOS[name]()
            line = {"name": name, "ok": True}
        except BaseException as e:  # noqa: BLE001 - reported to the parent
            line = {"name": name, "ok": False, "error": "".join(traceback.format_exception_only(type(e), e)).strip()}
        print(json.dumps(line), flush=True)
    sys.stdout.flush()
    os._exit(0)  # threads left behind by a deadlocked scenario must not keep the process alive


if __name__ == "__main__":
    main(sys.argv[1:])
