"""Batched exact k-NN on the GPU against the oracle's restatement of
testutil.BruteForceKNN (internal/testutil/data.go:66-93) over the reference's
FP32 batch distances: ids and distances must be identical, for every metric,
on both the exact SIMT path and the tensor-core screen."""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
METRICS = ["squared_euclidean", "euclidean", "manhattan", "cosine"]


def histogram_like(rng, n, dim):
    """Non-negative integers 0-255, 70% zeros, nonzeros geometric with mean 20."""
    x = np.minimum(rng.geometric(1.0 / 20.0, size=(n, dim)), 255).astype(np.float32)
    x[rng.random((n, dim)) < 0.7] = 0.0
    return x


def methods_for(metric, dim):
    out = ["exact", "auto"]
    if metric != "manhattan" and dim <= 128:
        out.append("tensor")
    return out


def check(idx, q, base, k, metric, method):
    ids, dist = idx.search(q, k, metric, method)
    rid, rdist = oracle.knn(q, base, k, metric, nthreads=NT)
    np.testing.assert_array_equal(ids, rid, err_msg=f"{metric}/{method}")
    np.testing.assert_array_equal(dist, rdist, err_msg=f"{metric}/{method}")


@pytest.mark.parametrize("metric", METRICS)
def test_histogram_data_top100(built, gpu, metric):
    import hann_gb300 as hg
    rng = np.random.default_rng(11)
    base = histogram_like(rng, 20000, 128)
    q = histogram_like(rng, 48, 128)
    idx = hg.KNN(base)
    for method in methods_for(metric, 128):
        check(idx, q, base, 100, metric, method)
    idx.close()


@pytest.mark.parametrize("dim", [96, 37, 200, 300])
def test_gaussian_dims(built, gpu, dim):
    import hann_gb300 as hg
    rng = np.random.default_rng(dim)
    base = rng.standard_normal((6000, dim)).astype(np.float32)
    q = rng.standard_normal((33, dim)).astype(np.float32)
    idx = hg.KNN(base)
    for metric in METRICS:
        for method in methods_for(metric, dim):
            for k in (1, 10, 64):
                check(idx, q, base, k, metric, method)
    idx.close()


def test_tensor_rejects_manhattan_and_wide(built, gpu):
    import hann_gb300 as hg
    rng = np.random.default_rng(3)
    idx = hg.KNN(rng.standard_normal((100, 16)).astype(np.float32))
    with pytest.raises(hg.HannError):
        idx.search(rng.standard_normal((2, 16)).astype(np.float32), 5, "manhattan", "tensor")
    wide = hg.KNN(rng.standard_normal((100, 130)).astype(np.float32))
    with pytest.raises(hg.HannError):
        wide.search(rng.standard_normal((2, 130)).astype(np.float32), 5, "squared_euclidean", "tensor")
    with pytest.raises(hg.HannError):
        idx.search(rng.standard_normal((2, 16)).astype(np.float32), 0)


def test_fewer_rows_than_k(built, gpu):
    import hann_gb300 as hg
    rng = np.random.default_rng(5)
    base = rng.standard_normal((50, 24)).astype(np.float32)
    q = rng.standard_normal((7, 24)).astype(np.float32)
    idx = hg.KNN(base)
    for metric in METRICS:
        for method in methods_for(metric, 24):
            ids, dist = idx.search(q, 80, metric, method)
            assert (ids[:, 50:] == -1).all() and np.isinf(dist[:, 50:]).all()
            check(idx, q, base, 80, metric, method)


def test_empty_base_and_empty_vectors(built, gpu):
    import hann_gb300 as hg
    empty = hg.KNN(np.zeros((0, 8), np.float32))
    ids, dist = empty.search(np.ones((3, 8), np.float32), 4)
    assert (ids == -1).all() and np.isinf(dist).all()
    flat0 = hg.KNN(np.zeros((5, 0), np.float32))
    ids, dist = flat0.search(np.zeros((2, 0), np.float32), 3)
    np.testing.assert_array_equal(ids, [[0, 1, 2]] * 2)
    assert (dist == 0).all()


def test_ties_broken_by_row(built, gpu):
    """Thousands of rows at the same distance: the lowest rows win."""
    import hann_gb300 as hg
    rng = np.random.default_rng(8)
    base = histogram_like(rng, 30000, 64)
    q = histogram_like(rng, 4, 64)
    base[1000:6000] = q[0]          # exact duplicates of query 0 (distance 0)
    base[9000:20000] = base[9000]   # one vector repeated 11000 times
    q[1] = base[9000]
    idx = hg.KNN(base)
    for metric in METRICS:
        for method in methods_for(metric, 64):
            check(idx, q, base, 100, metric, method)
    st = idx.stats()
    # the duplicated blocks fill the screen's band: those queries finish exactly
    assert st["fallback_queries"] > 0


def test_zero_vectors_cosine(built, gpu):
    """Zero norm gives cosine distance 1 (core/simd_kernels.inc.h:220-228)."""
    import hann_gb300 as hg
    rng = np.random.default_rng(9)
    base = rng.standard_normal((5000, 32)).astype(np.float32)
    base[::7] = 0.0
    q = rng.standard_normal((6, 32)).astype(np.float32)
    q[2] = 0.0
    idx = hg.KNN(base)
    for method in ("exact", "tensor"):
        check(idx, q, base, 50, "cosine", method)
        ids, dist = idx.search(q, 50, "cosine", method)
        np.testing.assert_array_equal(ids[2], np.arange(50))
        assert (dist[2] == 1.0).all()


def test_candidate_overflow_reruns_chunk(built, gpu):
    """Rows ordered from far to near: every later chunk beats the current
    k-th neighbour everywhere, so its candidates overflow and the chunk is
    rerun in pieces."""
    import hann_gb300 as hg
    rng = np.random.default_rng(10)
    base = rng.standard_normal((60000, 16)).astype(np.float32)
    q = rng.standard_normal((3, 16)).astype(np.float32)
    d = ((base - q[0]) ** 2).sum(1)
    base = base[np.argsort(-d, kind="stable")].copy()
    idx = hg.KNN(base)
    for metric in METRICS:
        check(idx, q, base, 100, metric, "exact")
    assert idx.stats()["redo_chunks"] > 0
    for metric in ("squared_euclidean", "cosine"):
        check(idx, q, base, 100, metric, "tensor")


def test_more_queries_than_one_block(built, gpu):
    import hann_gb300 as hg
    rng = np.random.default_rng(12)
    base = rng.standard_normal((1500, 20)).astype(np.float32)
    q = rng.standard_normal((8200, 20)).astype(np.float32)
    idx = hg.KNN(base)
    check(idx, q, base, 10, "squared_euclidean", "tensor")
    check(idx, q, base, 10, "manhattan", "exact")


def test_one_shot_and_matrix(built, gpu):
    import hann_gb300 as hg
    rng = np.random.default_rng(13)
    base = histogram_like(rng, 3000, 48)
    q = histogram_like(rng, 5, 48)
    ids, dist = hg.knn(q, base, 20, "cosine")
    rid, rdist = oracle.knn(q, base, 20, "cosine")
    np.testing.assert_array_equal(ids, rid)
    np.testing.assert_array_equal(dist, rdist)
    for m, name in enumerate(METRICS):
        mat = hg.distance_matrix(name, q, base)
        for i in range(q.shape[0]):
            np.testing.assert_array_equal(mat[i], oracle.batch(m, q[i], base))


def test_device_entry_point(built, gpu):
    torch = pytest.importorskip("torch")
    import hann_gb300 as hg
    rng = np.random.default_rng(14)
    base = rng.standard_normal((4000, 64)).astype(np.float32)
    q = rng.standard_normal((40, 64)).astype(np.float32)
    idx = hg.KNN(base)
    dq = torch.from_numpy(q).cuda()
    ids = torch.empty((40, 16), dtype=torch.int64, device="cuda")
    dist = torch.empty((40, 16), dtype=torch.float64, device="cuda")
    idx.search_device(dq.data_ptr(), 40, 16, ids.data_ptr(), dist.data_ptr(), "euclidean", "tensor",
                      torch.cuda.current_stream().cuda_stream)
    rid, rdist = oracle.knn(q, base, 16, "euclidean")
    np.testing.assert_array_equal(ids.cpu().numpy(), rid)
    np.testing.assert_array_equal(dist.cpu().numpy(), rdist)
