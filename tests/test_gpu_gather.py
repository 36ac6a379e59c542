"""Gathered distances for graph and tree indexes (hann_knn_distance_gather).

The reference's hnsw and rpt indexes rank candidates one Metric.Rank call at
a time (hnsw/index.go:1178, rpt/index.go:461). The gathered form takes many
(query, candidate list) pairs at once against a base resident on the GPU;
every value must equal, bit for bit, the oracle's reference-order batch
distance (oracle.batch, core/simd_kernels.inc.h:235-264) for the same pair,
for every metric, ragged and empty candidate lists, repeated ids, rows
appended after the base was uploaded, and device buffers."""
import ctypes

import numpy as np
import pytest

import hann_gb300 as hg
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _setup(gpu):
    oracle.set_tier(oracle.TIER_NEON)


def _expected(metric, q, base, cand):
    return oracle.batch(metric, q, base[np.asarray(cand, dtype=np.int64)]) if len(cand) else np.zeros(0)


@pytest.mark.parametrize("metric", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [3, 16, 96, 128])
def test_gather_matches_reference_batch(metric, dim):
    rng = np.random.default_rng(metric * 100 + dim)
    base = rng.standard_normal((3000, dim)).astype(np.float32)
    base[7] = 0  # a zero row (cosine's guarded case)
    q = rng.standard_normal((40, dim)).astype(np.float32)
    # ragged lists: empty, one id, repeats, the zero row, up to 500 ids
    cands = [rng.integers(0, len(base), int(n)) for n in rng.integers(0, 500, len(q))]
    cands[0] = np.zeros(0, np.int64)
    cands[1] = np.array([7])
    cands[2] = np.array([5, 5, 5, 0, len(base) - 1])
    k = hg.KNN(base)
    try:
        got = k.distance_gather(q, cands, metric=metric)
    finally:
        k.close()
    for i in range(len(q)):
        want = _expected(metric, q[i], base, cands[i])
        assert np.array_equal(got[i], want), (metric, dim, i)


def test_gather_after_append_and_bad_ids():
    rng = np.random.default_rng(3)
    base = rng.standard_normal((100, 24)).astype(np.float32)
    more = rng.standard_normal((250, 24)).astype(np.float32)
    k = hg.KNN(base)
    try:
        k.append(more)
        assert k.n == 350
        full = np.concatenate([base, more])
        q = rng.standard_normal((5, 24)).astype(np.float32)
        cands = [np.arange(0, 350, 7), np.array([349]), np.array([0, 100, 101]), np.arange(340, 350), []]
        got = k.distance_gather(q, cands, metric="squared_euclidean")
        for i in range(5):
            assert np.array_equal(got[i], _expected(0, q[i], full, cands[i]))
        # k-NN over the grown base sees the appended rows
        ids, _ = k.search(full[[120, 300]], 1)
        assert ids[:, 0].tolist() == [120, 300]
        for bad in ([350], [-1]):
            with pytest.raises(hg.HannError) as e:
                k.distance_gather(q[:1], [bad])
            assert e.value.code == hg.HANN_E_INVALID
    finally:
        k.close()


def test_gather_device_buffers():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(4)
    base = rng.standard_normal((2000, 64)).astype(np.float32)
    q = rng.standard_normal((30, 64)).astype(np.float32)
    lens = rng.integers(0, 200, len(q))
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    ids = rng.integers(0, len(base), int(offsets[-1])).astype(np.int32)
    k = hg.KNN(base)
    try:
        L = hg.load_library()
        dq = torch.from_numpy(q).cuda()
        doff = torch.from_numpy(offsets).cuda()
        dids = torch.from_numpy(ids).cuda()
        dout = torch.zeros(int(offsets[-1]), dtype=torch.float64, device="cuda")
        stream = torch.cuda.Stream()
        torch.cuda.synchronize()
        rc = L.hann_knn_distance_gather_device(k._h, 3, ctypes.c_void_p(dq.data_ptr()), len(q),
                                               ctypes.c_void_p(doff.data_ptr()), ctypes.c_void_p(dids.data_ptr()),
                                               int(offsets[-1]), ctypes.c_void_p(dout.data_ptr()),
                                               ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.hann_knn_last_error(k._h)
        got = dout.cpu().numpy()
        for i in range(len(q)):
            want = _expected(3, q[i], base, ids[offsets[i]:offsets[i + 1]])
            assert np.array_equal(got[offsets[i]:offsets[i + 1]], want)
    finally:
        k.close()
