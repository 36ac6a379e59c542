"""The device-buffer entry points at the C ABI: brute-force fallbacks counted
in Stats (pqivf/index.go:892-894), mutations ordered after the searches a
caller enqueued on its own stream, and the nprobe-from-recall tuner called
directly through hann_pqivf_tune_candidate_clusters."""
import ctypes

import numpy as np
import pytest

import hann_gb300 as hg
from tests.helpers import assert_same_results, gaussian_mixture

pytestmark = pytest.mark.gpu

_P = ctypes.c_void_p


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _device_search(torch, idx, q, k, nprobe, mode, stream):
    nq = q.shape[0]
    ids = torch.full((nq, k), -7, dtype=torch.int64, device="cuda")
    d = torch.zeros((nq, k), dtype=torch.float64, device="cuda")
    n = torch.zeros(nq, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    idx.SearchBatchDevice(q.data_ptr(), nq, k, nprobe, mode, ids.data_ptr(), d.data_ptr(), n.data_ptr(), stream)
    return ids, d, n


def test_device_search_counts_fallbacks(gpu):
    """Queries whose probed lists hold fewer than k rows fall back to every
    list; the device entry point counts them like the host call does."""
    torch = _torch()
    rng = np.random.default_rng(5)
    x, _ = gaussian_mixture(rng, 4000, 16, 40, 0.3)
    idx = hg.New(16, hg.WithCoarseK(64), hg.WithNumSubquantizers(4), hg.WithPQK(16), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(len(x)), x)
    idx.Train()
    q = x[rng.integers(0, len(x), 300)] + 0.05
    k = 150  # above most single lists' length: nprobe 1 falls back
    before = idx.Stats().FallbackSearches
    hi, hd, hn = idx.SearchBatch(q, k, nprobe=1, mode=0)
    host_fb = idx.Stats().FallbackSearches - before
    assert host_fb > 0
    qd = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float32)).cuda()
    stream = torch.cuda.Stream()
    di, dd, dn = _device_search(torch, idx, qd, k, 1, 0, stream.cuda_stream)
    # Stats waits for the searches enqueued on the caller's stream
    dev_fb = idx.Stats().FallbackSearches - before - host_fb
    assert dev_fb == host_fb
    torch.cuda.synchronize()
    assert_same_results(di.cpu().numpy(), dd.cpu().numpy(), dn.cpu().numpy(), hi, hd, hn)
    idx.close()


def test_mutation_waits_for_enqueued_device_search(gpu):
    """A BulkAdd that moves rows (a list outgrows its room) issued right after
    a device search was enqueued on a caller's stream waits for that search:
    its results equal those of the same search run alone."""
    torch = _torch()
    rng = np.random.default_rng(9)
    x, cent = gaussian_mixture(rng, 40000, 32, 64, 0.4)
    idx = hg.New(32, hg.WithCoarseK(64), hg.WithNumSubquantizers(8), hg.WithPQK(64), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(len(x)), x)
    idx.Train()
    q = np.ascontiguousarray(x[rng.integers(0, len(x), 20000)] + 0.01 * rng.normal(size=(20000, 32)),
                             dtype=np.float32)
    qd = torch.from_numpy(q).cuda()
    k, nprobe = 10, 64
    stream = torch.cuda.Stream()
    ai, ad, an = _device_search(torch, idx, qd, k, nprobe, 1, stream.cuda_stream)
    torch.cuda.synchronize()
    alone = (ai.cpu().numpy(), ad.cpu().numpy(), an.cpu().numpy())
    arena_before = np.zeros(5, dtype=np.int64)
    L = hg.load_library()
    L.hann_pqivf_arena_stats(idx.handle, arena_before.ctypes.data)
    # enqueue the long search, then at once add 20,000 vectors around one
    # centre: their list must move (or every list be laid out again)
    bi, bd, bn = _device_search(torch, idx, qd, k, nprobe, 1, stream.cuda_stream)
    extra = (cent[3] + 0.01 * rng.normal(size=(20000, 32))).astype(np.float32)
    idx.BulkAddArrays(np.arange(len(x), len(x) + len(extra)), extra)
    torch.cuda.synchronize()
    arena_after = np.zeros(5, dtype=np.int64)
    L.hann_pqivf_arena_stats(idx.handle, arena_after.ctypes.data)
    assert arena_after[3] + arena_after[4] > arena_before[3] + arena_before[4], "no row moved"
    assert_same_results(bi.cpu().numpy(), bd.cpu().numpy(), bn.cpu().numpy(), *alone)
    idx.close()


def test_tune_through_c_abi(gpu):
    """hann_pqivf_tune_candidate_clusters with an explicit ladder and given
    ground truth: the recall it reports for each nprobe equals the recall of
    hann_pqivf_search_batch at that nprobe, it stops at the first value that
    reaches the target, and apply sets the default nprobe."""
    rng = np.random.default_rng(21)
    x, _ = gaussian_mixture(rng, 12000, 32, 400, 0.4)
    idx = hg.New(32, hg.WithCoarseK(256), hg.WithNumSubquantizers(8), hg.WithPQK(32), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(len(x)), x)
    idx.Train()
    q = np.ascontiguousarray(x[rng.integers(0, len(x), 64)] + 0.05 * rng.normal(size=(64, 32)), dtype=np.float32)
    k = 10
    st = idx.export_state()
    rows, _ = hg.knn(q, st["vectors"], k)
    gt = np.ascontiguousarray(np.asarray(st["ids"])[rows], dtype=np.int64)

    def recall_at(p):
        ids, _, n = idx.SearchBatch(q, k, nprobe=p, mode=1)
        return sum(len(set(ids[i, :n[i]].tolist()) & set(gt[i].tolist())) for i in range(len(q))) / gt.size

    ladder = np.array([1, 2, 4, 8, 16, 32, 64, 128, 256], dtype=np.int32)
    rec_by = {int(p): recall_at(int(p)) for p in ladder}
    target = rec_by[16] - 1e-9
    expect = next(int(p) for p in ladder if rec_by[int(p)] >= target)
    L = hg.load_library()
    chosen = ctypes.c_int32(0)
    ntried = ctypes.c_int32(0)
    tried = np.zeros(len(ladder), dtype=np.int32)
    rec = np.zeros(len(ladder), dtype=np.float64)
    rc = L.hann_pqivf_tune_candidate_clusters(idx.handle, _P(q.ctypes.data), len(q), k, target,
                                              _P(ladder.ctypes.data), len(ladder), 1, _P(gt.ctypes.data), 1,
                                              ctypes.byref(chosen), _P(tried.ctypes.data), _P(rec.ctypes.data),
                                              ctypes.byref(ntried))
    assert rc == 0, L.hann_pqivf_last_error(idx.handle)
    assert chosen.value == expect
    assert ntried.value == list(ladder).index(expect) + 1
    for i in range(ntried.value):
        assert tried[i] == ladder[i]
        assert rec[i] == pytest.approx(rec_by[int(ladder[i])], abs=1e-12)
    # applied: Search without nprobe uses the chosen value
    a = idx.SearchBatch(q[:8], k, mode=1)
    b = idx.SearchBatch(q[:8], k, nprobe=expect, mode=1)
    np.testing.assert_array_equal(a[0], b[0])
    # without ground truth the library computes it from the stored vectors
    chosen2 = ctypes.c_int32(0)
    rc = L.hann_pqivf_tune_candidate_clusters(idx.handle, _P(q.ctypes.data), len(q), k, target,
                                              _P(ladder.ctypes.data), len(ladder), 1, None, 0,
                                              ctypes.byref(chosen2), None, None, None)
    assert rc == 0, L.hann_pqivf_last_error(idx.handle)
    assert chosen2.value == expect
    # invalid arguments are refused
    assert L.hann_pqivf_tune_candidate_clusters(idx.handle, _P(q.ctypes.data), len(q), 0, 0.9, None, 0, 1, None,
                                                0, ctypes.byref(chosen2), None, None, None) == hg.HANN_E_INVALID
    idx.close()
