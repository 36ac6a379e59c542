"""The allocation-free batch search entry point.

hann_pqivf_search_batch_device_noalloc is for callers that cannot allocate
device memory while they search (latency-bound serving threads that must not
stall on an allocator synchronisation, code recording a CUDA graph, processes
with a device-memory budget fixed at start-up). Its scratch is one fixed
16 MiB device array inside the library. These tests call it through the C
ABI and check it against hann_pqivf_search_batch_device, the entry point it
mirrors, on two calls in a row (the array keeps the previous call's contents),
on a batch that fills the array to within one query of its end, on queries
that take the brute-force fallback (counted in Stats like the mirrored call's),
and check that an oversized batch is refused with an error instead of running.
This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

import hann_gb300 as hg
from tests.helpers import assert_same_results

pytestmark = pytest.mark.gpu

_P = ctypes.c_void_p


def _noalloc_fn():
    L = hg.load_library()
    f = L.hann_pqivf_search_batch_device_noalloc
    f.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P, _P]
    f.restype = ctypes.c_int
    return L, f


@pytest.fixture(scope="module")
def index(gpu):
    rng = np.random.default_rng(2024)
    x = rng.normal(size=(20000, 32)).astype(np.float32)
    idx = hg.New(32, hg.WithCoarseK(64), hg.WithNumSubquantizers(8), hg.WithPQK(64), hg.WithKMeansIters(5),
                 hg.WithCandidateClusters(6))
    idx.BulkAddArrays(np.arange(20000), x)
    idx.Train()
    yield idx, rng
    idx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_noalloc_matches_device_search_two_calls(index, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    idx, rng = index
    L, noalloc = _noalloc_fn()
    k, nprobe = 10, 6
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        nq = 300 if call == 0 else 170
        q = torch.from_numpy(rng.normal(size=(nq, 32)).astype(np.float32)).cuda()
        ref_ids = torch.full((nq, k), -7, dtype=torch.int64, device="cuda")
        ref_d = torch.zeros((nq, k), dtype=torch.float64, device="cuda")
        ref_n = torch.zeros(nq, dtype=torch.int32, device="cuda")
        got_ids = torch.full((nq, k), -7, dtype=torch.int64, device="cuda")
        got_d = torch.zeros((nq, k), dtype=torch.float64, device="cuda")
        got_n = torch.zeros(nq, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()  # the fills above ran on torch's stream
        # The allocation-free call runs the table scan. With the exact rerank
        # the list-major scan may hand different candidates to the rerank at
        # the rerank depth, so that mode is compared with the device entry
        # point running the table scan too; the reference's PQ distances
        # (mode 0) agree whichever scan runs.
        if mode == 1:
            idx.ScanOptions(list_major=0)
        try:
            idx.SearchBatchDevice(q.data_ptr(), nq, k, nprobe, mode, ref_ids.data_ptr(), ref_d.data_ptr(),
                                  ref_n.data_ptr(), stream)
            torch.cuda.synchronize()
        finally:
            idx.ScanOptions(list_major=1)
        rc = noalloc(idx.handle, _P(q.data_ptr()), nq, k, nprobe, mode, _P(got_ids.data_ptr()),
                     _P(got_d.data_ptr()), _P(got_n.data_ptr()), _P(stream))
        assert rc == 0, L.hann_pqivf_last_error(idx.handle)
        torch.cuda.synchronize()
        ri, rd, rn = ref_ids.cpu().numpy(), ref_d.cpu().numpy(), ref_n.cpu().numpy()
        gi, gd, gn = got_ids.cpu().numpy(), got_d.cpu().numpy(), got_n.cpu().numpy()
        assert (gn == k).all()
        assert_same_results(gi, gd, gn, ri, rd, rn)


def test_noalloc_rejects_oversized_batch(index):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    idx, _ = index
    L, noalloc = _noalloc_fn()
    nq = 100_000  # 100k x 64 lists of coarse distances alone exceed 16 MiB
    q = torch.zeros((nq, 32), dtype=torch.float32, device="cuda")
    ids = torch.empty((nq, 10), dtype=torch.int64, device="cuda")
    d = torch.empty((nq, 10), dtype=torch.float64, device="cuda")
    n = torch.empty(nq, dtype=torch.int32, device="cuda")
    rc = noalloc(idx.handle, _P(q.data_ptr()), nq, 10, 6, 0, _P(ids.data_ptr()), _P(d.data_ptr()),
                 _P(n.data_ptr()), _P(0))
    assert rc == hg.HANN_E_UNSUPPORTED
    assert b"arena" in L.hann_pqivf_last_error(idx.handle)


ARENA = 16 << 20


def _scratch_bytes(nq, nlist, nprobe, R):
    """The entry point's scratch layout: every region rounded to 256 bytes
    (the parity-mode proof's cut, bound and rescan list included)."""
    a = lambda b: (b + 255) // 256 * 256  # noqa: E731
    return (a(nq * nlist * 4) + 2 * a(nq * nprobe * 4) + 5 * a(nq * 4) + 3 * a(nq * R * 4)
            + a((nq + 1) * 4))


def _compare(idx, L, noalloc, q, k, nprobe, mode, stream, torch):
    nq = q.shape[0]
    outs = []
    for use_noalloc in (False, True):
        ids = torch.full((nq, k), -7, dtype=torch.int64, device="cuda")
        d = torch.zeros((nq, k), dtype=torch.float64, device="cuda")
        n = torch.zeros(nq, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        if use_noalloc:
            rc = noalloc(idx.handle, _P(q.data_ptr()), nq, k, nprobe, mode, _P(ids.data_ptr()), _P(d.data_ptr()),
                         _P(n.data_ptr()), _P(stream))
            assert rc == 0, L.hann_pqivf_last_error(idx.handle)
        else:
            idx.SearchBatchDevice(q.data_ptr(), nq, k, nprobe, mode, ids.data_ptr(), d.data_ptr(), n.data_ptr(),
                                  stream)
        torch.cuda.synchronize()
        outs.append((ids.cpu().numpy(), d.cpu().numpy(), n.cpu().numpy()))
    assert_same_results(*outs[1], *outs[0])
    return outs


def test_noalloc_batch_filling_the_arena(index):
    """The largest batch whose scratch fits: the last region ends within one
    query's share of the array's end."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    idx, rng = index
    L, noalloc = _noalloc_fn()
    k, nprobe, nlist, R = 10, 6, 64, 64  # R: rerank depth of k 10 (k + 32, rounded up to 32)
    nq = ARENA // (4 * nlist)
    while _scratch_bytes(nq, nlist, nprobe, R) > ARENA:
        nq -= 1
    assert ARENA - _scratch_bytes(nq, nlist, nprobe, R) < _scratch_bytes(1, nlist, nprobe, R) + 10 * 256
    q = torch.from_numpy(rng.normal(size=(nq, 32)).astype(np.float32)).cuda()
    _compare(idx, L, noalloc, q, k, nprobe, 0, torch.cuda.current_stream().cuda_stream, torch)
    # one query more no longer fits and is refused
    q1 = torch.zeros((nq + 1, 32), dtype=torch.float32, device="cuda")
    ids = torch.empty((nq + 1, k), dtype=torch.int64, device="cuda")
    d = torch.empty((nq + 1, k), dtype=torch.float64, device="cuda")
    n = torch.empty(nq + 1, dtype=torch.int32, device="cuda")
    rc = noalloc(idx.handle, _P(q1.data_ptr()), nq + 1, k, nprobe, 0, _P(ids.data_ptr()), _P(d.data_ptr()),
                 _P(n.data_ptr()), _P(0))
    assert rc == hg.HANN_E_UNSUPPORTED


def test_noalloc_fallback_queries(gpu):
    """Lists emptied by deletions: queries whose probed list holds fewer than
    k rows scan every list (the brute-force fallback), with the same results
    and the same FallbackSearches count as the mirrored call."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(77)
    x = rng.normal(size=(6000, 16)).astype(np.float32)
    idx = hg.New(16, hg.WithCoarseK(64), hg.WithNumSubquantizers(4), hg.WithPQK(16), hg.WithKMeansIters(4))
    idx.BulkAddArrays(np.arange(len(x)), x)
    idx.Train()
    st = idx.export_state()
    lens = np.asarray(st["list_len"])
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    # empty every other list
    dead = np.concatenate([st["ids"][starts[c]:starts[c] + lens[c]] for c in range(0, len(lens), 2)])
    idx.BulkDelete(dead.tolist())
    L, noalloc = _noalloc_fn()
    k = 120
    q = torch.from_numpy(rng.normal(size=(200, 16)).astype(np.float32)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    f0 = idx.Stats().FallbackSearches
    outs = _compare(idx, L, noalloc, q, k, 1, 0, stream, torch)
    f1 = idx.Stats().FallbackSearches
    assert (outs[1][2] == k).all()  # every query found k rows: the fallback ran
    assert f1 > f0 and (f1 - f0) % 2 == 0  # the same count from each entry point
    outs2 = _compare(idx, L, noalloc, q, k, 1, 0, stream, torch)
    assert (f1 - f0) == (idx.Stats().FallbackSearches - f1)
    for a, b in zip(outs[1], outs2[1]):
        np.testing.assert_array_equal(a, b)
    idx.close()
