"""The allocation-free batch search entry point.

hann_pqivf_search_batch_device_noalloc is for callers that cannot allocate
device memory while they search (latency-bound serving threads that must not
stall on an allocator synchronisation, code recording a CUDA graph, processes
with a device-memory budget fixed at start-up). Its scratch is one fixed
16 MiB device array inside the library. These tests call it through the C
ABI and check it against hann_pqivf_search_batch_device, the entry point it
mirrors, on two calls in a row (the array keeps the previous call's contents),
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
        idx.SearchBatchDevice(q.data_ptr(), nq, k, nprobe, mode, ref_ids.data_ptr(), ref_d.data_ptr(),
                              ref_n.data_ptr(), stream)
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
