"""The subquantizer assignment of training's k-means (launch_pq_assign, the
packed FP32x2 kernel for sub-dimensions 4, 8 and 16 and the scalar kernels
for the others) against the oracle's assignPoints (pqivf/index.go:738-789)
on each subquantizer's columns: every row's codeword must be the oracle's,
bit for bit, with ties to the lower index (duplicate codewords, rows equal
to a codeword), rows of NaN and infinities, odd row counts (the packed
kernel's unpaired last row) and codebooks of 1 to 256 codewords."""
import ctypes

import numpy as np
import pytest

import hann_gb300 as hg
import oracle

pytestmark = pytest.mark.gpu
_P = ctypes.c_void_p


@pytest.fixture(scope="module", autouse=True)
def _setup(gpu):
    oracle.set_tier(oracle.TIER_NEON)


def gpu_assign(res, cbs):
    L = hg.load_library()
    f = L.hann_gpu_pq_assign
    f.argtypes = [_P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P, ctypes.c_int32, _P]
    n = res.shape[0]
    M, K, ds = cbs.shape
    res = np.ascontiguousarray(res, dtype=np.float32)
    cbs = np.ascontiguousarray(cbs, dtype=np.float32)
    out = np.full((n, M), -1, np.int32)
    rc = f(_P(res.ctypes.data), n, M, ds, _P(cbs.ctypes.data), K, _P(out.ctypes.data))
    assert rc == 0
    return out


def oracle_assign(res, cbs):
    M, _, ds = cbs.shape
    return np.stack([oracle.assign(np.ascontiguousarray(res[:, m * ds:(m + 1) * ds]), cbs[m], 8) for m in range(M)],
                    axis=1)


@pytest.mark.parametrize("ds", [1, 2, 3, 4, 8, 12, 16, 32])
@pytest.mark.parametrize("K", [1, 7, 256])
@pytest.mark.parametrize("n", [1, 2, 513, 3001])
def test_pq_assign_matches_oracle(ds, K, n):
    rng = np.random.default_rng(ds * 1000 + K * 10 + n)
    M = max(1, 64 // ds) if ds <= 16 else 2
    res = rng.standard_normal((n, M * ds)).astype(np.float32)
    cbs = rng.standard_normal((M, K, ds)).astype(np.float32)
    if K > 2:
        cbs[:, K - 1] = cbs[:, 1]  # a duplicate codeword: the lower index wins
    if n > 3:
        res[0, :ds] = cbs[0, min(1, K - 1)]  # a row equal to a codeword (distance 0, tied with its duplicate)
        res[1] = np.nan
        res[2, :ds] = np.inf
    got = gpu_assign(res, cbs)
    want = oracle_assign(res, cbs)
    assert np.array_equal(got, want), np.argwhere(got != want)[:5]


def test_pq_assign_near_ties():
    """Codewords one ulp apart around each row, magnitudes from 1e-20 to
    1e15: the chosen index follows the exact FP32 distances of the
    reference's summation order."""
    rng = np.random.default_rng(5)
    for ds in (4, 8, 16):
        M, K, n = 4, 256, 4001
        scale = np.float32(10.0) ** rng.integers(-20, 16, (n, 1)).astype(np.float32)
        res = (rng.standard_normal((n, M * ds)) * scale).astype(np.float32)
        base = rng.standard_normal((M, 1, ds)).astype(np.float32)
        cbs = np.repeat(base, K, axis=1)
        cbs = np.nextafter(cbs, np.float32(np.inf) * np.sign(rng.standard_normal(cbs.shape))).astype(np.float32)
        cbs[:, ::3] = base
        got = gpu_assign(res, cbs)
        want = oracle_assign(res, cbs)
        assert np.array_equal(got, want), (ds, np.argwhere(got != want)[:5])
