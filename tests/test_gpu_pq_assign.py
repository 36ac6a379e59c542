"""The subquantizer assignment of training's k-means (launch_pq_assign, the
packed FP32x2 kernel for sub-dimensions 4, 8 and 16 and the scalar kernels
for the others) against the oracle's assignPoints (pqivf/index.go:738-789)
on each subquantizer's columns: every row's codeword must be the oracle's,
bit for bit, with ties to the lower index (duplicate codewords, rows equal
to a codeword), rows of NaN and infinities, odd row counts (the packed
kernel's unpaired last row) and codebooks of 1 to 256 codewords; and the
k-means update's FP64 sums and counts that training accumulates with the
assignment (diagnostic entry point hann_gpu_pq_assign)."""
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


def gpu_assign(res, cbs, with_sums=False):
    L = hg.load_library()
    f = L.hann_gpu_pq_assign
    f.argtypes = [_P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P, ctypes.c_int32, _P, _P, _P]
    n = res.shape[0]
    M, K, ds = cbs.shape
    res = np.ascontiguousarray(res, dtype=np.float32)
    cbs = np.ascontiguousarray(cbs, dtype=np.float32)
    out = np.full((n, M), -1, np.int32)
    sums = np.full((M, K, ds), np.nan) if with_sums else None
    counts = np.full((M, K), -1, np.int64) if with_sums else None
    rc = f(_P(res.ctypes.data), n, M, ds, _P(cbs.ctypes.data), K, _P(out.ctypes.data),
           _P(sums.ctypes.data) if with_sums else None, _P(counts.ctypes.data) if with_sums else None)
    assert rc == 0
    return (out, sums, counts) if with_sums else out


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


@pytest.mark.parametrize("ds", [4, 8, 16])
def test_pq_assign_rounding_order(ds):
    """Codewords a few ulps apart in some coordinates: their distances to a
    row differ in the last bits, so any operation rounded otherwise than in
    the reference's order (a product and a sum fused into one fma, sums
    taken in another order) moves many assignments."""
    rng = np.random.default_rng(40 + ds)
    n, K = 60000, 8
    base = rng.standard_normal(ds).astype(np.float32)
    cbs = np.repeat(base[None, None, :], K, axis=1).astype(np.float32)
    for j in range(1, K):
        steps = rng.integers(-4, 5, ds)
        v = cbs[0, j]
        for e in range(ds):
            for _ in range(abs(int(steps[e]))):
                v[e] = np.nextafter(v[e], np.float32(np.inf) if steps[e] > 0 else np.float32(-np.inf))
    res = (base + rng.standard_normal((n, ds)) * rng.choice([0.5, 2.0, 8.0], (n, 1))).astype(np.float32)
    got = gpu_assign(res, cbs)
    want = oracle_assign(res, cbs)
    assert len(np.unique(want)) > 2  # the rows really split among the codewords
    assert np.array_equal(got, want), (ds, int((got != want).sum()))
    got2, _, _ = gpu_assign(res, cbs, with_sums=True)
    assert np.array_equal(got2, want), (ds, int((got2 != want).sum()))


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


@pytest.mark.parametrize("ds", [2, 4, 8, 16])
@pytest.mark.parametrize("K,n", [(256, 100_003), (5, 1025), (1, 3)])
def test_fused_accumulation(ds, K, n):
    """The k-means update's FP64 sums and counts (the fused kernel for
    sub-dimensions 4, 8, 16; separate kernels otherwise): the same
    assignments as the oracle, counts exact, sums equal to an FP64 sum of the
    same values within 1e-12 relative (the order of the additions differs)."""
    rng = np.random.default_rng(ds * 7 + K)
    M = 3
    res = (rng.standard_normal((n, M * ds)) * 3.0).astype(np.float32)
    cbs = rng.standard_normal((M, K, ds)).astype(np.float32)
    asg, sums, counts = gpu_assign(res, cbs, with_sums=True)
    assert np.array_equal(asg, oracle_assign(res, cbs))
    for m in range(M):
        sub = res[:, m * ds:(m + 1) * ds].astype(np.float64)
        want_c = np.bincount(asg[:, m], minlength=K)
        assert np.array_equal(counts[m], want_c)
        want_s = np.zeros((K, ds))
        np.add.at(want_s, asg[:, m], sub)
        scale = np.zeros((K, ds))
        np.add.at(scale, asg[:, m], np.abs(sub))
        assert np.all(np.abs(sums[m] - want_s) <= 1e-12 * np.maximum(scale, 1e-300)), m

