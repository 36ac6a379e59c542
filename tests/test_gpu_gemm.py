"""The BF16 tcgen05 distance GEMM against a host computation on the same
BF16-rounded operands (diagnostic entry point hann_gpu_bf16_scores)."""
import ctypes

import numpy as np
import pytest

import hann_gb300 as hg

pytestmark = pytest.mark.gpu
_P = ctypes.c_void_p


def bf16(x):
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def run(a, b):
    L = hg.load_library()
    f = L.hann_gpu_bf16_scores
    f.argtypes = [_P, ctypes.c_int64, _P, ctypes.c_int32, ctypes.c_int32, _P, _P, _P]
    n, dim = a.shape
    m = b.shape[0]
    s = np.zeros((n, m), np.float32)
    ti = np.zeros((n, 8), np.int32)
    tv = np.zeros((n, 8), np.float32)
    rc = f(_P(a.ctypes.data), n, _P(b.ctypes.data), m, dim, _P(s.ctypes.data), _P(ti.ctypes.data),
           _P(tv.ctypes.data))
    assert rc == 0
    return s, ti, tv


@pytest.mark.parametrize("n,m,dim", [(1, 1, 8), (5, 300, 16), (130, 513, 96), (257, 1000, 128),
                                     (128, 256, 96), (300, 773, 72), (64, 4096, 96)])
def test_scores_match_host(gpu, n, m, dim):
    rng = np.random.default_rng(n * 1000 + m + dim)
    a = rng.normal(size=(n, dim)).astype(np.float32)
    b = rng.normal(size=(m, dim)).astype(np.float32)
    s, ti, tv = run(a, b)
    ab, bb = bf16(a).astype(np.float64), bf16(b).astype(np.float64)
    bias = (b.astype(np.float64) ** 2).sum(1)
    ref = bias[None, :] - 2.0 * ab @ bb.T
    scale = bias[None, :] + 2.0 * np.abs(ab) @ np.abs(bb).T
    err = np.abs(s - ref)
    assert (err <= 1e-5 * scale + 1e-6).all(), float((err / scale).max())
    kk = min(8, m)
    order = np.argsort(s, axis=1, kind="stable")[:, :kk]
    np.testing.assert_array_equal(np.sort(tv[:, :kk], axis=1), np.sort(np.take_along_axis(s, order, 1), axis=1))
    assert (np.take_along_axis(s, ti[:, :kk].astype(np.int64), 1) == tv[:, :kk]).all()
