"""Warm k-means assignments (assign_rows in index.cu): after the first
iteration every row's nearest centroid is bounded from its previous
centroid's distance and how far that centroid moved, the filter GEMM keeps
the centroids under the bound and an exact rescore picks among them. The
assignment must stay the reference's exact argmin (lowest index on a tie), so
training with the tensor cores gives, bit for bit, the index the plain FP32
path trains (assignPoints, pqivf/index.go:738-789), also with empty clusters
reseeded (centroids that jump) and with anisotropic data."""
import numpy as np
import pytest

import hann_gb300 as hg

pytestmark = pytest.mark.gpu


def _anisotropic(rng, n, dim, k):
    c = rng.standard_normal((k, dim)).astype(np.float32) * 3.0
    scales = np.exp(rng.uniform(np.log(0.05), 0.0, (k, dim))).astype(np.float32)
    lab = rng.integers(0, k, n)
    return (c[lab] + rng.standard_normal((n, dim)).astype(np.float32) * scales[lab]).astype(np.float32)


@pytest.mark.parametrize("n,dim,k,iters", [(40000, 64, 512, 8), (20000, 128, 1024, 5), (6000, 32, 2048, 4)])
def test_warm_assignment_trains_the_plain_index(gpu, n, dim, k, iters):
    rng = np.random.default_rng(n + dim + k)
    x = _anisotropic(rng, n, dim, max(8, k // 4))
    idx = []
    for plain in (False, True):
        h = hg.New(dim, hg.WithCoarseK(k), hg.WithNumSubquantizers(8), hg.WithPQK(16), hg.WithKMeansIters(iters),
                   hg.WithPlainFP32(plain))
        h.BulkAddArrays(np.arange(n, dtype=np.int64), x)
        h.Train()
        idx.append(h)
    try:
        sa, sb = idx[0].export_state(), idx[1].export_state()
        for key in ("coarse", "list_len", "ids", "codes", "codebooks"):
            np.testing.assert_array_equal(sa[key], sb[key], err_msg=key)
        st = idx[0].TrainStats()
        # iterations 2..iters and the final assignment (a warm assignment
        # that overflows on many rows hands the next one to the top-8 screen)
        assert st["warm_assignments"] >= iters // 2, st
        assert idx[1].TrainStats()["warm_assignments"] == 0
    finally:
        for h in idx:
            h.close()
