"""Incremental re-Train (hann_pqivf_retrain): Lloyd iterations from the
index's own centroids and codebooks over every stored vector, then the same
reassignment and encoding as Train (pqivf/index.go:451-605), checked
against the oracle's exact assignment, encoding and search."""
import numpy as np
import pytest

import hann_gb300 as hg
import oracle
from tests.helpers import assert_same_results, gaussian_mixture, state_to_oracle

pytestmark = pytest.mark.gpu


def mutated_index():
    rng = np.random.default_rng(71)
    x, centers = gaussian_mixture(rng, 4000, 16, 24, 0.4)
    idx = hg.New(16, hg.WithCoarseK(32), hg.WithNumSubquantizers(4), hg.WithPQK(16), hg.WithKMeansIters(5),
                 hg.WithCandidateClusters(5), hg.WithSeed(3))
    idx.BulkAddArrays(np.arange(4000, dtype=np.int64), x.astype(np.float32))
    idx.Train()
    # the data drifts: new vectors around shifted centers, old ones deleted
    y = (centers[rng.integers(0, 24, 3000)] + 1.5 + 0.4 * rng.standard_normal((3000, 16))).astype(np.float32)
    idx.BulkAddArrays(np.arange(10_000, 13_000, dtype=np.int64), y)
    idx.BulkDelete(list(range(0, 4000, 4)))
    q = np.concatenate([x[:60], y[:60]]).astype(np.float32) + 0.05
    return idx, q


def check_consistent(idx, q):
    st = idx.export_state()
    cl = np.repeat(np.arange(st["layout"]["nlist"]), st["list_len"])
    assert np.array_equal(oracle.assign(st["vectors"], st["coarse"]), cl)
    assert np.array_equal(oracle.encode(st["vectors"], cl, st["coarse"], st["codebooks"]), st["codes"])
    ora = state_to_oracle(st)
    assert_same_results(*idx.SearchBatch(q, 10), *ora.search(q, 10, 5)[:3])
    return st, cl


def test_retrain_one_iteration_is_a_lloyd_step():
    idx, q = mutated_index()
    st0 = idx.export_state()
    ids0 = set(st0["ids"].tolist())
    x = st0["vectors"]
    # one Lloyd step by hand from the current centroids: exact assignment,
    # FP64 means
    asg = oracle.assign(x, st0["coarse"])
    want = st0["coarse"].copy()
    nonempty = np.zeros(len(want), bool)
    for c in range(len(want)):
        rows = x[asg == c]
        if len(rows):
            want[c] = (rows.astype(np.float64).sum(0) / len(rows)).astype(np.float32)
            nonempty[c] = True
    in0 = oracle.inertia_fp64(x, st0["coarse"], asg)
    idx.Retrain(1)
    st1, cl1 = check_consistent(idx, q)
    np.testing.assert_allclose(st1["coarse"][nonempty], want[nonempty], rtol=1e-6, atol=1e-7)
    assert set(st1["ids"].tolist()) == ids0
    order = np.argsort(st1["ids"])
    in1 = oracle.inertia_fp64(st1["vectors"][order], st1["coarse"], cl1[order])
    assert in1 <= in0 * (1 + 1e-6), (in1, in0)


def test_retrain_more_iterations_and_zero():
    idx, q = mutated_index()
    before = idx.export_state()
    idx.Retrain(0)
    st, _ = check_consistent(idx, q)
    # no iteration: the centroids and codebooks stay; the lists are repacked
    np.testing.assert_array_equal(st["coarse"], before["coarse"])
    np.testing.assert_array_equal(st["codebooks"], before["codebooks"])
    assert idx.ArenaStats()["hole_rows"] == 0
    x = st["vectors"]
    in0 = oracle.inertia_fp64(x, st["coarse"], oracle.assign(x, st["coarse"]))
    idx.Retrain(6)
    st6, cl6 = check_consistent(idx, q)
    in6 = oracle.inertia_fp64(st6["vectors"], st6["coarse"], cl6)
    assert in6 < in0
    # mutations keep working after a retrain
    idx.Add(50_000, q[0])
    assert idx.SearchBatch(q[:1], 1, mode=1)[0][0, 0] == 50_000


def test_retrain_errors():
    idx = hg.New(4, hg.WithCoarseK(2), hg.WithNumSubquantizers(2), hg.WithPQK(2))
    idx.BulkAdd({1: [1, 0, 0, 0], 2: [0, 1, 0, 0], 3: [0, 0, 1, 0]})
    with pytest.raises(hg.HannError, match="not trained"):
        idx.Retrain(2)
    idx.Train()
    with pytest.raises(hg.HannError):
        idx.Retrain(-1)
    # fewer vectors than lists, as for Train
    idx.BulkDelete([1, 2])
    with pytest.raises(hg.HannError, match="not enough vectors"):
        idx.Retrain(1)
