"""The binary snapshot (hann_pqivf_save_snapshot / hann_pqivf_load_snapshot):
the same index content as the gob stream of Save/Load (pqivf/index.go:
969-1101), checked sizes and checksum, and a bad file changes nothing."""
import io
import os

import numpy as np
import pytest

import hann_gb300 as hg
from tests.helpers import gaussian_mixture

pytestmark = pytest.mark.gpu

KEYS = ("coarse", "codebooks", "list_len", "list_key", "cluster_counts", "ids", "vectors", "codes", "pending_ids",
        "pending_vectors")


def same_state(a, b):
    sa, sb = a.export_state(), b.export_state()
    assert sa["layout"] == sb["layout"]
    for key in KEYS:
        np.testing.assert_array_equal(np.asarray(sa[key]), np.asarray(sb[key]), err_msg=key)


def trained_index(seed=3):
    rng = np.random.default_rng(seed)
    x, _ = gaussian_mixture(rng, 6000, 24, 40, 0.3)
    idx = hg.New(24, hg.WithCoarseK(64), hg.WithNumSubquantizers(6), hg.WithPQK(32), hg.WithKMeansIters(4),
                 hg.WithCandidateClusters(7), hg.WithSeed(99))
    idx.BulkAddArrays(np.arange(len(x), dtype=np.int64), x.astype(np.float32))
    idx.Train()
    # tombstones and rows appended after training travel too
    idx.BulkDelete(list(range(0, 600, 3)))
    idx.BulkAddArrays(np.arange(10_000, 10_300, dtype=np.int64), x[:300].astype(np.float32) + 0.01)
    return idx, rng


def test_snapshot_round_trip(tmp_path):
    idx, rng = trained_index()
    path = tmp_path / "index.snap"
    idx.SaveSnapshot(path)
    other = hg.New(3)
    other.LoadSnapshot(path)
    same_state(idx, other)
    q = rng.normal(size=(64, 24)).astype(np.float32)
    for mode in (0, 1):
        a = idx.SearchBatch(q, 9, mode=mode)
        b = other.SearchBatch(q, 9, mode=mode)
        for u, v in zip(a, b):
            np.testing.assert_array_equal(u, v)
    # the default nprobe travels (WithCandidateClusters)
    np.testing.assert_array_equal(idx.SearchBatch(q, 5)[0], other.SearchBatch(q, 5)[0])
    # same content as the gob stream: both indexes write the same bytes
    ga, gb = io.BytesIO(), io.BytesIO()
    idx.Save(ga)
    other.Save(gb)
    assert ga.getvalue() == gb.getvalue()
    # and the loaded index keeps working: mutations and a snapshot of it
    other.Add(20_000, q[0])
    assert other.SearchBatch(q[:1], 1, mode=1)[0][0, 0] == 20_000
    other.SaveSnapshot(tmp_path / "again.snap")
    third = hg.New(3)
    third.LoadSnapshot(tmp_path / "again.snap")
    same_state(other, third)


def test_snapshot_untrained_keeps_pending(tmp_path):
    idx = hg.New(4, hg.WithCoarseK(2), hg.WithNumSubquantizers(2), hg.WithPQK(2), hg.WithSeed(5))
    idx.BulkAdd({1: [1, 0, 0, 0], 2: [0, 1, 0, 0], 7: [0, 0, 1, 0]})
    idx.SaveSnapshot(tmp_path / "p.snap")
    other = hg.New(4)
    other.LoadSnapshot(tmp_path / "p.snap")
    same_state(idx, other)
    assert other.Stats().Count == 3
    # the seed travels, so training both gives the same index
    idx.Train()
    other.Train()
    same_state(idx, other)


def test_bad_snapshot_changes_nothing(tmp_path):
    idx, rng = trained_index(4)
    good = tmp_path / "good.snap"
    idx.SaveSnapshot(good)
    data = good.read_bytes()
    target, _ = trained_index(5)
    before = target.export_state()

    def check_unchanged():
        after = target.export_state()
        for key in KEYS:
            np.testing.assert_array_equal(np.asarray(before[key]), np.asarray(after[key]), err_msg=key)

    cases = {
        "flip.snap": data[: len(data) // 2] + bytes([data[len(data) // 2] ^ 0x40]) + data[len(data) // 2 + 1:],
        "short.snap": data[:-20],
        "long.snap": data + b"\0" * 8,
        "magic.snap": b"XANNGBS1" + data[8:],
        "empty.snap": b"",
    }
    for name, blob in cases.items():
        p = tmp_path / name
        p.write_bytes(blob)
        with pytest.raises(hg.HannError):
            target.LoadSnapshot(p)
        check_unchanged()
    with pytest.raises(hg.HannError):
        target.LoadSnapshot(tmp_path / "missing.snap")
    check_unchanged()
    # the good file still loads
    target.LoadSnapshot(good)
    same_state(idx, target)


def test_snapshot_write_failure(tmp_path):
    idx, _ = trained_index(6)
    d = tmp_path / "dir"
    os.mkdir(d)
    with pytest.raises(hg.HannError):
        idx.SaveSnapshot(d)  # a directory cannot be opened for writing


def test_gob_file_round_trip(tmp_path):
    """Save to a file and Load it back (the file is mapped, not read into
    memory): the same index, the same bytes as an in-memory stream."""
    idx, rng = trained_index(7)
    path = tmp_path / "index.gob"
    with open(path, "wb") as f:
        idx.Save(f)
    mem = io.BytesIO()
    idx.Save(mem)
    assert path.read_bytes() == mem.getvalue()
    other = hg.New(3)
    with open(path, "rb") as f:
        other.Load(f)
        assert f.read() == b""  # left at the end, as read() would
    same_state(idx, other)
    q = rng.normal(size=(32, 24)).astype(np.float32)
    for u, v in zip(idx.SearchBatch(q, 9, mode=1), other.SearchBatch(q, 9, mode=1)):
        np.testing.assert_array_equal(u, v)
