"""gob codec: the reference's golden file decodes; encode/decode round trips;
GobDecode's validation (pqivf/index.go:1020-1084). CPU only."""
import io
import os

import numpy as np
import pytest

import hann_gb300 as hg
from hann_gb300 import gob

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "index_v1.gob")


def test_decode_golden():
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    assert ser["Dimension"] == 8
    assert len(ser["CoarseCentroids"]) == 3
    assert set(ser["InvertedLists"]) == {0, 1, 2}
    assert ser["ClusterCounts"] == {0: 10, 1: 11, 2: 8}
    assert np.asarray(ser["Codebooks"]).shape == (2, 4, 4)
    for es in ser["InvertedLists"].values():
        for e in es:
            assert len(e["Vector"]) == 8 and len(e["Codes"]) == 2


def test_round_trip_golden():
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    st = hg.gob_to_state(ser)
    back = gob.decode_pqivf(gob.encode_pqivf(hg.state_to_gob(st)))
    assert back["Dimension"] == ser["Dimension"]
    assert back["ClusterCounts"] == ser["ClusterCounts"]
    assert back["FormatVersion"] == gob.FORMAT_VERSION
    for c, es in ser["InvertedLists"].items():
        got = back["InvertedLists"][c]
        assert [e.get("ID", 0) for e in got] == [e.get("ID", 0) for e in es]
        for a, b in zip(got, es):
            assert np.array_equal(np.float32(a["Vector"]), np.float32(b["Vector"]))
            assert list(a["Codes"]) == list(b["Codes"])
    assert np.array_equal(np.float32(back["Codebooks"]), np.float32(ser["Codebooks"]))
    assert np.array_equal(np.float32(back["CoarseCentroids"]), np.float32(ser["CoarseCentroids"]))


def test_primitives_round_trip():
    buf = bytearray()
    vals = [0, 1, -1, 127, 128, -129, 2**40, -(2**40)]
    for v in vals:
        gob._put_int(buf, v)
    r = gob._Reader(bytes(buf))
    assert [r.int() for _ in vals] == vals
    buf = bytearray()
    fl = [0.0, 1.5, -2.25, 1e-30, 3.4028234663852886e38]
    for v in fl:
        gob._put_float(buf, v)
    r = gob._Reader(bytes(buf))
    assert [r.float() for _ in fl] == fl


def _ser(**over):
    ser = gob.decode_pqivf(open(GOLDEN, "rb").read())
    ser.update(over)
    return ser


@pytest.mark.parametrize("over,msg", [
    ({"FormatVersion": 2}, "format version 2"),
    ({"Dimension": 0}, "invalid dimension 0"),
    ({"NumSubquantizers": 3}, "invalid subquantizer count 3"),
    ({"NumSubquantizers": 0}, "invalid subquantizer count 0"),
    ({"CoarseK": 0}, "invalid training parameters"),
    ({"PqK": -1}, "invalid training parameters"),
    ({"KMeansIters": 0}, "invalid training parameters"),
])
def test_decode_validation(over, msg):
    with pytest.raises(hg.HannError, match=msg):
        hg.gob_to_state(_ser(**over))


def test_legacy_candidate_clusters_default():
    # files without NumCandidateClusters keep the configured value, else 3
    st = hg.gob_to_state(_ser())
    assert st["layout"]["candidate_clusters"] == 3
    st = hg.gob_to_state(_ser(NumCandidateClusters=7))
    assert st["layout"]["candidate_clusters"] == 7


def test_truncated_stream_rejected():
    data = open(GOLDEN, "rb").read()
    with pytest.raises(gob.GobError):
        gob.decode_pqivf(data[: len(data) // 2])
