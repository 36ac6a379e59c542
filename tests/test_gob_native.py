"""Native gob codec (csrc/gob.cu) against the pure-Python codec (gob.py):
byte-identical encoding, identical decoding of the reference's golden file,
GobDecode's validation (pqivf/index.go:1020-1084), and malformed streams
rejected without a crash. Host code only: runs without a GPU."""
import os

import numpy as np
import pytest

import hann_gb300 as hg
from hann_gb300 import gob
from tests.helpers import flat_struct_stream

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "index_v1.gob")
KEYS = ("coarse", "codebooks", "list_len", "list_key", "cluster_counts", "ids", "vectors", "codes", "has_codes",
        "pending_ids", "pending_vectors")


@pytest.fixture(scope="module", autouse=True)
def _lib(built):
    hg.load_library()


def random_state(rng, dim=12, M=3, nl=7, kq=5, rows=60, pending=9, trained=True, fallback=False, ncc=4):
    llen = rng.multinomial(rows, np.ones(nl) / nl).astype(np.int64) if nl else np.zeros(0, np.int64)
    if nl > 2:
        llen[1] = 0  # a keyed list with no entries
    rows = int(llen.sum())
    lkey = (llen > 0).astype(np.uint8)
    if nl > 2:
        lkey[1] = 1
    ids = rng.permutation(np.arange(-5, rows + 40))[:rows].astype(np.int64)
    vals = rng.normal(size=(rows, dim)).astype(np.float32)
    if rows > 4:
        vals[0] = 0.0  # zero encodes as one byte
        vals[1] = -0.0
        vals[2, :2] = 1.5
        vals[4, :] = np.float32(3.4028235e38)
        vals[4, 0] = np.float32(1e-45)  # a denormal
    return {
        "layout": {"dimension": dim, "coarse_k": nl + 2, "num_subquantizers": M, "pq_k": kq + 1,
                   "kmeans_iters": 6, "candidate_clusters": ncc, "fallback": int(fallback), "trained": int(trained),
                   "nlist": nl, "pq_k_eff": kq, "n_rows": rows, "n_pending": pending},
        "coarse": rng.normal(size=(nl, dim)).astype(np.float32),
        "codebooks": rng.normal(size=(M, kq, dim // M)).astype(np.float32),
        "list_len": llen, "list_key": lkey,
        "cluster_counts": np.where(lkey > 0, llen + rng.integers(0, 3, nl), 0).astype(np.int64),
        "ids": ids, "vectors": vals,
        "codes": rng.integers(0, max(kq, 1), size=(rows, M)).astype(np.int32),
        "pending_ids": rng.permutation(np.arange(1000, 1000 + 3 * pending))[:pending].astype(np.int64),
        "pending_vectors": rng.normal(size=(pending, dim)).astype(np.float32),
    }


CASES = {
    "trained": {},
    "fallback_no_pending": {"pending": 0, "fallback": True},
    "untrained_pending_only": {"nl": 0, "kq": 0, "rows": 0, "trained": False, "pending": 30},
    "one_subquantizer": {"dim": 8, "M": 1, "kq": 3},
    "wide": {"dim": 96, "M": 24, "nl": 16, "kq": 256, "rows": 500, "ncc": 0},
    "no_codewords": {"kq": 0, "rows": 0, "pending": 3},
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_encode_matches_python_codec(case):
    st = random_state(np.random.default_rng(len(case)), **CASES[case])
    native = hg.gob_encode_state(st).tobytes()
    assert native == gob.encode_pqivf(hg.state_to_gob(st))


@pytest.mark.parametrize("case", sorted(CASES))
def test_round_trip(case):
    st = random_state(np.random.default_rng(3 + len(case)), **CASES[case])
    back = hg.gob_decode_state(hg.gob_encode_state(st).tobytes(), 11)
    lay = dict(st["layout"])
    if lay["candidate_clusters"] == 0:
        lay["candidate_clusters"] = 11  # the configured value is kept
    assert back["layout"] == lay
    order = np.argsort(st["pending_ids"], kind="stable")
    want = dict(st, pending_ids=st["pending_ids"][order], pending_vectors=st["pending_vectors"][order],
                has_codes=np.ones(len(st["ids"]), np.uint8))
    for k in KEYS:
        np.testing.assert_array_equal(back[k], np.asarray(want[k]).reshape(back[k].shape), err_msg=k)


def test_decode_golden_matches_python_codec():
    data = open(GOLDEN, "rb").read()
    a = hg.gob_decode_state(data)
    b = hg.gob_to_state(gob.decode_pqivf(data))
    assert a["layout"] == b["layout"]
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["layout"]["n_rows"] == 29 and a["layout"]["dimension"] == 8
    # and it re-encodes to what the Python codec writes for the same state
    assert hg.gob_encode_state(a).tobytes() == gob.encode_pqivf(hg.state_to_gob(b))


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
    ser = _ser(**over)
    data = gob.encode_pqivf(ser)
    if "FormatVersion" in over:  # the encoder always writes its own version: patch the value
        data = _with_format_version(ser, over["FormatVersion"])
    with pytest.raises(hg.HannError, match=msg):
        hg.gob_decode_state(data)


def _with_format_version(ser, v):
    old = gob.FORMAT_VERSION
    gob.FORMAT_VERSION = v
    try:
        return gob.encode_pqivf(ser)
    finally:
        gob.FORMAT_VERSION = old


def test_candidate_clusters_default():
    ser = _ser()
    ser.pop("NumCandidateClusters", None)
    data = gob.encode_pqivf(ser)
    assert hg.gob_decode_state(data)["layout"]["candidate_clusters"] == 3
    assert hg.gob_decode_state(data, 9)["layout"]["candidate_clusters"] == 9
    assert hg.gob_decode_state(gob.encode_pqivf(_ser(NumCandidateClusters=7)), 9)["layout"][
        "candidate_clusters"] == 7


def test_bad_codes_marked_for_reencoding():
    ser = _ser()
    lists = ser["InvertedLists"]
    c0 = sorted(lists)[0]
    lists[c0][0]["Codes"] = [9, 0]       # codeword 9 of 4
    lists[c0][1]["Codes"] = [1]          # one code for two subquantizers
    lists[c0][2]["Codes"] = None         # no codes at all
    st = hg.gob_decode_state(gob.encode_pqivf(ser))
    ref = hg.gob_to_state(gob.decode_pqivf(gob.encode_pqivf(ser)))
    assert list(st["has_codes"][:3]) == [0, 0, 0]
    assert st["has_codes"][3:].all()
    for k in KEYS:
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)


def test_wrong_vector_dimension_rejected():
    ser = _ser()
    c0 = sorted(ser["InvertedLists"])[0]
    ser["InvertedLists"][c0][0]["Vector"] = [1.0] * 5
    with pytest.raises(hg.HannError, match="has a vector of dimension 5"):
        hg.gob_decode_state(gob.encode_pqivf(ser))


def test_list_without_centroid_rejected():
    ser = _ser()
    c0 = sorted(ser["InvertedLists"])[0]
    ser["InvertedLists"][17] = ser["InvertedLists"][c0][:2]
    with pytest.raises(hg.HannError, match="inverted list 17 has no coarse centroid"):
        hg.gob_decode_state(gob.encode_pqivf(ser))


def test_malformed_streams_rejected_without_crash():
    data = open(GOLDEN, "rb").read()
    st = random_state(np.random.default_rng(8))
    other = hg.gob_encode_state(st).tobytes()
    rng = np.random.default_rng(0)
    for blob in (data, other):
        for cut in list(range(0, 64)) + list(rng.integers(0, len(blob), 80)):
            with pytest.raises(hg.HannError):
                hg.gob_decode_state(blob[:cut])
        ok = 0
        for _ in range(300):
            b = bytearray(blob)
            for i in rng.integers(0, len(b), rng.integers(1, 4)):
                b[i] = int(rng.integers(0, 256))
            try:
                got = hg.gob_decode_state(bytes(b))
            except hg.HannError:
                continue
            ok += 1
            try:  # where both codecs accept a mutated stream they agree
                with np.errstate(over="ignore"):  # a mutated float can overflow float32, in both
                    ref = hg.gob_to_state(gob.decode_pqivf(bytes(b)))
            except Exception:
                continue
            for k in KEYS:
                np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
        assert ok < 300
    with pytest.raises(hg.HannError):
        hg.gob_decode_state(b"")


def test_size_query_and_short_buffer():
    import ctypes

    st = random_state(np.random.default_rng(2))
    full = hg.gob_encode_state(st)
    L = hg.load_library()
    lay = hg._Layout(**st["layout"])
    arrs = [np.ascontiguousarray(st[k]) for k in ("coarse", "codebooks", "list_len", "list_key", "cluster_counts",
                                                   "ids", "vectors", "codes", "pending_ids", "pending_vectors")]
    n = ctypes.c_int64(0)
    out = np.zeros(full.size - 1, np.uint8)
    rc = L.hann_gob_encode(ctypes.byref(lay), *[hg._ptr(a) for a in arrs], hg._ptr(out), out.size, ctypes.byref(n))
    assert rc == hg.HANN_E_INVALID and n.value == full.size
    assert b"needed" in L.hann_gob_last_error()
    assert not out.any()  # nothing written


def test_mapped_file_reads_from_position(tmp_path):
    """Load maps a file on disk and decodes from the reader's position to
    the end, as read() would; a bad stream in a mapped file still raises."""
    st = random_state(np.random.default_rng(5))
    blob = hg.gob_encode_state(st).tobytes()
    p = tmp_path / "index.gob"
    p.write_bytes(b"HEADER" + blob)
    with open(p, "rb") as f:
        f.read(6)
        mm, off = hg._map_rest(f)
        try:
            got = hg.gob_decode_state(memoryview(mm)[off:])
        finally:
            mm.close()
    want = hg.gob_decode_state(blob)
    for k in KEYS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    # nothing after the position, a pipe-like reader, an in-memory stream
    with open(p, "rb") as f:
        f.seek(0, 2)
        assert hg._map_rest(f) is None
    import io
    assert hg._map_rest(io.BytesIO(blob)) is None
    bad = tmp_path / "bad.gob"
    bad.write_bytes(blob[: len(blob) // 3])
    with open(bad, "rb") as f:
        mm, off = hg._map_rest(f)
        with pytest.raises(hg.HannError):
            hg.gob_decode_state(memoryview(mm)[off:])
        try:
            mm.close()
        except BufferError:
            pass


def test_gob_decode_errors():
    """TestPQIVF_GobDecodeErrors (pqivf/index_test.go:741-764)."""
    with pytest.raises(hg.HannError):
        hg.gob_decode_state(b"not a gob stream")
    with pytest.raises(hg.HannError, match="format version"):
        hg.gob_decode_state(flat_struct_stream([("FormatVersion", 999)]))


def test_gob_decode_legacy_fields():
    """TestPQIVF_GobDecodeLegacyPendingVectors (pqivf/index_test.go:771-795):
    a struct with only the five parameters decodes to an empty, untrained
    index."""
    st = hg.gob_decode_state(flat_struct_stream([("Dimension", 4), ("CoarseK", 2), ("NumSubquantizers", 2),
                                                 ("PqK", 4), ("KMeansIters", 5)]))
    lay = st["layout"]
    assert (lay["dimension"], lay["coarse_k"], lay["num_subquantizers"], lay["pq_k"], lay["kmeans_iters"]) == \
        (4, 2, 2, 4, 5)
    assert (lay["nlist"], lay["n_rows"], lay["n_pending"], lay["trained"], lay["candidate_clusters"]) == \
        (0, 0, 0, 0, 3)


@pytest.mark.parametrize("fields", [
    [("Dimension", 0)],
    [("Dimension", 6), ("NumSubquantizers", 0)],
    [("Dimension", 6), ("NumSubquantizers", 4)],
    [("Dimension", 6), ("NumSubquantizers", 2), ("CoarseK", 0)],
])
def test_gob_decode_rejects_invalid_parameters(fields):
    """TestPQIVF_GobDecodeRejectsInvalidParameters (pqivf/index_test.go:
    944-980)."""
    with pytest.raises(hg.HannError):
        hg.gob_decode_state(flat_struct_stream(fields))


def test_payload_is_the_wrapped_streams_content():
    """GobEncode's bytes (pqivf/index.go:992-1017) are the serializedPQIVF
    stream that Save's GobEncoder value carries."""
    st = random_state(np.random.default_rng(12))
    wrapped = hg.gob_encode_state(st).tobytes()
    payload = hg.gob_encode_state(st, wrapped=False).tobytes()
    assert wrapped.endswith(payload)
    ((name, inner),) = gob.decode_stream(wrapped)
    assert name == "*pqivf.Index" and inner == payload
    ((name, ser),) = gob.decode_stream(payload)
    assert name == "serializedPQIVF" and ser["Dimension"] == 12
    a, b = hg.gob_decode_state(payload), hg.gob_decode_state(wrapped)
    assert a["layout"] == b["layout"]
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_out_of_range_type_ids_rejected():
    """A type definition with an id far beyond any stream's own numbering,
    or a value of an undefined type, is malformed."""
    for tid in (-(1 << 17), -(1 << 30), 1 << 17, 3, 70):
        msg = bytearray()
        gob._put_int(msg, tid)
        msg += b"\x01\x02\x03"
        data = bytearray()
        gob._put_uint(data, len(msg))
        data += msg
        with pytest.raises(hg.HannError):
            hg.gob_decode_state(bytes(data))


def test_huge_dimension_rejected_without_large_allocation():
    """A small stream claiming a huge dimension is refused; nothing is sized
    from the claimed dimension before the stream shows the floats."""
    import resource
    import time

    before = resource.getrusage(resource.RUSAGE_SELF).ru_maxrss
    for dim in (10**9, 2**40):
        for ser in (_ser(Dimension=dim),
                    {"Dimension": dim, "CoarseK": 2, "NumSubquantizers": 1, "PqK": 2, "KMeansIters": 1,
                     "PendingVectors": {i: [1.0, 2.0] for i in range(2000)}}):
            t = time.time()
            with pytest.raises(hg.HannError):
                hg.gob_decode_state(gob.encode_pqivf(ser))
            assert time.time() - t < 5
    assert resource.getrusage(resource.RUSAGE_SELF).ru_maxrss - before < 512 * 1024  # KiB: under 512 MiB
