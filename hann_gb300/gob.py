"""Go ``encoding/gob`` codec for the PQIVF index's persisted form.

The reference saves an index as a gob stream whose one value is the
``*pqivf.Index`` GobEncoder; its bytes are themselves a gob stream holding a
``serializedPQIVF`` struct (pqivf/index.go:969-984, 992-1017, 1086-1101).
This module reads and writes that layout so an index can move between the
reference and this package in both directions.

The wire format follows the published encoding/gob specification:
messages are ``(uint length)(int type id)(payload)``; a negative type id
introduces a ``wireType`` definition; unsigned integers are one byte below
128, else a negated byte count followed by big-endian bytes; signed integers
fold the sign into bit 0; floats are IEEE-754 float64 bits byte-reversed and
sent as an unsigned integer; structs are (field delta, value) pairs ended by a
zero delta and omit zero-valued fields; a top-level non-struct value is
preceded by a zero byte.
"""
from __future__ import annotations

import io
import struct

import numpy as np

# Predefined gob type ids.
T_BOOL, T_INT, T_UINT, T_FLOAT, T_BYTES, T_STRING, T_COMPLEX, T_INTERFACE = 1, 2, 3, 4, 5, 6, 7, 8
T_WIRETYPE, T_ARRAYTYPE, T_COMMONTYPE, T_SLICETYPE, T_STRUCTTYPE, T_FIELDTYPE = 16, 17, 18, 19, 20, 21
T_FIELDTYPE_SLICE, T_MAPTYPE = 22, 23
FIRST_USER_ID = 65


class GobError(ValueError):
    pass


# ---------------------------------------------------------------------------
# primitive readers


class _Reader:
    def __init__(self, data: bytes):
        self.b = memoryview(bytes(data))
        self.i = 0

    def eof(self) -> bool:
        return self.i >= len(self.b)

    def byte(self) -> int:
        if self.i >= len(self.b):
            raise GobError("unexpected end of gob data")
        v = self.b[self.i]
        self.i += 1
        return v

    def take(self, n: int) -> bytes:
        if n < 0 or self.i + n > len(self.b):
            raise GobError("unexpected end of gob data")
        v = bytes(self.b[self.i:self.i + n])
        self.i += n
        return v

    def uint(self) -> int:
        c = self.byte()
        if c < 0x80:
            return c
        n = 256 - c
        if n > 8:
            raise GobError("invalid uint length")
        return int.from_bytes(self.take(n), "big")

    def int(self) -> int:
        u = self.uint()
        return ~(u >> 1) if u & 1 else (u >> 1)

    def float(self) -> float:
        u = self.uint()
        rev = int.from_bytes(u.to_bytes(8, "big")[::-1], "big")
        return struct.unpack(">d", rev.to_bytes(8, "big"))[0]


# ---------------------------------------------------------------------------
# decoding


class _WireType:
    __slots__ = ("kind", "name", "elem", "key", "length", "fields")

    def __init__(self, kind, name="", elem=None, key=None, length=0, fields=None):
        self.kind, self.name, self.elem, self.key = kind, name, elem, key
        self.length, self.fields = length, fields or []


def _decode_common(r: _Reader):
    name, tid = "", 0
    field = -1
    while True:
        d = r.uint()
        if d == 0:
            return name, tid
        field += d
        if field == 0:
            name = r.take(r.uint()).decode()
        elif field == 1:
            tid = r.int()
        else:
            raise GobError("bad CommonType field")


def _decode_wiretype(r: _Reader) -> _WireType:
    field = -1
    wt = None
    while True:
        d = r.uint()
        if d == 0:
            break
        field += d
        if field == 0:  # ArrayT
            name, elem, length = "", 0, 0
            f = -1
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                f += dd
                if f == 0:
                    name, _ = _decode_common(r)
                elif f == 1:
                    elem = r.int()
                elif f == 2:
                    length = r.int()
            wt = _WireType("array", name, elem=elem, length=length)
        elif field == 1:  # SliceT
            name, elem = "", 0
            f = -1
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                f += dd
                if f == 0:
                    name, _ = _decode_common(r)
                elif f == 1:
                    elem = r.int()
            wt = _WireType("slice", name, elem=elem)
        elif field == 2:  # StructT
            name, fields = "", []
            f = -1
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                f += dd
                if f == 0:
                    name, _ = _decode_common(r)
                elif f == 1:
                    for _ in range(r.uint()):
                        fname, fid = "", 0
                        g = -1
                        while True:
                            ddd = r.uint()
                            if ddd == 0:
                                break
                            g += ddd
                            if g == 0:
                                fname = r.take(r.uint()).decode()
                            elif g == 1:
                                fid = r.int()
                        fields.append((fname, fid))
            wt = _WireType("struct", name, fields=fields)
        elif field == 3:  # MapT
            name, key, elem = "", 0, 0
            f = -1
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                f += dd
                if f == 0:
                    name, _ = _decode_common(r)
                elif f == 1:
                    key = r.int()
                elif f == 2:
                    elem = r.int()
            wt = _WireType("map", name, key=key, elem=elem)
        elif field in (4, 5, 6):  # GobEncoderT, BinaryMarshalerT, TextMarshalerT
            name = ""
            f = -1
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                f += dd
                if f == 0:
                    name, _ = _decode_common(r)
            wt = _WireType("gobencoder", name)
        else:
            raise GobError("unknown wireType field %d" % field)
    if wt is None:
        raise GobError("empty wireType")
    return wt


class _Decoder:
    def __init__(self):
        self.types: dict[int, _WireType] = {}

    def value(self, r: _Reader, tid: int):
        if tid == T_BOOL:
            return r.uint() != 0
        if tid == T_INT:
            return r.int()
        if tid == T_UINT:
            return r.uint()
        if tid == T_FLOAT:
            return r.float()
        if tid == T_BYTES:
            return r.take(r.uint())
        if tid == T_STRING:
            return r.take(r.uint()).decode()
        if tid == T_COMPLEX:
            return complex(r.float(), r.float())
        wt = self.types.get(tid)
        if wt is None:
            raise GobError("unknown type id %d" % tid)
        if wt.kind == "struct":
            return self.struct(r, wt)
        if wt.kind in ("slice", "array"):
            n = r.uint()
            if wt.elem == T_FLOAT:
                return [r.float() for _ in range(n)]
            return [self.value(r, wt.elem) for _ in range(n)]
        if wt.kind == "map":
            n = r.uint()
            out = {}
            for _ in range(n):
                k = self.value(r, wt.key)
                out[k] = self.value(r, wt.elem)
            return out
        if wt.kind == "gobencoder":
            return r.take(r.uint())
        raise GobError("unsupported kind %s" % wt.kind)

    def struct(self, r: _Reader, wt: _WireType):
        out = {}
        field = -1
        while True:
            d = r.uint()
            if d == 0:
                return out
            field += d
            if field >= len(wt.fields):
                raise GobError("field index out of range in %s" % wt.name)
            fname, fid = wt.fields[field]
            out[fname] = self.value(r, fid)


def decode_stream(data: bytes):
    """Decode every top-level value of a gob stream. Returns a list of
    (type name, value) pairs; a GobEncoder value is returned as its bytes."""
    r = _Reader(data)
    dec = _Decoder()
    out = []
    while not r.eof():
        n = r.uint()
        msg = _Reader(r.take(n))
        tid = msg.int()
        if tid < 0:
            dec.types[-tid] = _decode_wiretype(msg)
            continue
        wt = dec.types.get(tid)
        if wt is not None and wt.kind == "struct":
            out.append((wt.name, dec.struct(msg, wt)))
        else:
            if msg.uint() != 0:
                raise GobError("singleton value without its zero prefix")
            out.append((wt.name if wt else "", dec.value(msg, tid)))
    return out


# ---------------------------------------------------------------------------
# encoding


def _put_uint(buf: bytearray, v: int) -> None:
    if v < 0:
        raise GobError("negative uint")
    if v < 0x80:
        buf.append(v)
        return
    b = v.to_bytes((v.bit_length() + 7) // 8, "big")
    buf.append(256 - len(b))
    buf += b


def _put_int(buf: bytearray, v: int) -> None:
    _put_uint(buf, (~v << 1) | 1 if v < 0 else v << 1)


def _put_float(buf: bytearray, v: float) -> None:
    bits = struct.unpack(">Q", struct.pack(">d", float(v)))[0]
    _put_uint(buf, int.from_bytes(bits.to_bytes(8, "big")[::-1], "big"))


def _put_str(buf: bytearray, s) -> None:
    b = s.encode() if isinstance(s, str) else bytes(s)
    _put_uint(buf, len(b))
    buf += b


def _float_list(buf: bytearray, vals) -> None:
    arr = np.asarray(vals, dtype=np.float32).astype(np.float64).ravel()
    _put_uint(buf, arr.size)
    for v in arr.tolist():
        _put_float(buf, v)


class _Encoder:
    """Writes the type definitions and values of one gob stream."""

    def __init__(self):
        self.out = bytearray()
        self.next_id = FIRST_USER_ID

    def _msg(self, tid: int, payload: bytes) -> None:
        m = bytearray()
        _put_int(m, tid)
        m += payload
        _put_uint(self.out, len(m))
        self.out += m

    def _common(self, buf: bytearray, name: str, tid: int) -> None:
        if name:
            _put_uint(buf, 1)
            _put_str(buf, name)
            _put_uint(buf, 1)
        else:
            _put_uint(buf, 2)
        _put_int(buf, tid)
        _put_uint(buf, 0)

    def define_slice(self, name: str, elem: int) -> int:
        tid = self.next_id
        self.next_id += 1
        w = bytearray()
        _put_uint(w, 2)  # field 1: SliceT
        _put_uint(w, 1)  # sliceType field 0: CommonType
        self._common(w, name, tid)
        _put_uint(w, 1)  # field 1: Elem
        _put_int(w, elem)
        _put_uint(w, 0)
        _put_uint(w, 0)
        self._msg(-tid, bytes(w))
        return tid

    def define_map(self, name: str, key: int, elem: int) -> int:
        tid = self.next_id
        self.next_id += 1
        w = bytearray()
        _put_uint(w, 4)  # field 3: MapT
        _put_uint(w, 1)
        self._common(w, name, tid)
        _put_uint(w, 1)
        _put_int(w, key)
        _put_uint(w, 1)
        _put_int(w, elem)
        _put_uint(w, 0)
        _put_uint(w, 0)
        self._msg(-tid, bytes(w))
        return tid

    def define_struct(self, name: str, fields, tid: int | None = None) -> int:
        if tid is None:
            tid = self.next_id
            self.next_id += 1
        w = bytearray()
        _put_uint(w, 3)  # field 2: StructT
        _put_uint(w, 1)
        self._common(w, name, tid)
        _put_uint(w, 1)  # Field []fieldType
        _put_uint(w, len(fields))
        for fname, fid in fields:
            _put_uint(w, 1)
            _put_str(w, fname)
            _put_uint(w, 1)
            _put_int(w, fid)
            _put_uint(w, 0)
        _put_uint(w, 0)
        _put_uint(w, 0)
        self._msg(-tid, bytes(w))
        return tid

    def define_gobencoder(self, name: str) -> int:
        tid = self.next_id
        self.next_id += 1
        w = bytearray()
        _put_uint(w, 5)  # field 4: GobEncoderT
        _put_uint(w, 1)  # gobEncoderType field 0: CommonType
        self._common(w, name, tid)
        _put_uint(w, 0)
        _put_uint(w, 0)
        self._msg(-tid, bytes(w))
        return tid

    def value(self, tid: int, payload: bytes) -> None:
        self._msg(tid, payload)


# ---------------------------------------------------------------------------
# the PQIVF persisted form

FORMAT_VERSION = 1


def encode_pqivf(state: dict) -> bytes:
    """Encode an index state as the reference's Save writes it.

    ``state`` keys: Dimension, CoarseK, CoarseCentroids [k][d],
    ClusterCounts {cluster: n}, InvertedLists {cluster: [entry]},
    NumSubquantizers, Codebooks [M][pqK][dsub], PqK, KMeansIters,
    AllowBruteForceFallback, Trained, PendingVectors {id: vec},
    NumCandidateClusters. An entry is a dict with ID, Vector, Codes (list
    of int or None) and Cluster."""
    inner = _Encoder()
    # Types are defined in the order the value's fields first need them.
    t_f32s = inner.define_slice("", T_FLOAT)
    t_f32ss = inner.define_slice("", t_f32s)
    t_mapii = inner.define_map("", T_INT, T_INT)
    t_ints = inner.define_slice("", T_INT)
    t_entry_id = inner.next_id + 2  # entry struct id after the map and slice ids
    t_entries = inner.next_id + 1
    t_maplist = inner.next_id
    inner.next_id += 3
    # map[int][]pqEntry, []pqEntry, pqEntry
    w = _Encoder()
    w.next_id = 0
    inner_defs = inner
    # map type
    buf = bytearray()
    _put_uint(buf, 4)
    _put_uint(buf, 1)
    inner_defs._common(buf, "", t_maplist)
    _put_uint(buf, 1)
    _put_int(buf, T_INT)
    _put_uint(buf, 1)
    _put_int(buf, t_entries)
    _put_uint(buf, 0)
    _put_uint(buf, 0)
    inner_defs._msg(-t_maplist, bytes(buf))
    buf = bytearray()
    _put_uint(buf, 2)
    _put_uint(buf, 1)
    inner_defs._common(buf, "", t_entries)
    _put_uint(buf, 1)
    _put_int(buf, t_entry_id)
    _put_uint(buf, 0)
    _put_uint(buf, 0)
    inner_defs._msg(-t_entries, bytes(buf))
    inner_defs.define_struct("pqEntry", [("ID", T_INT), ("Vector", t_f32s), ("Codes", t_ints),
                                         ("Cluster", T_INT)], tid=t_entry_id)
    t_f32sss = inner.define_slice("", t_f32ss)
    t_mapivec = inner.define_map("", T_INT, t_f32s)
    fields = [("Dimension", T_INT), ("CoarseK", T_INT), ("CoarseCentroids", t_f32ss),
              ("ClusterCounts", t_mapii), ("InvertedLists", t_maplist), ("NumSubquantizers", T_INT),
              ("Codebooks", t_f32sss), ("PqK", T_INT), ("KMeansIters", T_INT),
              ("AllowBruteForceFallback", T_BOOL), ("Trained", T_BOOL), ("PendingVectors", t_mapivec),
              ("FormatVersion", T_INT), ("NumCandidateClusters", T_INT)]
    t_ser = inner.define_struct("serializedPQIVF", fields)

    v = bytearray()
    last = -1

    def field(i):
        nonlocal last
        _put_uint(v, i - last)
        last = i

    def put_vec2(rows):
        _put_uint(v, len(rows))
        for row in rows:
            _float_list(v, row)

    if state.get("Dimension", 0):
        field(0)
        _put_int(v, int(state["Dimension"]))
    if state.get("CoarseK", 0):
        field(1)
        _put_int(v, int(state["CoarseK"]))
    cc = state.get("CoarseCentroids")
    if cc is not None and len(cc):
        field(2)
        put_vec2(cc)
    counts = state.get("ClusterCounts") or {}
    if counts:
        field(3)
        _put_uint(v, len(counts))
        for c in sorted(counts):
            _put_int(v, int(c))
            _put_int(v, int(counts[c]))
    lists = state.get("InvertedLists") or {}
    if lists:
        field(4)
        _put_uint(v, len(lists))
        for c in sorted(lists):
            _put_int(v, int(c))
            entries = lists[c]
            _put_uint(v, len(entries))
            for e in entries:
                sub_last = -1
                def sf(i):
                    nonlocal sub_last
                    _put_uint(v, i - sub_last)
                    sub_last = i
                if int(e["ID"]) != 0:
                    sf(0)
                    _put_int(v, int(e["ID"]))
                vec = e.get("Vector")
                if vec is not None and len(vec):
                    sf(1)
                    _float_list(v, vec)
                codes = e.get("Codes")
                if codes is not None and len(codes):
                    sf(2)
                    _put_uint(v, len(codes))
                    for cval in codes:
                        _put_int(v, int(cval))
                if int(e.get("Cluster", 0)) != 0:
                    sf(3)
                    _put_int(v, int(e["Cluster"]))
                _put_uint(v, 0)
    if state.get("NumSubquantizers", 0):
        field(5)
        _put_int(v, int(state["NumSubquantizers"]))
    cbs = state.get("Codebooks")
    if cbs is not None and len(cbs):
        field(6)
        _put_uint(v, len(cbs))
        for cb in cbs:
            put_vec2(cb)
    if state.get("PqK", 0):
        field(7)
        _put_int(v, int(state["PqK"]))
    if state.get("KMeansIters", 0):
        field(8)
        _put_int(v, int(state["KMeansIters"]))
    if state.get("AllowBruteForceFallback"):
        field(9)
        _put_uint(v, 1)
    if state.get("Trained"):
        field(10)
        _put_uint(v, 1)
    pend = state.get("PendingVectors") or {}
    if pend:
        field(11)
        _put_uint(v, len(pend))
        for pid in sorted(pend):
            _put_int(v, int(pid))
            _float_list(v, pend[pid])
    field(12)
    _put_int(v, FORMAT_VERSION)
    if state.get("NumCandidateClusters", 0):
        field(13)
        _put_int(v, int(state["NumCandidateClusters"]))
    _put_uint(v, 0)
    inner.value(t_ser, bytes(v))
    inner_bytes = bytes(inner.out)

    outer = _Encoder()
    t_idx = outer.define_gobencoder("*pqivf.Index")
    payload = bytearray()
    _put_uint(payload, 0)  # singleton prefix
    _put_str(payload, inner_bytes)
    outer.value(t_idx, bytes(payload))
    return bytes(outer.out)


def decode_pqivf(data: bytes) -> dict:
    """Decode a stream written by the reference's Save (or encode_pqivf)
    into a state dict with numpy arrays where the shapes allow."""
    outer = decode_stream(data)
    if not outer:
        raise GobError("empty gob stream")
    name, val = outer[0]
    if isinstance(val, (bytes, bytearray)):
        inner = decode_stream(val)
        if not inner:
            raise GobError("empty inner gob stream")
        _, ser = inner[0]
    elif isinstance(val, dict):
        ser = val
    else:
        raise GobError("unexpected top-level gob value")
    return ser


def read_pqivf(path_or_file) -> dict:
    if isinstance(path_or_file, (str, bytes)) and not isinstance(path_or_file, bytes):
        with open(path_or_file, "rb") as f:
            return decode_pqivf(f.read())
    if isinstance(path_or_file, (bytes, bytearray)):
        return decode_pqivf(path_or_file)
    return decode_pqivf(path_or_file.read())
