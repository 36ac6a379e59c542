"""Shared test helpers: tie-aware result comparison and state conversion."""
from __future__ import annotations

import numpy as np

import oracle
from hann_gb300 import gob

# Distance tolerance of the parity bar: 1e-5 relative.
REL = 1e-5


def state_to_oracle(st: dict, fallback=None) -> oracle.OracleIndex:
    lay = st["layout"]
    ids, vecs, codes = {}, {}, {}
    off = 0
    for c in range(lay["nlist"]):
        n = int(st["list_len"][c])
        ids[c] = st["ids"][off:off + n]
        vecs[c] = st["vectors"][off:off + n]
        codes[c] = st["codes"][off:off + n]
        off += n
    fb = bool(lay["fallback"]) if fallback is None else fallback
    return oracle.OracleIndex(lay["dimension"], lay["num_subquantizers"], lay["pq_k_eff"], st["coarse"],
                              st["codebooks"], ids, vecs, codes, fallback=fb)


def gob_to_oracle(ser: dict) -> oracle.OracleIndex:
    dim = ser["Dimension"]
    M = ser["NumSubquantizers"]
    coarse = np.asarray(ser["CoarseCentroids"], np.float32)
    cbs = np.asarray(ser["Codebooks"], np.float32)
    lists = ser.get("InvertedLists") or {}
    ids = {c: [e.get("ID", 0) for e in es] for c, es in lists.items()}
    vecs = {c: [e["Vector"] for e in es] for c, es in lists.items()}
    codes = {c: [e.get("Codes") for e in es] for c, es in lists.items()}
    return oracle.OracleIndex(dim, M, cbs.shape[1], coarse, cbs, ids, vecs, codes,
                              fallback=bool(ser.get("AllowBruteForceFallback")))


def assert_same_results(g_ids, g_d, g_n, o_ids, o_d, o_n, rel=REL):
    """Identical ids except inside ties (reference distances within rel),
    distances within rel, counts equal."""
    g_n = np.asarray(g_n)
    o_n = np.asarray(o_n)
    assert (g_n == o_n).all(), ("result counts differ", np.nonzero(g_n != o_n)[0][:10])
    for i in range(len(g_n)):
        c = int(g_n[i])
        gd, od = np.asarray(g_d[i][:c], np.float64), np.asarray(o_d[i][:c], np.float64)
        tol = rel * np.maximum(np.abs(od), 1e-12) + 1e-12
        bad = np.abs(gd - od) > tol
        assert not bad.any(), ("distance mismatch", i, gd[bad][:5], od[bad][:5])
        gi, oi = list(g_ids[i][:c]), list(o_ids[i][:c])
        for j in range(c):
            if gi[j] == oi[j]:
                continue
            # gi[j] must sit in the oracle list at a tied distance, or tie the
            # oracle's last distance (the cut-off).
            ok = False
            if gi[j] in oi:
                jj = oi.index(gi[j])
                ok = abs(od[jj] - od[j]) <= rel * max(abs(od[j]), 1e-12) + 1e-12
            else:
                ok = abs(gd[j] - od[c - 1]) <= rel * max(abs(od[c - 1]), 1e-12) + 1e-12
            assert ok, ("id mismatch outside a tie", i, j, gi, oi, gd, od)


def gaussian_mixture(rng, n, dim, centers, sigma, center_scale=1.0):
    c = rng.normal(size=(centers, dim)) * center_scale
    lab = rng.integers(0, centers, n)
    x = c[lab] + sigma * rng.normal(size=(n, dim))
    return x.astype(np.float32), c.astype(np.float32)


def flat_struct_stream(fields):
    """A gob stream holding one struct of int fields, as gob.NewEncoder
    writes an anonymous struct value (the reference's tests build old and
    future formats this way: fields are matched by name)."""
    enc = gob._Encoder()
    tid = enc.define_struct("", [(name, gob.T_INT) for name, _ in fields])
    v = bytearray()
    last = -1
    for i, (_, val) in enumerate(fields):
        if val:
            gob._put_uint(v, i - last)
            last = i
            gob._put_int(v, val)
    gob._put_uint(v, 0)
    enc.value(tid, bytes(v))
    return bytes(enc.out)
