"""CPU oracle for the hann PQIVF path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this package, and only as the checker or the timed CPU baseline.
The ``hann_gb300`` product never imports it.

Contents:
  * ctypes bindings to ``libhann_oracle.so`` (``hann_oracle.c``), the C
    restatement of the reference's FP32 arithmetic (core/simd_kernels.inc.h,
    pqivf/index.go);
  * ``train`` -- pqivf/index.go:451-605 (Train) composed from the C pieces,
    with the k-means init and reseed indices as explicit inputs;
  * ``brute_force_knn_fp64`` -- FP64 ground truth with the id tie-break of
    internal/testutil/data.go:66-93;
  * ``RefKernels`` -- the reference's own distance kernels compiled from the
    reference tree into ``_ref/libhannref.so`` (only where that tree exists),
    used to pin the restated summation orders.

Parity pins for the restatement are in tests/test_oracle.py: the known answers
of core/distance_test.go:14-123, bit-exact agreement with the compiled
reference kernels for every tier this CPU runs, and the golden fixture
pqivf/testdata/index_v1.gob (codes and cluster assignments re-derived).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhann_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libhannref.so")

TIER_FALLBACK, TIER_AVX, TIER_AVX2, TIER_NEON = 0, 1, 2, 3
METRIC_SQEUCLID, METRIC_EUCLID, METRIC_MANHATTAN, METRIC_COSINE = 0, 1, 2, 3

_lock = threading.Lock()
_lib = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def build(force: bool = False) -> None:
    """Compile the oracle (and, where the reference tree exists, _ref)."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "hann_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)
    ref = os.environ.get("HANN_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True, stdout=subprocess.DEVNULL)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = ctypes.CDLL(LIB_PATH)
            L.hann_oracle_sqeuclid_tier.restype = ctypes.c_float
            L.hann_oracle_sqeuclid_tier.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_int]
            L.hann_oracle_manhattan_tier.restype = ctypes.c_float
            L.hann_oracle_manhattan_tier.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_int]
            L.hann_oracle_cosine_tier.restype = ctypes.c_float
            L.hann_oracle_cosine_tier.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_int]
            L.hann_oracle_set_tier.argtypes = [ctypes.c_int]
            L.hann_oracle_get_tier.restype = ctypes.c_int
            L.hann_oracle_batch.argtypes = [ctypes.c_int, _f32p, _f32p, ctypes.c_size_t, ctypes.c_size_t, _f64p]
            L.hann_oracle_assign.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, _f32p, ctypes.c_int, _i32p,
                                             ctypes.c_int]
            L.hann_oracle_kmeans.restype = ctypes.c_int
            L.hann_oracle_kmeans.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             _i64p, _i64p, ctypes.c_int64, _f32p, _i64p, ctypes.c_int]
            L.hann_oracle_encode.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, _i32p, _f32p, ctypes.c_int,
                                             ctypes.c_int, _f32p, _i32p, ctypes.c_int]
            L.hann_oracle_search_batch.argtypes = [
                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p, _f32p, _i64p, _i64p, _f32p,
                _i32p, _u8p, _i32p, _f32p, ctypes.c_int64, _i32p, _i32p, ctypes.c_int, ctypes.c_int,
                _i64p, _f64p, _i32p, _i32p, ctypes.c_int]
            L.hann_oracle_search_batch_rerank.argtypes = [
                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p, _f32p, _i64p, _i64p, _f32p,
                _i32p, _u8p, _i32p, _f32p, ctypes.c_int64, _i32p, _i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                _i64p, _f64p, _i32p, _i32p, ctypes.c_int]
            L.hann_oracle_probe.argtypes = [ctypes.c_int, ctypes.c_int, _f32p, _f32p, ctypes.c_int, _i32p]
            L.hann_oracle_knn.argtypes = [ctypes.c_int, _f32p, ctypes.c_int64, _f32p, ctypes.c_int64, ctypes.c_int,
                                          ctypes.c_int, _i64p, _f64p, ctypes.c_int]
            _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def set_tier(tier: int) -> None:
    lib().hann_oracle_set_tier(tier)


def get_tier() -> int:
    return lib().hann_oracle_get_tier()


def sqeuclid(a, b, tier: int | None = None) -> float:
    a, b = _f32(a), _f32(b)
    t = get_tier() if tier is None else tier
    return float(lib().hann_oracle_sqeuclid_tier(_p(a, _f32p), _p(b, _f32p), a.size, t))


def manhattan(a, b, tier: int | None = None) -> float:
    a, b = _f32(a), _f32(b)
    t = get_tier() if tier is None else tier
    return float(lib().hann_oracle_manhattan_tier(_p(a, _f32p), _p(b, _f32p), a.size, t))


def cosine(a, b, tier: int | None = None) -> float:
    a, b = _f32(a), _f32(b)
    t = get_tier() if tier is None else tier
    return float(lib().hann_oracle_cosine_tier(_p(a, _f32p), _p(b, _f32p), a.size, t))


def batch(metric: int, q, flat) -> np.ndarray:
    """core/simd_kernels.inc.h:235-264: one query against every row."""
    q, flat = _f32(q), _f32(flat)
    dim = q.size
    n = flat.size // dim if dim else 0
    out = np.zeros(n, dtype=np.float64)
    if n:
        lib().hann_oracle_batch(metric, _p(q, _f32p), _p(flat, _f32p), dim, n, _p(out, _f64p))
    return out


METRICS = {"squared_euclidean": 0, "euclidean": 1, "manhattan": 2, "cosine": 3}


def knn(queries, base, k: int, metric="squared_euclidean", nthreads: int = 1):
    """testutil.BruteForceKNN (internal/testutil/data.go:66-93) per query over
    the tier's FP32 batch distances; ids are row numbers. Returns (ids int64
    [nq][k], dist float64 [nq][k]); slots past n hold -1 / +inf."""
    m = METRICS[metric] if isinstance(metric, str) else int(metric)
    base = _f32(base)
    n, dim = base.shape if base.ndim == 2 else (0, 0)
    q = _f32(queries).reshape(-1, dim) if dim else np.zeros((np.asarray(queries).shape[0], 0), np.float32)
    nq = q.shape[0]
    ids = np.zeros((nq, k), dtype=np.int64)
    dist = np.zeros((nq, k), dtype=np.float64)
    if nq:
        lib().hann_oracle_knn(m, _p(q, _f32p), nq, _p(base, _f32p), n, dim, k, _p(ids, _i64p), _p(dist, _f64p),
                              nthreads)
    return ids, dist


def assign(data, centroids, nthreads: int = 1) -> np.ndarray:
    """assignPoints (pqivf/index.go:738-789)."""
    data, centroids = _f32(data), _f32(centroids)
    n, dim = data.shape
    out = np.zeros(n, dtype=np.int32)
    if n:
        lib().hann_oracle_assign(_p(data, _f32p), n, dim, _p(centroids, _f32p), centroids.shape[0],
                                 _p(out, _i32p), nthreads)
    return out


def kmeans(data, k: int, iters: int, init_idx, reseed_idx=(), nthreads: int = 1):
    """runKMeans (pqivf/index.go:795-847) with explicit init/reseed rows.

    Returns (centroids[k_eff, dim], reseeds_used)."""
    data = _f32(data)
    n, dim = data.shape
    keff = min(k, n)
    init = np.ascontiguousarray(init_idx, dtype=np.int64)[:keff]
    if init.size < keff:
        raise ValueError("init_idx too short")
    rs = np.ascontiguousarray(reseed_idx, dtype=np.int64)
    if rs.size == 0:
        rs = np.zeros(1, dtype=np.int64)
        nrs = 0
    else:
        nrs = rs.size
    out = np.zeros((keff, dim), dtype=np.float32)
    used = ctypes.c_int64(0)
    rc = lib().hann_oracle_kmeans(_p(data, _f32p), n, dim, k, iters, _p(init, _i64p), _p(rs, _i64p), nrs,
                                  _p(out, _f32p), ctypes.byref(used), nthreads)
    if rc == -1:
        raise RuntimeError("reseed stream exhausted")
    if rc < 0:
        raise RuntimeError("no data for k-means training")
    return out, int(used.value)


def encode(x, cluster, coarse, codebooks, nthreads: int = 1) -> np.ndarray:
    """encodeWithCodebooks (pqivf/index.go:641-666). codebooks [M][pqK][dsub]."""
    x = _f32(x)
    cb = _f32(codebooks)
    M, pqK, _ = cb.shape
    cl = np.ascontiguousarray(cluster, dtype=np.int32)
    coarse = _f32(coarse)
    n, dim = x.shape
    out = np.zeros((n, M), dtype=np.int32)
    if n:
        lib().hann_oracle_encode(_p(x, _f32p), n, dim, _p(cl, _i32p), _p(coarse, _f32p), M, pqK,
                                 _p(cb, _f32p), _p(out, _i32p), nthreads)
    return out


class OracleIndex:
    """A trained PQIVF index in CSR form, as the oracle searches it.

    Lists are stored in ascending cluster order; within a list, entries keep
    the reference's storage order (ascending id after Train,
    pqivf/index.go:497-506)."""

    def __init__(self, dim, M, pqK, coarse, codebooks, list_ids, list_vectors, list_codes, fallback=True):
        self.dim, self.M, self.pqK = int(dim), int(M), int(pqK)
        self.coarse = _f32(coarse)
        self.nlist = self.coarse.shape[0]
        self.codebooks = _f32(codebooks).reshape(M, pqK, dim // M)
        off = [0]
        ids, vecs, codes, has, ecl = [], [], [], [], []
        for c in range(self.nlist):
            li = list_ids.get(c, []) if isinstance(list_ids, dict) else list_ids[c]
            lv = list_vectors.get(c, []) if isinstance(list_vectors, dict) else list_vectors[c]
            lc = list_codes.get(c, []) if isinstance(list_codes, dict) else list_codes[c]
            for j in range(len(li)):
                ids.append(int(li[j]))
                vecs.append(np.asarray(lv[j], dtype=np.float32))
                cj = lc[j] if lc is not None and j < len(lc) else None
                if cj is not None and len(cj) == M:
                    codes.append(np.asarray(cj, dtype=np.int32))
                    has.append(1)
                else:
                    codes.append(np.zeros(M, dtype=np.int32))
                    has.append(0)
                ecl.append(c)
            off.append(len(ids))
        self.list_off = np.asarray(off, dtype=np.int64)
        self.ids = np.asarray(ids, dtype=np.int64)
        self.vectors = np.asarray(vecs, dtype=np.float32).reshape(-1, dim)
        self.codes = np.asarray(codes, dtype=np.int32).reshape(-1, M)
        self.has_codes = np.asarray(has, dtype=np.uint8)
        self.entry_cluster = np.asarray(ecl, dtype=np.int32)
        self.fallback = bool(fallback)

    @classmethod
    def from_csr(cls, dim, M, pqK, coarse, codebooks, list_len, ids, vectors, codes, fallback=True):
        """Build directly from list-ordered arrays (no per-entry Python work)."""
        self = cls.__new__(cls)
        self.dim, self.M, self.pqK = int(dim), int(M), int(pqK)
        self.coarse = _f32(coarse)
        self.nlist = self.coarse.shape[0]
        self.codebooks = _f32(codebooks).reshape(M, pqK, dim // M)
        ll = np.asarray(list_len, dtype=np.int64)
        self.list_off = np.concatenate([[0], np.cumsum(ll)]).astype(np.int64)
        self.ids = np.ascontiguousarray(ids, dtype=np.int64)
        self.vectors = _f32(vectors).reshape(-1, dim)
        self.codes = np.ascontiguousarray(codes, dtype=np.int32).reshape(-1, M)
        self.has_codes = np.ones(self.ids.size, dtype=np.uint8)
        self.entry_cluster = np.repeat(np.arange(self.nlist, dtype=np.int32), ll)
        self.fallback = bool(fallback)
        return self

    @property
    def count(self) -> int:
        return int(self.ids.size)

    def search(self, queries, k, nprobe, nthreads: int = 1, rerank: int = 0):
        """Independent Search calls (pqivf/index.go:850-949). With rerank > 0,
        the `rerank` best candidates by PQ distance are reordered by the exact
        distance to their stored vectors (the GPU's exact-rerank mode on the
        CPU; the reference itself has no such mode).

        Returns (ids[nq][kmax], dist[nq][kmax], n[nq], fallback[nq])."""
        q = _f32(queries).reshape(-1, self.dim)
        nq = q.shape[0]
        kk = np.broadcast_to(np.asarray(k, dtype=np.int32), (nq,)).copy()
        npr = np.broadcast_to(np.asarray(nprobe, dtype=np.int32), (nq,)).copy()
        kmax = int(kk.max()) if nq else 1
        ids = np.full((nq, kmax), -1, dtype=np.int64)
        dist = np.zeros((nq, kmax), dtype=np.float64)
        nout = np.zeros(nq, dtype=np.int32)
        fb = np.zeros(nq, dtype=np.int32)
        # empty arrays still need valid pointers
        vecs = self.vectors if self.vectors.size else np.zeros((1, self.dim), np.float32)
        codes = self.codes if self.codes.size else np.zeros((1, self.M), np.int32)
        has = self.has_codes if self.has_codes.size else np.zeros(1, np.uint8)
        ecl = self.entry_cluster if self.entry_cluster.size else np.zeros(1, np.int32)
        idsin = self.ids if self.ids.size else np.zeros(1, np.int64)
        if nq:
            lib().hann_oracle_search_batch_rerank(
                self.dim, self.M, self.pqK, self.nlist, _p(self.coarse, _f32p), _p(self.codebooks, _f32p),
                _p(self.list_off, _i64p), _p(idsin, _i64p), _p(vecs, _f32p), _p(codes, _i32p),
                _p(has, _u8p), _p(ecl, _i32p), _p(q, _f32p), nq, _p(kk, _i32p), _p(npr, _i32p),
                int(self.fallback), int(rerank), kmax, _p(ids, _i64p), _p(dist, _f64p), _p(nout, _i32p),
                _p(fb, _i32p), nthreads)
        return ids, dist, nout, fb

    def probe(self, query, nprobe):
        q = _f32(query)
        npb = min(nprobe, self.nlist)
        out = np.zeros(npb, dtype=np.int32)
        lib().hann_oracle_probe(self.dim, self.nlist, _p(self.coarse, _f32p), _p(q, _f32p), nprobe,
                                _p(out, _i32p))
        return out


def train(ids, vectors, coarse_k, M, pqK, iters, coarse_init, pq_init, reseed_idx=(), nthreads: int = 1,
          fallback=True):
    """Train (pqivf/index.go:451-605) with explicit k-means init rows.

    ids/vectors: every vector the index holds (any order; Train sorts by id).
    coarse_init: row indices into the id-sorted data (perm[:coarse_k]).
    pq_init[m]: row indices into the residual data of subquantizer m, whose
    rows are in ascending cluster order, then list (ascending id) order.
    reseed_idx: one stream of rows for empty clusters, consumed in order by
    the coarse run and then subquantizers 0, 1, ... (the reference's single
    package RNG, pqivf/index.go:22, 830-837).
    Returns (OracleIndex, info dict)."""
    ids = np.asarray(ids, dtype=np.int64)
    vectors = _f32(vectors)
    if ids.size < coarse_k:
        raise ValueError("not enough vectors (%d) to train coarse quantizer with %d clusters"
                         % (ids.size, coarse_k))
    order = np.argsort(ids, kind="stable")
    ids_s = ids[order]
    data = vectors[order]
    n, dim = data.shape
    stream = np.asarray(reseed_idx, dtype=np.int64)
    coarse, cr_used = kmeans(data, coarse_k, iters, coarse_init, stream, nthreads)
    pos = cr_used
    asg = assign(data, coarse, nthreads)
    nl = coarse.shape[0]
    dsub = dim // M
    # residuals in ascending cluster order, then ascending id order
    res_order = np.lexsort((ids_s, asg))
    residual = data[res_order] - coarse[asg[res_order]]
    codebooks = []
    pq_used = []
    for m in range(M):
        sub = np.ascontiguousarray(residual[:, m * dsub:(m + 1) * dsub])
        cb, used = kmeans(sub, pqK, iters, pq_init[m], stream[pos:], nthreads)
        pos += used
        codebooks.append(cb)
        pq_used.append(used)
    kpq = codebooks[0].shape[0]
    cbs = np.stack(codebooks).reshape(M, kpq, dsub)
    codes = encode(data, asg, coarse, cbs, nthreads)
    list_ids = {c: [] for c in range(nl)}
    list_vecs = {c: [] for c in range(nl)}
    list_codes = {c: [] for c in range(nl)}
    for r in res_order:
        c = int(asg[r])
        list_ids[c].append(int(ids_s[r]))
        list_vecs[c].append(data[r])
        list_codes[c].append(codes[r])
    ix = OracleIndex(dim, M, kpq, coarse, cbs, list_ids, list_vecs, list_codes, fallback=fallback)
    info = {"assign": asg, "ids_sorted": ids_s, "codes": codes, "coarse_reseeds": cr_used,
            "pq_reseeds": pq_used}
    return ix, info


def inertia_fp64(data, centroids, assignment) -> float:
    """Sum of squared distances of every point to its assigned centroid, FP64."""
    d = np.asarray(data, dtype=np.float64) - np.asarray(centroids, dtype=np.float64)[assignment]
    return float(np.einsum("ij,ij->", d, d))


def brute_force_knn_fp64(queries, base, k, metric="euclidean", base_ids=None):
    """FP64 exact k-NN, ties broken by id (internal/testutil/data.go:66-93)."""
    q = np.asarray(queries, dtype=np.float64).reshape(-1, np.asarray(base).shape[1])
    x = np.asarray(base, dtype=np.float64)
    ids = np.arange(x.shape[0]) if base_ids is None else np.asarray(base_ids)
    out_ids = np.zeros((q.shape[0], min(k, x.shape[0])), dtype=np.int64)
    out_d = np.zeros_like(out_ids, dtype=np.float64)
    xn = np.einsum("ij,ij->i", x, x)
    for s in range(0, q.shape[0], 256):
        qb = q[s:s + 256]
        if metric in ("euclidean", "sqeuclidean"):
            d = np.einsum("ij,ij->i", qb, qb)[:, None] - 2.0 * qb @ x.T + xn[None, :]
            np.maximum(d, 0, out=d)
            if metric == "euclidean":
                d = np.sqrt(d)
        elif metric == "manhattan":
            d = np.abs(qb[:, None, :] - x[None, :, :]).sum(-1)
        elif metric == "cosine":
            qn = np.sqrt(np.einsum("ij,ij->i", qb, qb))
            bn = np.sqrt(xn)
            dot = qb @ x.T
            den = qn[:, None] * bn[None, :]
            with np.errstate(divide="ignore", invalid="ignore"):
                s_ = np.where(den == 0, 0.0, dot / np.where(den == 0, 1, den))
            d = np.where(den == 0, 1.0, 1.0 - np.clip(s_, -1, 1))
        else:
            raise ValueError(metric)
        for i in range(qb.shape[0]):
            o = np.lexsort((ids, d[i]))[:out_ids.shape[1]]
            out_ids[s + i] = ids[o]
            out_d[s + i] = d[i][o]
    return out_ids, out_d


class RefKernels:
    """The reference's own C distance kernels (core/simd_distance.c,
    core/simd_ops.c), compiled unchanged into _ref/libhannref.so."""

    def __init__(self):
        if not os.path.exists(REF_PATH):
            raise FileNotFoundError(REF_PATH)
        L = ctypes.CDLL(REF_PATH)
        for name in ("simd_euclidean", "simd_squared_euclidean", "simd_manhattan", "simd_cosine_distance"):
            f = getattr(L, name)
            f.restype = ctypes.c_float
            f.argtypes = [_f32p, _f32p, ctypes.c_size_t]
        for name in ("simd_euclidean_batch", "simd_squared_euclidean_batch", "simd_manhattan_batch",
                     "simd_cosine_distance_batch"):
            f = getattr(L, name)
            f.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_size_t, _f64p]
        L.hann_cpu_init.argtypes = [ctypes.c_int]
        self.L = L

    def init(self, tier: int) -> None:
        self.L.hann_cpu_init(tier)

    def pair(self, name, a, b) -> float:
        a, b = _f32(a), _f32(b)
        return float(getattr(self.L, "simd_" + name)(_p(a, _f32p), _p(b, _f32p), a.size))

    def batch(self, name, q, flat) -> np.ndarray:
        q, flat = _f32(q), _f32(flat)
        n = flat.size // q.size
        out = np.zeros(n, dtype=np.float64)
        getattr(self.L, "simd_" + name + "_batch")(_p(q, _f32p), _p(flat, _f32p), q.size, n, _p(out, _f64p))
        return out
