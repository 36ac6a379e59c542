"""hann_gb300 -- GB300-native PQIVF index with the interface of hann's pqivf.

The index lives on one GPU; this module is a thin ctypes binding over the C
ABI in ``include/hann_gb300.h`` (``libhann_gb300.so``, built by
``hann_gb300.build``). It mirrors the reference's Go API
(pqivf/index.go, core/index.go): ``New(dim, With...(...))`` and the methods
Add, BulkAdd, Delete, BulkDelete, Update, BulkUpdate, Train, Search, Stats,
Save and Load, with the same argument meaning, error conditions and error
messages. Errors raise :class:`HannError`.

There is no CPU fallback: if the CUDA library is missing or cannot load,
importing the binding's entry points raises.
"""
from __future__ import annotations

import ctypes
import io
import os
import threading
from typing import Dict, Iterable, List, NamedTuple, Sequence

import numpy as np

from . import gob

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhann_gb300.so")

HANN_OK = 0
HANN_E_INVALID = -1
HANN_E_NOT_FOUND = -2
HANN_E_EXISTS = -3
HANN_E_STATE = -4
HANN_E_CUDA = -5
HANN_E_NOMEM = -6
HANN_E_UNSUPPORTED = -7
HANN_E_CHANGED = -8

MODE_PARITY = 0
MODE_EXACT_RERANK = 1

METRIC_SQEUCLID, METRIC_EUCLID, METRIC_MANHATTAN, METRIC_COSINE = 0, 1, 2, 3

HANN_TUNE_LADDER_MAX = 14


class HannError(Exception):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class Neighbor(NamedTuple):
    """core.Neighbor (core/index.go:125-128)."""
    ID: int
    Distance: float


class IndexStats(NamedTuple):
    """core.IndexStats (core/index.go:131-140)."""
    Count: int
    Dimension: int
    Distance: str
    FallbackSearches: int


class _Options(ctypes.Structure):
    _fields_ = [("dimension", ctypes.c_int32), ("coarse_k", ctypes.c_int32),
                ("num_subquantizers", ctypes.c_int32), ("pq_k", ctypes.c_int32),
                ("kmeans_iters", ctypes.c_int32), ("candidate_clusters", ctypes.c_int32),
                ("fallback", ctypes.c_int32), ("seed", ctypes.c_uint64), ("device", ctypes.c_int32),
                ("rerank", ctypes.c_int32), ("plain_fp32", ctypes.c_int32)]


class _Stats(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("dimension", ctypes.c_int32),
                ("fallback_searches", ctypes.c_int64), ("trained", ctypes.c_int32), ("nlist", ctypes.c_int32),
                ("rows_capacity", ctypes.c_int64)]


class _Layout(ctypes.Structure):
    _fields_ = [("dimension", ctypes.c_int32), ("coarse_k", ctypes.c_int32),
                ("num_subquantizers", ctypes.c_int32), ("pq_k", ctypes.c_int32),
                ("kmeans_iters", ctypes.c_int32), ("candidate_clusters", ctypes.c_int32),
                ("fallback", ctypes.c_int32), ("trained", ctypes.c_int32), ("nlist", ctypes.c_int32),
                ("pq_k_eff", ctypes.c_int32), ("n_rows", ctypes.c_int64), ("n_pending", ctypes.c_int64)]


_P = ctypes.c_void_p
_lib = None
_lib_lock = threading.Lock()

# Every entry point include/hann_gb300.h declares.
EXPORTED = (
    "hann_pqivf_options_init", "hann_pqivf_new", "hann_pqivf_free", "hann_pqivf_last_error", "hann_pqivf_add",
    "hann_pqivf_bulk_add", "hann_pqivf_delete", "hann_pqivf_bulk_delete", "hann_pqivf_update",
    "hann_pqivf_bulk_update", "hann_pqivf_train", "hann_pqivf_train_seeded", "hann_pqivf_search",
    "hann_pqivf_search_batch", "hann_pqivf_search_batch_device", "hann_pqivf_stats", "hann_pqivf_export_layout",
    "hann_pqivf_export", "hann_pqivf_import", "hann_gpu_distance_batch", "hann_pqivf_set_profiling",
    "hann_pqivf_stage_times", "hann_pqivf_list_lengths", "hann_pqivf_search_batch_device_noalloc",
    "hann_gpu_distance_matrix", "hann_knn_new", "hann_knn_free", "hann_knn_last_error", "hann_knn_search",
    "hann_knn_search_device", "hann_knn_get_stats", "hann_gpu_knn", "hann_pqivf_set_plain_fp32",
    "hann_serve_submit_priority", "hann_serve_cancel", "hann_pqivf_set_candidate_clusters",
    "hann_pqivf_save_snapshot", "hann_pqivf_load_snapshot", "hann_pqivf_retrain", "hann_gob_encode",
    "hann_gob_decode", "hann_gob_state_layout", "hann_gob_state_arrays", "hann_gob_state_free",
    "hann_gob_last_error", "hann_gob_encode_payload", "hann_pqivf_tune_candidate_clusters",
    "hann_pqivf_autotune_scan", "hann_pqivf_set_adc_tables", "hann_knn_append", "hann_knn_distance_gather",
    "hann_knn_distance_gather_device",
)
# Entry points of include/hann_gb300_diag.h.
EXPORTED_DIAG = ("hann_gpu_bf16_scores", "hann_gpu_pq_assign", "hann_pqivf_arena_stats", "hann_pqivf_rows_decoded",
                 "hann_pqivf_adc_redos",
                 "hann_pqivf_train_stats", "hann_pqivf_train_phases",
                 "hann_pqivf_scan_options")


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libhann_gb300.so. Raises when it is missing: there is no fallback."""
    global _lib
    with _lib_lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                "libhann_gb300.so is not built (run hann_gb300.build.build()); the GPU index has no CPU fallback")
        L = ctypes.CDLL(p)
        L.hann_pqivf_options_init.argtypes = [ctypes.POINTER(_Options), ctypes.c_int32]
        L.hann_pqivf_options_init.restype = None
        L.hann_pqivf_new.argtypes = [ctypes.POINTER(_Options), ctypes.POINTER(_P)]
        L.hann_pqivf_free.argtypes = [_P]
        L.hann_pqivf_free.restype = None
        L.hann_pqivf_last_error.argtypes = [_P]
        L.hann_pqivf_last_error.restype = ctypes.c_char_p
        L.hann_pqivf_add.argtypes = [_P, ctypes.c_int64, _P]
        L.hann_pqivf_bulk_add.argtypes = [_P, _P, _P, ctypes.c_int64]
        L.hann_pqivf_delete.argtypes = [_P, ctypes.c_int64]
        L.hann_pqivf_bulk_delete.argtypes = [_P, _P, ctypes.c_int64]
        L.hann_pqivf_update.argtypes = [_P, ctypes.c_int64, _P]
        L.hann_pqivf_bulk_update.argtypes = [_P, _P, _P, ctypes.c_int64]
        L.hann_pqivf_train.argtypes = [_P]
        L.hann_pqivf_train_seeded.argtypes = [_P, _P, _P, _P, ctypes.c_int64]
        L.hann_pqivf_search.argtypes = [_P, _P, ctypes.c_int32, _P, _P, _P]
        L.hann_pqivf_search_batch.argtypes = [_P, _P, ctypes.c_int64, _P, _P, ctypes.c_int32, ctypes.c_int32, _P,
                                              _P, _P]
        L.hann_pqivf_search_batch_device.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                                     ctypes.c_int32, _P, _P, _P, _P]
        L.hann_pqivf_stats.argtypes = [_P, ctypes.POINTER(_Stats)]
        L.hann_pqivf_export_layout.argtypes = [_P, ctypes.POINTER(_Layout)]
        L.hann_pqivf_export.argtypes = [_P, ctypes.POINTER(_Layout)] + [_P] * 10
        L.hann_pqivf_import.argtypes = [_P, ctypes.POINTER(_Layout)] + [_P] * 11
        L.hann_gpu_distance_batch.argtypes = [ctypes.c_int32, _P, _P, ctypes.c_size_t, ctypes.c_size_t, _P]
        L.hann_pqivf_set_profiling.argtypes = [_P, ctypes.c_int32]
        L.hann_pqivf_set_plain_fp32.argtypes = [_P, ctypes.c_int32]
        L.hann_pqivf_set_adc_tables.argtypes = [_P, ctypes.c_int32]
        L.hann_pqivf_adc_redos.argtypes = [_P, _P]
        L.hann_pqivf_train_stats.argtypes = [_P, _P]
        L.hann_pqivf_train_phases.argtypes = [_P, _P]
        L.hann_pqivf_set_candidate_clusters.argtypes = [_P, ctypes.c_int32]
        L.hann_pqivf_autotune_scan.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P, _P, _P]
        L.hann_pqivf_tune_candidate_clusters.argtypes = [_P, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                                         _P, ctypes.c_int32, ctypes.c_int32, _P, ctypes.c_int32,
                                                         _P, _P, _P, _P]
        L.hann_pqivf_arena_stats.argtypes = [_P, _P]
        L.hann_pqivf_rows_decoded.argtypes = [_P, _P]
        L.hann_pqivf_scan_options.argtypes = [_P, _P, _P]
        L.hann_pqivf_retrain.argtypes = [_P, ctypes.c_int32]
        L.hann_pqivf_save_snapshot.argtypes = [_P, ctypes.c_char_p]
        L.hann_pqivf_load_snapshot.argtypes = [_P, ctypes.c_char_p]
        L.hann_gob_encode.argtypes = [ctypes.POINTER(_Layout)] + [_P] * 11 + [ctypes.c_int64, _P]
        L.hann_gob_encode_payload.argtypes = L.hann_gob_encode.argtypes
        L.hann_gob_decode.argtypes = [_P, ctypes.c_int64, ctypes.POINTER(_P)]
        L.hann_gob_state_layout.argtypes = [_P, ctypes.c_int32, ctypes.POINTER(_Layout)]
        L.hann_gob_state_arrays.argtypes = [_P] * 12
        L.hann_gob_state_free.argtypes = [_P]
        L.hann_gob_state_free.restype = None
        L.hann_gob_last_error.argtypes = []
        L.hann_gob_last_error.restype = ctypes.c_char_p
        L.hann_pqivf_stage_times.argtypes = [_P, _P, _P, _P]
        L.hann_pqivf_list_lengths.argtypes = [_P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.hann_gpu_distance_matrix.argtypes = [ctypes.c_int32, _P, ctypes.c_int64, _P, ctypes.c_int64,
                                               ctypes.c_int32, _P]
        L.hann_knn_new.argtypes = [_P, ctypes.c_int64, ctypes.c_int32]
        L.hann_knn_append.argtypes = [_P, _P, ctypes.c_int64]
        L.hann_knn_distance_gather.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int64, _P, _P, _P]
        L.hann_knn_distance_gather_device.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int64, _P, _P,
                                                      ctypes.c_int64, _P, _P]
        L.hann_knn_new.restype = _P
        L.hann_knn_free.argtypes = [_P]
        L.hann_knn_free.restype = None
        L.hann_knn_last_error.argtypes = [_P]
        L.hann_knn_last_error.restype = ctypes.c_char_p
        L.hann_knn_search.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P,
                                      _P]
        L.hann_knn_search_device.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int64, ctypes.c_int32,
                                             ctypes.c_int32, _P, _P, _P]
        L.hann_knn_get_stats.argtypes = [_P, _P]
        L.hann_gpu_knn.argtypes = [ctypes.c_int32, _P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int32,
                                   ctypes.c_int32, ctypes.c_int32, _P, _P]
        if path is None:
            _lib = L
        return L


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


# ---------------------------------------------------------------------------
# Options, as the reference's functional options (pqivf/index.go:56-94).

def WithCoarseK(k: int):
    return lambda o: setattr(o, "coarse_k", int(k))


def WithNumSubquantizers(m: int):
    return lambda o: setattr(o, "num_subquantizers", int(m))


def WithPQK(k: int):
    return lambda o: setattr(o, "pq_k", int(k))


def WithKMeansIters(n: int):
    return lambda o: setattr(o, "kmeans_iters", int(n))


def WithCandidateClusters(n: int):
    return lambda o: setattr(o, "candidate_clusters", int(n))


def WithBruteForceFallback(allow: bool):
    return lambda o: setattr(o, "fallback", 1 if allow else 0)


def WithPlainFP32(on: bool = True):
    """Every assignment and probe on the FP32 SIMT kernels (no tensor-core
    preselection); the results are the same."""
    return lambda o: setattr(o, "plain_fp32", 1 if on else 0)


def WithSeed(seed: int):
    """The index's k-means seeding source (the reference reads HANN_SEED)."""
    return lambda o: setattr(o, "seed", int(seed) & 0xFFFFFFFFFFFFFFFF)


def WithDevice(device: int):
    return lambda o: setattr(o, "device", int(device))


def WithRerank(r: int):
    """Candidates rescored exactly per query (0 = automatic)."""
    return lambda o: setattr(o, "rerank", int(r))


def New(dimension: int, *opts) -> "Index":
    """pqivf.New (pqivf/index.go:106-146)."""
    return Index(dimension, *opts)


class Index:
    """GPU PQIVF index with the method set of the reference's pqivf.Index."""

    def __init__(self, dimension: int, *opts):
        L = load_library()
        o = _Options()
        L.hann_pqivf_options_init(ctypes.byref(o), int(dimension))
        if "HANN_SEED" in os.environ:
            try:
                o.seed = int(os.environ["HANN_SEED"]) & 0xFFFFFFFFFFFFFFFF
            except ValueError:
                pass
        for fn in opts:
            fn(o)
        h = _P()
        rc = L.hann_pqivf_new(ctypes.byref(o), ctypes.byref(h))
        if rc != HANN_OK:
            raise HannError(rc, L.hann_pqivf_last_error(None).decode())
        self._L = L
        self._h = h
        self._opts = o
        self._dim = int(dimension)

    # -- plumbing ----------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != HANN_OK:
            raise HannError(rc, self._L.hann_pqivf_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.hann_pqivf_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def dimension(self) -> int:
        return self._dim

    def _vec(self, v) -> np.ndarray:
        return np.ascontiguousarray(v, dtype=np.float32).reshape(-1)

    def _dim_error(self, got: int) -> HannError:
        return HannError(HANN_E_INVALID, "vector dimension %d does not match index dimension %d" % (got, self._dim))

    # -- core.Index ----------------------------------------------------------
    def Add(self, id: int, vector) -> None:
        v = self._vec(vector)
        if v.size != self._dim:
            raise self._dim_error(v.size)
        self._check(self._L.hann_pqivf_add(self._h, int(id), _ptr(v)))

    def BulkAdd(self, vectors: Dict[int, Sequence[float]]) -> None:
        keys = sorted(int(k) for k in vectors)
        good: List[int] = []
        bad = None
        for k in keys:
            v = self._vec(vectors[k])
            if v.size != self._dim:
                bad = (k, v.size)
                break
            good.append(k)
        if good:
            ids = np.asarray(good, dtype=np.int64)
            mat = np.stack([self._vec(vectors[k]) for k in good]).astype(np.float32)
            self._check(self._L.hann_pqivf_bulk_add(self._h, _ptr(ids), _ptr(mat), ids.size))
        if bad is not None:
            raise HannError(HANN_E_INVALID, "vector dimension %d does not match index dimension %d for id %d"
                            % (bad[1], self._dim, bad[0]))

    def BulkAddArrays(self, ids, matrix) -> None:
        """BulkAdd from an id array and a row-major [n, dim] float32 matrix."""
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        mat = np.ascontiguousarray(matrix, dtype=np.float32)
        if mat.ndim != 2 or mat.shape[1] != self._dim or mat.shape[0] != ids.size:
            raise HannError(HANN_E_INVALID, "matrix shape does not match ids and index dimension")
        self._check(self._L.hann_pqivf_bulk_add(self._h, _ptr(ids), _ptr(mat), ids.size))

    def Delete(self, id: int) -> None:
        self._check(self._L.hann_pqivf_delete(self._h, int(id)))

    def BulkDelete(self, ids: Iterable[int]) -> None:
        a = np.asarray(list(ids), dtype=np.int64)
        self._check(self._L.hann_pqivf_bulk_delete(self._h, _ptr(a), a.size))

    def Update(self, id: int, vector) -> None:
        v = self._vec(vector)
        if v.size != self._dim:
            raise self._dim_error(v.size)
        self._check(self._L.hann_pqivf_update(self._h, int(id), _ptr(v)))

    def BulkUpdate(self, updates: Dict[int, Sequence[float]]) -> None:
        keys = sorted(int(k) for k in updates)
        for k in keys:
            v = self._vec(updates[k])
            if v.size != self._dim:
                raise HannError(HANN_E_INVALID, "invalid vector for id %d: vector dimension %d does not match "
                                "index dimension %d" % (k, v.size, self._dim))
        if not keys:
            return
        ids = np.asarray(keys, dtype=np.int64)
        mat = np.stack([self._vec(updates[k]) for k in keys]).astype(np.float32)
        self._check(self._L.hann_pqivf_bulk_update(self._h, _ptr(ids), _ptr(mat), ids.size))

    def Train(self) -> None:
        self._check(self._L.hann_pqivf_train(self._h))

    def TrainSeeded(self, coarse_init=None, pq_init=None, reseed=None) -> None:
        """Train with explicit k-means init rows and reseed stream."""
        ci = None if coarse_init is None else np.ascontiguousarray(coarse_init, dtype=np.int64)
        pi = None if pq_init is None else np.ascontiguousarray(pq_init, dtype=np.int64)
        rs = None if reseed is None else np.ascontiguousarray(reseed, dtype=np.int64)
        nrs = 0 if rs is None else rs.size
        if rs is not None and rs.size == 0:
            rs = np.zeros(1, dtype=np.int64)
        self._check(self._L.hann_pqivf_train_seeded(
            self._h, _ptr(ci) if ci is not None else None, _ptr(pi) if pi is not None else None,
            _ptr(rs) if rs is not None else None, nrs))

    def _stats_raw(self) -> _Stats:
        s = _Stats()
        self._check(self._L.hann_pqivf_stats(self._h, ctypes.byref(s)))
        return s

    def Search(self, query, k: int) -> List[Neighbor]:
        if int(k) <= 0:
            raise HannError(HANN_E_INVALID, "k must be positive")
        if not self._stats_raw().trained:
            raise HannError(HANN_E_STATE,
                            "PQIVF index is not trained. Call Train() after adding data before searching")
        q = self._vec(query)
        if q.size != self._dim:
            raise HannError(HANN_E_INVALID, "query dimension %d does not match index dimension %d"
                            % (q.size, self._dim))
        k = int(k)
        ids = np.zeros(k, dtype=np.int64)
        dist = np.zeros(k, dtype=np.float64)
        n = ctypes.c_int32(0)
        self._check(self._L.hann_pqivf_search(self._h, _ptr(q), k, _ptr(ids), _ptr(dist), ctypes.byref(n)))
        return [Neighbor(int(ids[i]), float(dist[i])) for i in range(n.value)]

    def SearchBatch(self, queries, k, nprobe=None, mode: int = MODE_PARITY):
        """Batched Search. Returns (ids [nq, kmax], distances [nq, kmax], counts [nq])."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q.reshape(1, -1)
        if q.shape[1] != self._dim:
            raise HannError(HANN_E_INVALID, "query dimension %d does not match index dimension %d"
                            % (q.shape[1], self._dim))
        nq = q.shape[0]
        kk = np.broadcast_to(np.asarray(k, dtype=np.int32), (nq,)).copy()
        kmax = int(kk.max()) if nq else 1
        npb = None if nprobe is None else np.broadcast_to(np.asarray(nprobe, dtype=np.int32), (nq,)).copy()
        ids = np.full((nq, kmax), -1, dtype=np.int64)
        dist = np.zeros((nq, kmax), dtype=np.float64)
        nout = np.zeros(nq, dtype=np.int32)
        self._check(self._L.hann_pqivf_search_batch(
            self._h, _ptr(q), nq, _ptr(kk), _ptr(npb) if npb is not None else None, kmax, int(mode), _ptr(ids),
            _ptr(dist), _ptr(nout)))
        return ids, dist, nout

    def SearchBatchDevice(self, d_queries: int, nq: int, k: int, nprobe: int, mode: int, d_ids: int, d_dist: int,
                          d_nout: int, stream: int = 0) -> None:
        """Device-pointer batch search (integers are device addresses)."""
        self._check(self._L.hann_pqivf_search_batch_device(
            self._h, ctypes.c_void_p(d_queries), int(nq), int(k), int(nprobe), int(mode), ctypes.c_void_p(d_ids),
            ctypes.c_void_p(d_dist), ctypes.c_void_p(d_nout), ctypes.c_void_p(stream)))

    def SetCandidateClusters(self, n: int) -> None:
        """The default nprobe of Search (WithCandidateClusters on a live index)."""
        self._check(self._L.hann_pqivf_set_candidate_clusters(self._h, int(n)))

    def TuneCandidateClusters(self, queries, k: int, target_recall: float, ladder=None, mode: int = 1,
                              ground_truth=None, apply: bool = True):
        """The smallest nprobe of `ladder` whose recall@k on `queries` reaches
        `target_recall` against exact k-NN over the stored vectors (computed on
        the GPU by the batched exact k-NN unless ground_truth ids are given),
        through hann_pqivf_tune_candidate_clusters. Returns (nprobe, {nprobe:
        recall}); with apply, the index's default nprobe becomes the chosen
        value. When no value reaches the target the largest tried is chosen."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self._dim)
        nq = q.shape[0]
        k = int(k)
        lad = None if ladder is None else np.ascontiguousarray(ladder, dtype=np.int32)
        cap = HANN_TUNE_LADDER_MAX if lad is None else max(1, lad.size)
        gt = None
        if ground_truth is not None:
            gt = np.full((nq, k), -1, dtype=np.int64)
            g = np.asarray(ground_truth, dtype=np.int64).reshape(nq, -1)
            gt[:, :min(k, g.shape[1])] = g[:, :k]
        chosen = ctypes.c_int32(0)
        ntried = ctypes.c_int32(0)
        tried = np.zeros(cap, dtype=np.int32)
        rec = np.zeros(cap, dtype=np.float64)
        self._check(self._L.hann_pqivf_tune_candidate_clusters(
            self._h, _ptr(q), nq, k, float(target_recall), _ptr(lad) if lad is not None else None,
            0 if lad is None else int(lad.size), int(mode), _ptr(gt) if gt is not None else None,
            1 if apply else 0, ctypes.byref(chosen), _ptr(tried), _ptr(rec), ctypes.byref(ntried)))
        return int(chosen.value), {int(tried[i]): float(rec[i]) for i in range(ntried.value)}

    def SetPlainFP32(self, on: bool) -> None:
        """Switch the FP32 SIMT-only mode (same results, no tensor cores)."""
        self._check(self._L.hann_pqivf_set_plain_fp32(self._h, 1 if on else 0))

    ADC_TABLES = {"fp32": 0, "fp16": 1, "fixed16": 2}

    def SetADCTables(self, kind: str) -> None:
        """Lookup tables of the list scan: "fixed16" (default), "fp16" or
        "fp32". Parity-mode results do not change; exact-rerank candidates
        can at the rerank depth."""
        if kind not in self.ADC_TABLES:
            raise ValueError(f"unknown lookup-table kind {kind!r}")
        self._check(self._L.hann_pqivf_set_adc_tables(self._h, self.ADC_TABLES[kind]))

    def TrainStats(self) -> dict:
        """Coarse k-means assignments that took the warm filter, and the rows
        they sent to the exact kernel, over the index's life."""
        out = np.zeros(2, dtype=np.int64)
        self._check(self._L.hann_pqivf_train_stats(self._h, _ptr(out)))
        return {"warm_assignments": int(out[0]), "warm_overflow_rows": int(out[1])}

    def TrainPhases(self) -> dict:
        """Wall milliseconds of the last Train or Retrain by phase: staging the
        vectors, coarse k-means, subquantizer k-means, lists and layout."""
        out = np.zeros(4, dtype=np.float64)
        self._check(self._L.hann_pqivf_train_phases(self._h, _ptr(out)))
        return dict(zip(("stage_ms", "coarse_ms", "pq_ms", "layout_ms"), (round(float(v), 2) for v in out)))

    def ADCRedos(self) -> int:
        """Parity-mode queries the 16-bit screen could not prove, scanned again
        with FP32 tables, over the index's life."""
        out = np.zeros(1, dtype=np.int64)
        self._check(self._L.hann_pqivf_adc_redos(self._h, _ptr(out)))
        return int(out[0])

    def SetProfiling(self, on: bool) -> None:
        self._check(self._L.hann_pqivf_set_profiling(self._h, 1 if on else 0))

    def StageTimes(self):
        """Device ms of [coarse distances, probe select, scan, rerank], the
        launch count and the rows scanned since the last call (profiling on)."""
        ms = np.zeros(4, dtype=np.float64)
        n = ctypes.c_int64(0)
        rows = ctypes.c_int64(0)
        self._check(self._L.hann_pqivf_stage_times(self._h, _ptr(ms), ctypes.byref(n), ctypes.byref(rows)))
        return ms, int(n.value), int(rows.value)

    def ListLengths(self) -> np.ndarray:
        n = ctypes.c_int32(self.DeviceStats()["nlist"])
        for _ in range(100):
            out = np.zeros(max(n.value, 1), dtype=np.int64)
            rc = self._L.hann_pqivf_list_lengths(self._h, _ptr(out), out.size, ctypes.byref(n))
            if rc != HANN_E_CHANGED:  # else a Train changed the list count: size again
                break
        self._check(rc)
        return out[:n.value]

    def Stats(self) -> IndexStats:
        s = self._stats_raw()
        return IndexStats(int(s.count), int(s.dimension), "euclidean", int(s.fallback_searches))

    def DeviceStats(self) -> dict:
        s = self._stats_raw()
        return {"trained": bool(s.trained), "nlist": int(s.nlist), "rows_capacity": int(s.rows_capacity)}

    # -- persistence ---------------------------------------------------------
    def export_state(self) -> dict:
        """The index state as arrays (the GobEncode payload, pqivf/index.go:992-1017),
        one consistent state even while other threads mutate the index."""
        for _ in range(10_000):
            lay = _Layout()
            self._check(self._L.hann_pqivf_export_layout(self._h, ctypes.byref(lay)))
            dim, M = lay.dimension, lay.num_subquantizers
            nl, kq, nr, npd = lay.nlist, lay.pq_k_eff, lay.n_rows, lay.n_pending
            coarse = np.empty((nl, dim), np.float32)
            cbs = np.empty((M, kq, dim // M), np.float32)
            llen = np.empty(nl, np.int64)
            lkey = np.empty(nl, np.uint8)
            counts = np.empty(nl, np.int64)
            ids = np.empty(nr, np.int64)
            vecs = np.empty((nr, dim), np.float32)
            codes = np.empty((nr, M), np.int32)
            pids = np.empty(npd, np.int64)
            pvecs = np.empty((npd, dim), np.float32)
            rc = self._L.hann_pqivf_export(self._h, ctypes.byref(lay), _ptr(coarse), _ptr(cbs), _ptr(llen),
                                           _ptr(lkey), _ptr(counts), _ptr(ids), _ptr(vecs), _ptr(codes), _ptr(pids),
                                           _ptr(pvecs))
            if rc != HANN_E_CHANGED:  # else a mutation resized the index after the layout was read
                break
        self._check(rc)
        return {"layout": {f: getattr(lay, f) for f, _ in _Layout._fields_}, "coarse": coarse, "codebooks": cbs,
                "list_len": llen, "list_key": lkey, "cluster_counts": counts, "ids": ids, "vectors": vecs,
                "codes": codes, "pending_ids": pids, "pending_vectors": pvecs}

    def import_state(self, st: dict) -> None:
        lay = _Layout(**{f: int(st["layout"][f]) for f, _ in _Layout._fields_})
        has = st.get("has_codes")
        arrs = [np.ascontiguousarray(st["coarse"], np.float32), np.ascontiguousarray(st["codebooks"], np.float32),
                np.ascontiguousarray(st["list_len"], np.int64), np.ascontiguousarray(st["list_key"], np.uint8),
                np.ascontiguousarray(st["cluster_counts"], np.int64), np.ascontiguousarray(st["ids"], np.int64),
                np.ascontiguousarray(st["vectors"], np.float32), np.ascontiguousarray(st["codes"], np.int32),
                None if has is None else np.ascontiguousarray(has, np.uint8),
                np.ascontiguousarray(st["pending_ids"], np.int64),
                np.ascontiguousarray(st["pending_vectors"], np.float32)]
        ptrs = [(_ptr(a) if a is not None else None) for a in arrs]
        self._check(self._L.hann_pqivf_import(self._h, ctypes.byref(lay), *ptrs))
        self._dim = lay.dimension

    def Save(self, w) -> None:
        """Write the reference's gob format (pqivf/index.go:1086-1093)."""
        w.write(memoryview(gob_encode_state(self.export_state())))

    def GobEncode(self) -> bytes:
        """The serializedPQIVF gob stream (pqivf/index.go:992-1017)."""
        return gob_encode_state(self.export_state(), wrapped=False).tobytes()

    def GobDecode(self, data) -> None:
        """Replace the index with a gob stream's content, GobDecode's checks
        and defaults included (pqivf/index.go:1020-1084). Either GobEncode's
        bytes or Save's stream."""
        self.import_state(gob_decode_state(data, self._opts.candidate_clusters))

    def Load(self, r) -> None:
        """Read the reference's gob format (pqivf/index.go:1095-1101): the
        stream from the reader's position to its end. A file on disk is
        mapped rather than copied into memory."""
        mapped = _map_rest(r)
        if mapped is not None:
            mm, off = mapped
            try:
                st = gob_decode_state(memoryview(mm)[off:], self._opts.candidate_clusters)
                r.seek(0, os.SEEK_END)  # as read() would leave it
            finally:
                try:
                    mm.close()
                except BufferError:  # a traceback still holds a view: the map closes when that is freed
                    pass
        else:
            data = r.read() if hasattr(r, "read") else bytes(r)
            st = gob_decode_state(data, self._opts.candidate_clusters)
        self.import_state(st)

    def Retrain(self, iters: int) -> None:
        """Incremental re-Train: `iters` Lloyd iterations from the current
        centroids and codebooks, then every vector reassigned and re-encoded."""
        self._check(self._L.hann_pqivf_retrain(self._h, int(iters)))

    def ArenaStats(self) -> dict:
        """Row arena of the device layout (diagnostics)."""
        out = np.zeros(5, dtype=np.int64)
        self._check(self._L.hann_pqivf_arena_stats(self._h, _ptr(out)))
        return dict(zip(("rows_allocated", "rows_packed", "hole_rows", "list_moves", "full_relayouts"),
                        (int(v) for v in out)))

    TUNE_NPROBES = (8, 16, 32, 64, 128, 256)

    def AutotuneScan(self, queries, k: int = 10, mode: int = 1) -> dict:
        """Times the table scan and forms of the list-major scan on these
        queries at nprobe 8..256 and keeps the fastest routing (see
        hann_pqivf_autotune_scan). Returns the chosen options and the
        measured milliseconds per nprobe of both scans."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self._dim)
        chosen = np.zeros(8, dtype=np.int32)
        tab = np.zeros(6, dtype=np.float64)
        lm = np.zeros(6, dtype=np.float64)
        self._check(self._L.hann_pqivf_autotune_scan(self._h, _ptr(q), q.shape[0], int(k), int(mode), _ptr(chosen),
                                                     _ptr(tab), _ptr(lm)))
        return {"options": dict(zip(self.SCAN_OPTION_KEYS, (int(v) for v in chosen))),
                "ms_table_scan": {p: float(t) for p, t in zip(self.TUNE_NPROBES, tab) if t >= 0},
                "ms_list_major": {p: float(t) for p, t in zip(self.TUNE_NPROBES, lm) if t >= 0}}

    SCAN_OPTION_KEYS = ("list_major", "min_queries", "first_chunk", "chunk_growth", "rows_per_item", "ctas_per_sm",
                        "seed_threshold", "min_nprobe")

    def ScanOptions(self, **set_) -> dict:
        """The list scan's choices (diagnostics; results do not depend on
        them): list_major (the tensor-core list-major scan, else the table
        scan), min_queries, first_chunk, chunk_growth, rows_per_item,
        ctas_per_sm, seed_threshold, min_nprobe. Keyword arguments replace
        the named ones."""
        cur = np.zeros(8, dtype=np.int32)
        self._check(self._L.hann_pqivf_scan_options(self._h, None, _ptr(cur)))
        if set_:
            for key, val in set_.items():
                cur[self.SCAN_OPTION_KEYS.index(key)] = int(val)
            self._check(self._L.hann_pqivf_scan_options(self._h, _ptr(cur), None))
        return dict(zip(self.SCAN_OPTION_KEYS, (int(v) for v in cur)))

    def RowsDecoded(self) -> int:
        """Rows the list-major scan decoded while profiling was on, as of the
        last StageTimes call."""
        out = np.zeros(1, dtype=np.int64)
        self._check(self._L.hann_pqivf_rows_decoded(self._h, _ptr(out)))
        return int(out[0])

    def SaveSnapshot(self, path) -> None:
        """Write the binary snapshot (the gob stream's content as flat arrays;
        fast for large indexes)."""
        self._check(self._L.hann_pqivf_save_snapshot(self._h, os.fsencode(path)))

    def LoadSnapshot(self, path) -> None:
        """Replace the index with a binary snapshot (sizes and checksum are
        checked first; a bad file leaves the index as it was)."""
        self._check(self._L.hann_pqivf_load_snapshot(self._h, os.fsencode(path)))
        lay = _Layout()
        self._check(self._L.hann_pqivf_export_layout(self._h, ctypes.byref(lay)))
        self._dim = lay.dimension


# ---------------------------------------------------------------------------
# gob <-> array state. Save and Load use the native codec (csrc/gob.cu);
# state_to_gob and gob_to_state pair the arrays with the pure-Python codec
# in gob.py, which reads and writes the same bytes.


def _map_rest(r):
    """(read-only mmap of r's file, r's position) for a seekable file with
    bytes after its position; None for anything else."""
    import mmap

    try:
        fd, pos = r.fileno(), r.tell()
        size = os.fstat(fd).st_size
    except (AttributeError, OSError, ValueError, io.UnsupportedOperation):
        return None
    if pos >= size:
        return None
    try:
        return mmap.mmap(fd, 0, access=mmap.ACCESS_READ), pos
    except (OSError, ValueError):
        return None


def _gob_check(L, rc: int) -> None:
    if rc != HANN_OK:
        raise HannError(rc, L.hann_gob_last_error().decode())


def gob_encode_state(st: dict, wrapped: bool = True) -> np.ndarray:
    """The gob stream Save writes for export_state()'s arrays (GobEncode,
    pqivf/index.go:992-1017, inside Save's encoder), as uint8; with
    wrapped=False, GobEncode's bytes alone."""
    L = load_library()
    enc = L.hann_gob_encode if wrapped else L.hann_gob_encode_payload
    lay = _Layout(**{f: int(st["layout"][f]) for f, _ in _Layout._fields_})
    arrs = [np.ascontiguousarray(st["coarse"], np.float32), np.ascontiguousarray(st["codebooks"], np.float32),
            np.ascontiguousarray(st["list_len"], np.int64), np.ascontiguousarray(st["list_key"], np.uint8),
            np.ascontiguousarray(st["cluster_counts"], np.int64), np.ascontiguousarray(st["ids"], np.int64),
            np.ascontiguousarray(st["vectors"], np.float32), np.ascontiguousarray(st["codes"], np.int32),
            np.ascontiguousarray(st["pending_ids"], np.int64),
            np.ascontiguousarray(st["pending_vectors"], np.float32)]
    ptrs = [_ptr(a) for a in arrs]
    n = ctypes.c_int64(0)
    _gob_check(L, enc(ctypes.byref(lay), *ptrs, None, 0, ctypes.byref(n)))
    out = np.empty(n.value, np.uint8)
    _gob_check(L, enc(ctypes.byref(lay), *ptrs, _ptr(out), out.size, ctypes.byref(n)))
    return out


def gob_decode_state(data, default_candidate_clusters: int = 0) -> dict:
    """Parse a gob stream and apply GobDecode's checks and defaults
    (pqivf/index.go:1020-1084); the arrays import_state takes."""
    L = load_library()
    buf = np.frombuffer(data, np.uint8)
    h = _P()
    _gob_check(L, L.hann_gob_decode(_ptr(buf), buf.size, ctypes.byref(h)))
    try:
        lay = _Layout()
        _gob_check(L, L.hann_gob_state_layout(h, int(default_candidate_clusters), ctypes.byref(lay)))
        dim, M = lay.dimension, lay.num_subquantizers
        nl, kq, nr, npd = lay.nlist, lay.pq_k_eff, lay.n_rows, lay.n_pending
        st = {"layout": {f: getattr(lay, f) for f, _ in _Layout._fields_},
              "coarse": np.zeros((nl, dim), np.float32), "codebooks": np.zeros((M, kq, dim // M), np.float32),
              "list_len": np.zeros(nl, np.int64), "list_key": np.zeros(nl, np.uint8),
              "cluster_counts": np.zeros(nl, np.int64), "ids": np.zeros(nr, np.int64),
              "vectors": np.zeros((nr, dim), np.float32), "codes": np.zeros((nr, M), np.int32),
              "has_codes": np.zeros(nr, np.uint8), "pending_ids": np.zeros(npd, np.int64),
              "pending_vectors": np.zeros((npd, dim), np.float32)}
        keys = ("coarse", "codebooks", "list_len", "list_key", "cluster_counts", "ids", "vectors", "codes",
                "has_codes", "pending_ids", "pending_vectors")
        _gob_check(L, L.hann_gob_state_arrays(h, *[_ptr(st[k]) for k in keys]))
    finally:
        L.hann_gob_state_free(h)
    return st


def state_to_gob(st: dict) -> dict:
    lay = st["layout"]
    dim = lay["dimension"]
    lists, counts = {}, {}
    off = 0
    for c in range(lay["nlist"]):
        n = int(st["list_len"][c])
        if st["list_key"][c]:
            counts[c] = int(st["cluster_counts"][c])
            lists[c] = [{"ID": int(st["ids"][off + j]), "Vector": st["vectors"][off + j],
                         "Codes": [int(x) for x in st["codes"][off + j]], "Cluster": c} for j in range(n)]
        off += n
    return {
        "Dimension": dim, "CoarseK": lay["coarse_k"], "CoarseCentroids": list(st["coarse"]),
        "ClusterCounts": counts, "InvertedLists": lists, "NumSubquantizers": lay["num_subquantizers"],
        "Codebooks": [list(cb) for cb in st["codebooks"]] if lay["nlist"] else None, "PqK": lay["pq_k"],
        "KMeansIters": lay["kmeans_iters"], "AllowBruteForceFallback": bool(lay["fallback"]),
        "Trained": bool(lay["trained"]),
        "PendingVectors": {int(i): st["pending_vectors"][j] for j, i in enumerate(st["pending_ids"])},
        "NumCandidateClusters": lay["candidate_clusters"],
    }


def gob_to_state(ser: dict, opts: _Options | None = None) -> dict:
    """GobDecode (pqivf/index.go:1020-1084): validation and defaults."""
    fv = int(ser.get("FormatVersion", 0))
    if fv > gob.FORMAT_VERSION:
        raise HannError(HANN_E_INVALID, "index file has format version %d, but this build supports up to %d"
                        % (fv, gob.FORMAT_VERSION))
    dim = int(ser.get("Dimension", 0))
    M = int(ser.get("NumSubquantizers", 0))
    ck, pk, it = int(ser.get("CoarseK", 0)), int(ser.get("PqK", 0)), int(ser.get("KMeansIters", 0))
    if dim <= 0:
        raise HannError(HANN_E_INVALID, "serialized index has invalid dimension %d" % dim)
    if M <= 0 or dim % M != 0:
        raise HannError(HANN_E_INVALID, "serialized index has invalid subquantizer count %d for dimension %d"
                        % (M, dim))
    if ck <= 0 or pk <= 0 or it <= 0:
        raise HannError(HANN_E_INVALID, "serialized index has invalid training parameters: coarseK %d, pqK %d, "
                        "kMeansIters %d" % (ck, pk, it))
    ncc = int(ser.get("NumCandidateClusters", 0))
    if ncc <= 0:
        ncc = opts.candidate_clusters if opts is not None and opts.candidate_clusters > 0 else 3
    coarse = np.asarray(ser.get("CoarseCentroids") or [], dtype=np.float32).reshape(-1, dim)
    nl = coarse.shape[0]
    cbl = ser.get("Codebooks") or []
    kq = len(cbl[0]) if cbl else 0
    cbs = np.asarray(cbl, dtype=np.float32).reshape(M, kq, dim // M) if kq else np.zeros((M, 0, dim // M),
                                                                                            np.float32)
    lists = ser.get("InvertedLists") or {}
    counts_map = ser.get("ClusterCounts") or {}
    for c in list(lists) + list(counts_map):
        if c < 0 or c >= max(nl, 1) and lists.get(c):
            raise HannError(HANN_E_UNSUPPORTED, "inverted list %d has no coarse centroid" % c)
    llen = np.zeros(nl, np.int64)
    lkey = np.zeros(nl, np.uint8)
    counts = np.zeros(nl, np.int64)
    ids, vecs, codes, has = [], [], [], []
    for c in range(nl):
        if c in lists or c in counts_map:
            lkey[c] = 1
        counts[c] = int(counts_map.get(c, 0))
        ents = lists.get(c) or []
        llen[c] = len(ents)
        for e in ents:
            ids.append(int(e.get("ID", 0)))
            v = np.asarray(e.get("Vector") or [], dtype=np.float32)
            if v.size != dim:
                raise HannError(HANN_E_INVALID, "entry %d has a vector of dimension %d" % (ids[-1], v.size))
            vecs.append(v)
            cd = e.get("Codes") or []
            ok = len(cd) == M and all(0 <= int(x) < kq for x in cd)
            codes.append(np.asarray(cd if ok else [0] * M, dtype=np.int32))
            has.append(1 if ok else 0)
    pend = ser.get("PendingVectors") or {}
    pids = np.asarray(sorted(pend), dtype=np.int64)
    pvecs = np.asarray([pend[i] for i in sorted(pend)], dtype=np.float32).reshape(-1, dim)
    layout = {"dimension": dim, "coarse_k": ck, "num_subquantizers": M, "pq_k": pk, "kmeans_iters": it,
              "candidate_clusters": ncc, "fallback": 1 if ser.get("AllowBruteForceFallback") else 0,
              "trained": 1 if ser.get("Trained") else 0, "nlist": nl, "pq_k_eff": kq, "n_rows": len(ids),
              "n_pending": int(pids.size)}
    return {"layout": layout, "coarse": coarse, "codebooks": cbs, "list_len": llen, "list_key": lkey,
            "cluster_counts": counts, "ids": np.asarray(ids, np.int64),
            "vectors": np.asarray(vecs, np.float32).reshape(-1, dim),
            "codes": np.asarray(codes, np.int32).reshape(-1, M), "has_codes": np.asarray(has, np.uint8),
            "pending_ids": pids, "pending_vectors": pvecs}


def distance_batch(metric: int, query, flat) -> np.ndarray:
    """simd_<metric>_batch on the GPU (core/simd_kernels.inc.h:235-264)."""
    L = load_library()
    q = np.ascontiguousarray(query, dtype=np.float32).reshape(-1)
    x = np.ascontiguousarray(flat, dtype=np.float32).reshape(-1)
    dim = q.size
    n = x.size // dim if dim else 0
    out = np.zeros(n, dtype=np.float64)
    rc = L.hann_gpu_distance_batch(int(metric), _ptr(q), _ptr(x), dim, n, _ptr(out))
    if rc != HANN_OK:
        raise HannError(rc, "distance batch failed")
    return out


def distance_matrix(metric, queries, base) -> np.ndarray:
    """Every query against every base row, the values of distance_batch."""
    L = load_library()
    m = _metric_id(metric)
    x = np.ascontiguousarray(base, dtype=np.float32)
    dim = x.shape[1] if x.ndim == 2 else 0
    q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, dim) if dim else \
        np.zeros((len(queries), 0), np.float32)
    out = np.zeros((q.shape[0], x.shape[0]), dtype=np.float64)
    rc = L.hann_gpu_distance_matrix(m, _ptr(q), q.shape[0], _ptr(x), x.shape[0], dim, _ptr(out))
    if rc != HANN_OK:
        raise HannError(rc, "distance matrix failed")
    return out


# ---------------------------------------------------------------------------
# batched exact k-NN over a flat base (testutil.BruteForceKNN,
# internal/testutil/data.go:66-93, for many queries at once)

METRICS = {"squared_euclidean": 0, "euclidean": 1, "manhattan": 2, "cosine": 3}
KNN_METHODS = {"auto": 0, "exact": 1, "tensor": 2}


def _metric_id(metric) -> int:
    return METRICS[metric] if isinstance(metric, str) else int(metric)


class _KnnStats(ctypes.Structure):
    _fields_ = [("queries", ctypes.c_int64), ("exact_queries", ctypes.c_int64), ("tensor_queries", ctypes.c_int64),
                ("fallback_queries", ctypes.c_int64), ("chunks", ctypes.c_int64), ("redo_chunks", ctypes.c_int64)]


class KNN:
    """A flat base resident on the GPU, searched in batches. Results are
    ordered by (distance, row) with the reference's FP32 distances, so they
    equal testutil.BruteForceKNN over the same rows (ids = row numbers)."""

    def __init__(self, base):
        self._L = load_library()
        x = np.ascontiguousarray(base, dtype=np.float32)
        if x.ndim != 2:
            raise ValueError("base must be [n][dim]")
        self.n, self.dim = x.shape
        self._h = self._L.hann_knn_new(_ptr(x), self.n, self.dim)
        if not self._h:
            raise HannError(HANN_E_CUDA, "hann_knn_new failed")

    def close(self):
        if self._h:
            self._L.hann_knn_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != HANN_OK:
            raise HannError(rc, self._L.hann_knn_last_error(self._h).decode())

    def search(self, queries, k: int, metric="squared_euclidean", method="auto"):
        """(ids int64 [nq][k], dist float64 [nq][k]); slots past n hold -1 / +inf."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dim) if self.dim else \
            np.zeros((len(queries), 0), np.float32)
        nq = q.shape[0]
        ids = np.zeros((nq, k), dtype=np.int64)
        dist = np.zeros((nq, k), dtype=np.float64)
        self._check(self._L.hann_knn_search(self._h, _metric_id(metric), _ptr(q), nq, int(k),
                                            KNN_METHODS.get(method, method) if isinstance(method, str) else method,
                                            _ptr(ids), _ptr(dist)))
        return ids, dist

    def search_device(self, q_ptr: int, nq: int, k: int, ids_ptr: int, dist_ptr: int, metric="squared_euclidean",
                      method="auto", stream: int = 0):
        """Device buffers (raw pointers, e.g. torch tensor data_ptr())."""
        self._check(self._L.hann_knn_search_device(self._h, _metric_id(metric), ctypes.c_void_p(q_ptr), nq, int(k),
                                                   KNN_METHODS[method] if isinstance(method, str) else method,
                                                   ctypes.c_void_p(ids_ptr), ctypes.c_void_p(dist_ptr),
                                                   ctypes.c_void_p(stream)))

    def append(self, rows) -> None:
        """Add rows to the base (they get the next row numbers)."""
        x = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, self.dim)
        self._check(self._L.hann_knn_append(self._h, _ptr(x), x.shape[0]))
        self.n += x.shape[0]

    def distance_gather(self, queries, candidates, metric="squared_euclidean"):
        """Metric.RankBatch for many queries at once: candidates[q] is a
        sequence of row numbers; returns one float64 array of distances per
        query (the values distance_batch gives for those pairs)."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dim)
        lens = np.array([len(c) for c in candidates], dtype=np.int64)
        if len(lens) != q.shape[0]:
            raise ValueError("one candidate list per query")
        offsets = np.zeros(len(lens) + 1, dtype=np.int64)
        np.cumsum(lens, out=offsets[1:])
        ids = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.int64) for c in candidates])
                                   if len(candidates) else np.zeros(0, np.int64))
        if ids.size and (ids.min() < -2**31 or ids.max() >= 2**31):
            raise ValueError("candidate id out of range")
        ids32 = ids.astype(np.int32)
        out = np.zeros(int(offsets[-1]), dtype=np.float64)
        self._check(self._L.hann_knn_distance_gather(self._h, _metric_id(metric), _ptr(q), q.shape[0],
                                                     _ptr(offsets), _ptr(ids32), _ptr(out)))
        return [out[offsets[i]:offsets[i + 1]] for i in range(len(lens))]

    def stats(self) -> dict:
        st = _KnnStats()
        self._check(self._L.hann_knn_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _KnnStats._fields_}


def knn(queries, base, k: int, metric="squared_euclidean", method="auto"):
    """One-shot batched k-NN (copies base to the GPU, searches, frees)."""
    idx = KNN(base)
    try:
        return idx.search(queries, k, metric, method)
    finally:
        idx.close()


# ---------------------------------------------------------------------------
# continuous-batching server


class _ServeOptions(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int32), ("max_batch_queries", ctypes.c_int32), ("max_k", ctypes.c_int32),
                ("max_nprobe", ctypes.c_int32), ("mode", ctypes.c_int32), ("memory_budget", ctypes.c_int64),
                ("max_batch_probes", ctypes.c_int64)]


class _ServeStats(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_int64), ("queries", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("mutations", ctypes.c_int64), ("peak_admitted_bytes", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("queries_per_s", ctypes.c_double), ("relayouts", ctypes.c_int64),
                ("mutation_ms", ctypes.c_double), ("drain_ms", ctypes.c_double), ("relayout_ms", ctypes.c_double),
                ("relayout_max_ms", ctypes.c_double)]


def _serve_lib():
    L = load_library()
    if getattr(L, "_serve_ready", False):
        return L
    L.hann_serve_options_init.argtypes = [ctypes.POINTER(_ServeOptions)]
    L.hann_serve_options_init.restype = None
    L.hann_serve_start.argtypes = [_P, ctypes.POINTER(_ServeOptions), ctypes.POINTER(_P)]
    L.hann_serve_submit.argtypes = [_P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_uint64)]
    L.hann_serve_submit_priority.argtypes = [_P, _P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)]
    L.hann_serve_cancel.argtypes = [_P, ctypes.c_uint64]
    L.hann_serve_submit_add.argtypes = [_P, _P, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
    L.hann_serve_submit_delete.argtypes = [_P, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
    L.hann_serve_wait.argtypes = [_P, ctypes.c_uint64, _P, _P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
    L.hann_serve_stats.argtypes = [_P, ctypes.POINTER(_ServeStats)]
    L.hann_serve_last_error.argtypes = [_P]
    L.hann_serve_last_error.restype = ctypes.c_char_p
    L.hann_serve_stop.argtypes = [_P]
    L.hann_serve_replay.argtypes = [_P, _P, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.c_int64, _P, _P,
                                    ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.c_int64, _P, _P]
    L._serve_ready = True
    return L


class Server:
    """Continuous-batching server over an Index (hann_serve_* in the C ABI).

    submit() may be called from many threads; wait() returns the request's
    (ids [nq, k], distances [nq, k], counts [nq], latency_ms)."""

    def __init__(self, index: Index, slots=4, max_batch_queries=4096, max_k=100, max_nprobe=256,
                 mode=MODE_EXACT_RERANK, memory_budget=120 << 30, max_batch_probes=0):
        L = _serve_lib()
        o = _ServeOptions()
        L.hann_serve_options_init(ctypes.byref(o))
        o.slots, o.max_batch_queries, o.max_k, o.max_nprobe = slots, max_batch_queries, max_k, max_nprobe
        o.mode, o.memory_budget, o.max_batch_probes = mode, memory_budget, max_batch_probes
        h = _P()
        rc = L.hann_serve_start(index.handle, ctypes.byref(o), ctypes.byref(h))
        if rc != HANN_OK:
            raise HannError(rc, L.hann_pqivf_last_error(index.handle).decode())
        self._L, self._h, self._index, self._dim = L, h, index, index.dimension
        self._meta = {}
        self._meta_lock = threading.Lock()

    def _check(self, rc):
        if rc != HANN_OK:
            raise HannError(rc, self._L.hann_serve_last_error(self._h).decode())

    def submit(self, queries, k: int, nprobe: int = 0, priority: int = 0) -> int:
        """Queue a search; priority 1 goes ahead of every normal one still queued."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self._dim)
        t = ctypes.c_uint64(0)
        if priority:
            self._check(self._L.hann_serve_submit_priority(self._h, _ptr(q), q.shape[0], int(k), int(nprobe),
                                                           int(priority), ctypes.byref(t)))
        else:
            self._check(self._L.hann_serve_submit(self._h, _ptr(q), q.shape[0], int(k), int(nprobe),
                                                  ctypes.byref(t)))
        with self._meta_lock:
            self._meta[t.value] = (q.shape[0], int(k))
        return t.value

    def cancel(self, ticket: int) -> bool:
        """Withdraw a queued search: True if it had not started (its wait then
        raises), False if it already runs or finished."""
        rc = self._L.hann_serve_cancel(self._h, ctypes.c_uint64(ticket))
        if rc == HANN_OK:
            return True
        if rc == HANN_E_STATE:
            return False
        raise HannError(rc, "unknown ticket")

    def submit_add(self, ids, matrix) -> int:
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        m = np.ascontiguousarray(matrix, dtype=np.float32).reshape(-1, self._dim)
        t = ctypes.c_uint64(0)
        self._check(self._L.hann_serve_submit_add(self._h, _ptr(ids), _ptr(m), ids.size, ctypes.byref(t)))
        with self._meta_lock:
            self._meta[t.value] = (0, 0)
        return t.value

    def submit_delete(self, ids) -> int:
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        t = ctypes.c_uint64(0)
        self._check(self._L.hann_serve_submit_delete(self._h, _ptr(ids), ids.size, ctypes.byref(t)))
        with self._meta_lock:
            self._meta[t.value] = (0, 0)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000, results: bool = True):
        """Wait for a ticket: (ids, distances, counts, latency ms); with
        results=False only the latency (the results are dropped uncopied)."""
        with self._meta_lock:
            nq, k = self._meta.pop(ticket)
        lat = ctypes.c_double(0)
        if not results:
            self._check(self._L.hann_serve_wait(self._h, ticket, None, None, None, int(timeout_ms),
                                                ctypes.byref(lat)))
            return None, None, None, lat.value
        ids = np.zeros((nq, max(k, 1)), np.int64)
        dist = np.zeros((nq, max(k, 1)), np.float64)
        n = np.zeros(max(nq, 1), np.int32)
        self._check(self._L.hann_serve_wait(self._h, ticket, _ptr(ids), _ptr(dist), _ptr(n), int(timeout_ms),
                                            ctypes.byref(lat)))
        return ids, dist, n[:nq], lat.value

    # hann_serve_request (include/hann_gb300.h)
    REQUEST_DTYPE = np.dtype([("at_ms", "<f8"), ("kind", "<i4"), ("k", "<i4"), ("nprobe", "<i4"), ("pad", "<i4"),
                              ("first", "<i8"), ("count", "<i8"), ("out_offset", "<i8")])

    def replay(self, reqs, queries, query_rows, add_ids=None, add_vectors=None, del_ids=None, n_out_ids=0):
        """Drive the server from the native load generator
        (hann_serve_replay): reqs is an array of REQUEST_DTYPE sorted by
        at_ms. Returns (latency_ms, late_ms, out_ids) per request."""
        reqs = np.ascontiguousarray(reqs, dtype=self.REQUEST_DTYPE)
        q = np.ascontiguousarray(queries, dtype=np.float32)
        rows = np.ascontiguousarray(query_rows, dtype=np.int64)
        aid = np.ascontiguousarray(add_ids if add_ids is not None else np.zeros(0), dtype=np.int64)
        avec = np.ascontiguousarray(add_vectors if add_vectors is not None else np.zeros((0, q.shape[1])),
                                    dtype=np.float32)
        did = np.ascontiguousarray(del_ids if del_ids is not None else np.zeros(0), dtype=np.int64)
        if aid.size != avec.shape[0]:
            raise ValueError("add_ids and add_vectors must have the same rows")
        out = np.zeros(max(int(n_out_ids), 1), dtype=np.int64)
        lat = np.zeros(max(len(reqs), 1), dtype=np.float64)
        late = np.zeros(max(len(reqs), 1), dtype=np.float64)
        self._check(self._L.hann_serve_replay(self._h, reqs.ctypes.data, len(reqs), _ptr(q), q.shape[0], _ptr(rows),
                                              rows.size, _ptr(aid), _ptr(avec), aid.size, _ptr(did), did.size,
                                              _ptr(out), int(n_out_ids), _ptr(lat), _ptr(late)))
        return lat[:len(reqs)], late[:len(reqs)], out[:int(n_out_ids)]

    def stats(self) -> dict:
        s = _ServeStats()
        self._check(self._L.hann_serve_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in _ServeStats._fields_}

    def stop(self):
        if self._h:
            self._L.hann_serve_stop(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()
