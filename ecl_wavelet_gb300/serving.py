"""Python binding of the serving engine (ewt_server_* in include/ewt.h) and
of its CUDA-free scheduling core (include/ewt_sched.h, libewt_sched.so).

The engine itself is native: a dispatcher, a completer and a builder thread
inside libewt.so; this module only marshals buffers and keeps them alive
until their requests complete."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import EwtError, WaveletTree, _check, _ptr, lib

_PKG = os.path.dirname(os.path.abspath(__file__))
SCHED_LIB_PATH = os.path.join(_PKG, "libewt_sched.so")


class ServerConfig(C.Structure):
    _fields_ = [("batch_queries", C.c_uint64), ("batch_requests", C.c_uint32),
                ("inflight", C.c_uint32), ("memory_budget", C.c_uint64),
                ("elem_size", C.c_uint32), ("force_staging", C.c_uint32)]


class SchedStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64),
                ("cancelled", C.c_uint64), ("failed", C.c_uint64),
                ("batches", C.c_uint64), ("batched_requests", C.c_uint64),
                ("queries", C.c_uint64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("mean_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LoadConfig(C.Structure):
    _fields_ = [("rate", C.c_double), ("duration_s", C.c_double),
                ("max_request", C.c_uint32), ("first_tree", C.c_uint32),
                ("num_trees", C.c_uint32), ("frac_access", C.c_double),
                ("frac_rank", C.c_double), ("seed", C.c_uint64),
                ("plain", C.c_int), ("build_n", C.c_uint64),
                ("build_interval_s", C.c_double)]


class LoadResult(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("queries", C.c_uint64),
                ("wall_s", C.c_double), ("qps", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("batches", C.c_uint64), ("builds", C.c_uint64),
                ("build_p50_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SIGNATURES_SERVER = _SIGS = {
    "ewt_server_create": (C.c_int, [C.c_int, C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "ewt_server_destroy": (C.c_int, [C.c_void_p]),
    "ewt_server_add_tree": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]),
    "ewt_server_remove_tree": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ewt_server_submit": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                    C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64)]),
    "ewt_server_submit_build": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                          C.c_uint64, C.POINTER(C.c_uint64)]),
    "ewt_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_int),
                                  C.POINTER(C.c_double), C.POINTER(C.c_uint32)]),
    "ewt_server_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ewt_server_stats": (C.c_int, [C.c_void_p, C.POINTER(SchedStats), C.c_int]),
    "ewt_server_run_load": (C.c_int, [C.c_void_p, C.POINTER(LoadConfig),
                                      C.POINTER(LoadResult)]),
}

_bound = False


def _lib():
    global _bound
    L = lib()
    if not _bound:
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _bound = True
    return L


class Server:
    """Resident trees + continuous batching of mixed query requests."""

    def __init__(self, batch_queries=1 << 20, batch_requests=4096, inflight=2,
                 memory_budget=200 << 30, elem_size=1, gpu_index=0,
                 force_staging=False):
        L = _lib()
        cfg = ServerConfig(batch_queries, batch_requests, inflight, memory_budget,
                           elem_size, 1 if force_staging else 0)
        self._h = C.c_void_p()
        _check(L.ewt_server_create(gpu_index, C.byref(cfg), C.byref(self._h)),
               "Server")
        self._keep = {}  # request id -> buffers that must outlive it
        self.elem_size = elem_size

    def add_tree(self, tree: WaveletTree) -> int:
        tid = C.c_uint32()
        _check(_lib().ewt_server_add_tree(self._h, tree.handle, C.byref(tid)),
               "add_tree")
        return tid.value

    def remove_tree(self, tree_id: int):
        _check(_lib().ewt_server_remove_tree(self._h, tree_id), "remove_tree")

    def submit(self, tree_id: int, types, queries):
        """Queues a request; returns (request id, results array filled on
        completion)."""
        types = np.ascontiguousarray(types, dtype=np.uint8)
        queries = np.ascontiguousarray(queries)
        out = np.empty(types.size, dtype=np.uint64)
        rid = C.c_uint64()
        _check(_lib().ewt_server_submit(self._h, tree_id, _ptr(types), _ptr(queries),
                                        types.size, _ptr(out), C.byref(rid)),
               "submit")
        self._keep[rid.value] = (types, queries, out)
        return rid.value, out

    def submit_build(self, text, alphabet=None) -> int:
        text = np.ascontiguousarray(text)
        a = None if alphabet is None else np.ascontiguousarray(alphabet, dtype=text.dtype)
        rid = C.c_uint64()
        _check(_lib().ewt_server_submit_build(
            self._h, _ptr(text), text.size, None if a is None else _ptr(a),
            0 if a is None else a.size, C.byref(rid)), "submit_build")
        self._keep[rid.value] = (text, a)
        return rid.value

    def wait(self, request_id: int):
        """Returns (status, latency ms, built tree id)."""
        st, ms, tid = C.c_int(), C.c_double(), C.c_uint32()
        _check(_lib().ewt_server_wait(self._h, request_id, C.byref(st), C.byref(ms),
                                      C.byref(tid)), "wait")
        self._keep.pop(request_id, None)
        return st.value, ms.value, tid.value

    def cancel(self, request_id: int) -> bool:
        return _lib().ewt_server_cancel(self._h, request_id) == 0

    def stats(self, reset=False) -> dict:
        s = SchedStats()
        _check(_lib().ewt_server_stats(self._h, C.byref(s), 1 if reset else 0), "stats")
        return s.as_dict()

    def run_load(self, rate, duration_s, max_request=1 << 16, first_tree=0,
                 num_trees=1, frac_access=0.4, frac_rank=0.4, seed=1, plain=False,
                 build_n=0, build_interval_s=0.0) -> dict:
        cfg = LoadConfig(rate, duration_s, max_request, first_tree, num_trees,
                         frac_access, frac_rank, seed, 1 if plain else 0, build_n,
                         build_interval_s)
        res = LoadResult()
        _check(_lib().ewt_server_run_load(self._h, C.byref(cfg), C.byref(res)),
               "run_load")
        return res.as_dict()

    def close(self):
        if self._h.value:
            _check(_lib().ewt_server_destroy(self._h), "close")
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SIGNATURES_SCHED = {
    "ewt_sched_create": (C.c_void_p, [C.c_uint64, C.c_uint32, C.c_uint64]),
    "ewt_sched_destroy": (None, [C.c_void_p]),
    "ewt_sched_submit_query": (C.c_uint64, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_double]),
    "ewt_sched_submit_build": (C.c_uint64, [C.c_void_p, C.c_uint64, C.c_double]),
    "ewt_sched_cancel": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double]),
    "ewt_sched_take_batch": (C.c_uint32, [C.c_void_p, C.c_double, C.c_void_p, C.c_uint32]),
    "ewt_sched_take_build": (C.c_uint64, [C.c_void_p, C.c_double]),
    "ewt_sched_reserve": (None, [C.c_void_p, C.c_uint64]),
    "ewt_sched_release": (None, [C.c_void_p, C.c_uint64]),
    "ewt_sched_used": (C.c_uint64, [C.c_void_p]),
    "ewt_sched_complete": (None, [C.c_void_p, C.c_uint64, C.c_int, C.c_double]),
    "ewt_sched_state": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ewt_sched_get_stats": (None, [C.c_void_p, C.POINTER(SchedStats)]),
}


class Sched:
    """The scheduling core alone (libewt_sched.so, no CUDA needed)."""

    _L = None

    @classmethod
    def lib(cls):
        if cls._L is None:
            if not os.path.exists(SCHED_LIB_PATH):
                raise RuntimeError("libewt_sched.so is not built (run "
                                   "ecl_wavelet_gb300.buildlib.build_sched())")
            L = C.CDLL(SCHED_LIB_PATH)
            sigs = SIGNATURES_SCHED
            for name, (res, args) in sigs.items():
                f = getattr(L, name)
                f.restype, f.argtypes = res, args
            cls._L = L
        return cls._L

    def __init__(self, batch_queries, batch_requests, budget):
        self._h = self.lib().ewt_sched_create(batch_queries, batch_requests, budget)
        if not self._h:
            raise ValueError("invalid scheduler capacities")

    def submit_query(self, tree, m, now):
        return self.lib().ewt_sched_submit_query(self._h, tree, m, now)

    def submit_build(self, footprint, now):
        return self.lib().ewt_sched_submit_build(self._h, footprint, now)

    def cancel(self, rid, now):
        return bool(self.lib().ewt_sched_cancel(self._h, rid, now))

    def take_batch(self, now, cap=1 << 16):
        ids = np.zeros(cap, np.uint64)
        n = self.lib().ewt_sched_take_batch(self._h, now, _ptr(ids), cap)
        return [int(x) for x in ids[:min(n, cap)]]

    def take_build(self, now):
        return int(self.lib().ewt_sched_take_build(self._h, now))

    def reserve(self, b):
        self.lib().ewt_sched_reserve(self._h, b)

    def release(self, b):
        self.lib().ewt_sched_release(self._h, b)

    def used(self):
        return int(self.lib().ewt_sched_used(self._h))

    def complete(self, rid, status, now):
        self.lib().ewt_sched_complete(self._h, rid, status, now)

    def state(self, rid):
        return int(self.lib().ewt_sched_state(self._h, rid))

    def stats(self):
        s = SchedStats()
        self.lib().ewt_sched_get_stats(self._h, C.byref(s))
        return s.as_dict()

    def close(self):
        if self._h:
            self.lib().ewt_sched_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
