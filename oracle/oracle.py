"""Python handle on the CPU oracle (oracle/libewt_oracle.so) — test infrastructure.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; it is the checker, never the product.
The library restates mfranzreb/ECL_wavelet's levelwise wavelet tree and
RankSelect on the CPU (see ewt_oracle.cpp for the per-function citations).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_HERE, "libewt_oracle.so")

EXP = dict(COUNTS=1, LEVEL_WORDS=2, L1=3, L2=4, SAMPLES0=5, SAMPLES1=6,
           TOTAL_ONES=7, LEVEL_SIZES=8, NODE_RANKS=9, NODE_INFOS=10, CODES=11,
           NODES_AT_LEVEL=12, ALPHABET=13, NUM_LAST_L2=14)
EXP_DTYPE = {1: np.uint64, 2: np.uint32, 3: np.uint64, 4: np.uint16,
             5: np.uint64, 6: np.uint64, 7: np.uint64, 8: np.uint64,
             9: np.uint64, 10: np.uint64, 11: np.uint64, 12: np.uint64,
             13: np.uint64, 14: np.uint64}
PER_LEVEL = {2, 3, 4, 5, 6}


class Info(C.Structure):
    _fields_ = [("n", C.c_uint64), ("sigma", C.c_uint64),
                ("num_ranks", C.c_uint64), ("codes_start", C.c_uint64),
                ("num_codes", C.c_uint64),
                ("num_nodes_until_last_level", C.c_uint64),
                ("levels", C.c_uint32), ("elem_size", C.c_uint32),
                ("is_min_alphabet", C.c_uint32), ("is_pow2", C.c_uint32),
                ("device_bytes", C.c_uint64)]


def build_library(force: bool = False) -> str:
    """Compile ewt_oracle.cpp with g++ (seconds); returns the .so path."""
    src = os.path.join(_HERE, "ewt_oracle.cpp")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(
                os.path.getmtime(src),
                os.path.getmtime(os.path.join(_HERE, "ewt_oracle.h")),
                os.path.getmtime(os.path.join(_REPO, "include", "ewt.h")))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-shared",
                           "-fPIC", "-I", os.path.join(_REPO, "include"), src,
                           "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_library()
        L = C.CDLL(LIB_PATH)
        u64p = C.POINTER(C.c_uint64)
        L.ewto_build.argtypes = [C.c_void_p, C.c_uint64, C.c_int, u64p,
                                 C.c_uint64, C.POINTER(C.c_void_p)]
        L.ewto_free.argtypes = [C.c_void_p]
        L.ewto_build_mt.argtypes = [C.c_void_p, C.c_uint64, C.c_int, u64p,
                                    C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]
        L.ewto_scan_batch.argtypes = [C.c_void_p, C.c_uint64, C.c_int,
                                      C.c_uint64, C.POINTER(C.c_uint8), u64p,
                                      u64p, C.c_uint64, u64p, C.c_int]
        L.ewto_info.argtypes = [C.c_void_p, C.POINTER(Info)]
        L.ewto_export.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                  C.c_uint64, u64p]
        for f in ("ewto_access",):
            getattr(L, f).argtypes = [C.c_void_p, u64p, C.c_uint64, u64p,
                                      C.c_int]
        for f in ("ewto_rank", "ewto_select"):
            getattr(L, f).argtypes = [C.c_void_p, u64p, u64p, C.c_uint64,
                                      u64p, C.c_int]
        L.ewto_mixed.argtypes = [C.c_void_p, C.POINTER(C.c_uint8), u64p, u64p,
                                 C.c_uint64, u64p, C.c_int]
        L.ewto_scan_access.argtypes = [C.c_void_p, u64p, C.c_uint64, u64p]
        for f in ("ewto_scan_rank", "ewto_scan_select"):
            getattr(L, f).argtypes = [C.c_void_p, u64p, u64p, C.c_uint64, u64p]
        L.ewto_rs_build.argtypes = [C.POINTER(C.c_uint32), u64p, C.c_uint32,
                                    C.POINTER(C.c_void_p)]
        L.ewto_rs_free.argtypes = [C.c_void_p]
        L.ewto_rs_export.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                     C.c_uint64, u64p]
        L.ewto_rs_rank.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.c_int]
        L.ewto_rs_rank.restype = C.c_uint64
        L.ewto_rs_select.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.c_int]
        L.ewto_rs_select.restype = C.c_uint64
        for name in ("ewto_rs_rank_batch", "ewto_rs_select_batch"):
            f = getattr(L, name)
            f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_uint64, C.c_int,
                          C.c_void_p, C.c_int]
            f.restype = None
        L.ewto_minimal_codes.argtypes = [C.c_uint64, u64p, u64p, C.c_uint64,
                                         u64p]
        L.ewto_node_infos.argtypes = [C.c_uint64, u64p, u64p, C.c_uint64, u64p]
        L.ewto_node_pos.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32]
        L.ewto_node_pos.restype = C.c_uint64
        L.ewto_prev_pow2.argtypes = [C.c_uint64]
        L.ewto_prev_pow2.restype = C.c_uint64
        L.ewto_ceil_log2.argtypes = [C.c_uint64]
        L.ewto_ceil_log2.restype = C.c_uint32
        _lib = L
    return _lib


def _p(a, t=C.c_uint64):
    return a.ctypes.data_as(C.POINTER(t))


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


class OracleTree:
    """CPU restatement of ecl::WaveletTree<T> over a numpy text.

    threads=None: the plain restatement (keeps the text; the plain-scan
    answers work).  threads=k (0 = all cores): the multithreaded build of
    the same structure, which keeps no text (plain-scan answers of large
    texts come from scan_batch)."""

    def __init__(self, text: np.ndarray, alphabet=None, threads=None):
        text = np.ascontiguousarray(text)
        assert text.dtype in (np.uint8, np.uint16, np.uint32, np.uint64)
        self.text = text if threads is None else None
        h = C.c_void_p()
        if alphabet is None:
            a, s = None, 0
        else:
            self._alpha = _u64(alphabet)
            a, s = _p(self._alpha), len(self._alpha)
        if threads is None:
            st = lib().ewto_build(text.ctypes.data, text.size, text.itemsize,
                                  a, s, C.byref(h))
        else:
            st = lib().ewto_build_mt(text.ctypes.data, text.size,
                                     text.itemsize, a, s, threads, C.byref(h))
        if st != 0:
            raise ValueError("oracle build failed: status %d" % st)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().ewto_free(self.h)
            self.h = None

    def info(self) -> Info:
        i = Info()
        lib().ewto_info(self.h, C.byref(i))
        return i

    def export(self, comp: str, level: int = 0) -> np.ndarray:
        cid = EXP[comp]
        size = C.c_uint64()
        lib().ewto_export(self.h, cid, level, None, 0, C.byref(size))
        dt = EXP_DTYPE[cid]
        out = np.zeros(size.value // np.dtype(dt).itemsize, dtype=dt)
        st = lib().ewto_export(self.h, cid, level, out.ctypes.data, size.value,
                               C.byref(size))
        assert st == 0, st
        return out

    def access(self, idx, nthreads=0):
        idx = _u64(idx)
        out = np.zeros(idx.size, np.uint64)
        lib().ewto_access(self.h, _p(idx), idx.size, _p(out), nthreads)
        return out

    def rank(self, idx, sym, nthreads=0):
        idx, sym = _u64(idx), _u64(sym)
        out = np.zeros(idx.size, np.uint64)
        st = lib().ewto_rank(self.h, _p(idx), _p(sym), idx.size, _p(out),
                             nthreads)
        return out, st

    def select(self, k, sym, nthreads=0):
        k, sym = _u64(k), _u64(sym)
        out = np.zeros(k.size, np.uint64)
        st = lib().ewto_select(self.h, _p(k), _p(sym), k.size, _p(out),
                               nthreads)
        return out, st

    def mixed(self, types, idx, sym, nthreads=0):
        types = np.ascontiguousarray(types, dtype=np.uint8)
        idx, sym = _u64(idx), _u64(sym)
        out = np.zeros(idx.size, np.uint64)
        st = lib().ewto_mixed(self.h, _p(types, C.c_uint8), _p(idx), _p(sym),
                              idx.size, _p(out), nthreads)
        return out, st

    def scan_access(self, idx):
        idx = _u64(idx)
        out = np.zeros(idx.size, np.uint64)
        lib().ewto_scan_access(self.h, _p(idx), idx.size, _p(out))
        return out

    def scan_rank(self, idx, sym):
        idx, sym = _u64(idx), _u64(sym)
        out = np.zeros(idx.size, np.uint64)
        st = lib().ewto_scan_rank(self.h, _p(idx), _p(sym), idx.size, _p(out))
        return out, st

    def scan_select(self, k, sym):
        k, sym = _u64(k), _u64(sym)
        out = np.zeros(k.size, np.uint64)
        st = lib().ewto_scan_select(self.h, _p(k), _p(sym), k.size, _p(out))
        return out, st


def scan_batch(text, sigma, types, idx, sym, threads=0):
    """Plain-scan answers of a mixed batch over a 1- or 2-byte text whose
    alphabet is [0, sigma), in O(n + m log m) on all cores: (answers,
    status)."""
    text = np.ascontiguousarray(text)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    idx, sym = _u64(idx), _u64(sym)
    out = np.zeros(idx.size, np.uint64)
    st = lib().ewto_scan_batch(text.ctypes.data, text.size, text.itemsize,
                               sigma, _p(types, C.c_uint8), _p(idx), _p(sym),
                               idx.size, _p(out), threads)
    return out, st


class OracleRS:
    """CPU restatement of ecl::RankSelect over caller-given bit arrays."""

    def __init__(self, words_per_array, bits):
        bits = _u64(bits)
        words = np.concatenate([np.asarray(w, dtype=np.uint32)
                                for w in words_per_array]).astype(np.uint32)
        h = C.c_void_p()
        st = lib().ewto_rs_build(_p(words, C.c_uint32), _p(bits), bits.size,
                                 C.byref(h))
        if st != 0:
            raise ValueError("oracle rs build failed: %d" % st)
        self.h = h
        self.bits = bits

    def __del__(self):
        if getattr(self, "h", None):
            lib().ewto_rs_free(self.h)
            self.h = None

    def export(self, comp: str, array: int = 0) -> np.ndarray:
        cid = EXP[comp]
        size = C.c_uint64()
        lib().ewto_rs_export(self.h, cid, array, None, 0, C.byref(size))
        dt = EXP_DTYPE[cid]
        out = np.zeros(size.value // np.dtype(dt).itemsize, dtype=dt)
        lib().ewto_rs_export(self.h, cid, array, out.ctypes.data, size.value,
                             C.byref(size))
        return out

    def rank(self, array, pos, value):
        return lib().ewto_rs_rank(self.h, array, pos, value)

    def select(self, array, i, value):
        return lib().ewto_rs_select(self.h, array, i, value)

    def rank_batch(self, array, pos, value, nthreads=0):
        pos = _u64(pos)
        out = np.empty(pos.size, dtype=np.uint64)
        lib().ewto_rs_rank_batch(self.h, array, pos.ctypes.data, pos.size, value,
                                 out.ctypes.data, nthreads)
        return out

    def select_batch(self, array, idx, value, nthreads=0):
        idx = _u64(idx)
        out = np.empty(idx.size, dtype=np.uint64)
        lib().ewto_rs_select_batch(self.h, array, idx.ctypes.data, idx.size, value,
                                   out.ctypes.data, nthreads)
        return out


def minimal_codes(sigma: int):
    n = C.c_uint64()
    lib().ewto_minimal_codes(sigma, None, None, 0, C.byref(n))
    lens = np.zeros(max(n.value, 1), np.uint64)
    codes = np.zeros(max(n.value, 1), np.uint64)
    lib().ewto_minimal_codes(sigma, _p(lens), _p(codes), n.value, C.byref(n))
    return [(int(l), int(c)) for l, c in zip(lens[:n.value], codes[:n.value])]


def node_infos(sigma: int):
    n = C.c_uint64()
    lib().ewto_node_infos(sigma, None, None, 0, C.byref(n))
    s = np.zeros(max(n.value, 1), np.uint64)
    lv = np.zeros(max(n.value, 1), np.uint64)
    lib().ewto_node_infos(sigma, _p(s), _p(lv), n.value, C.byref(n))
    return [(int(a), int(b)) for a, b in zip(s[:n.value], lv[:n.value])]


def node_pos(sigma: int, symbol: int, level: int) -> int:
    return int(lib().ewto_node_pos(sigma, symbol, level))


def prev_pow2(n: int) -> int:
    return int(lib().ewto_prev_pow2(n))


def ceil_log2(n: int) -> int:
    return int(lib().ewto_ceil_log2(n))
