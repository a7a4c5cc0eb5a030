"""GB300 wavelet tree: Python binding of libewt.so over its C ABI (ewt.h).

Mirrors the reference's ``ecl::WaveletTree<T>`` host API
(include/ecl_wavelet/tree/wavelet_tree.cuh in mfranzreb/ECL_wavelet):
construction from a text and an optional alphabet, batched ``access``,
``rank`` and ``select``, and the getters.  Queries use the reference's
``RankSelectQuery<T>`` record (uint64 index + symbol, 16 bytes), exposed
here as the numpy dtype ``QUERY_DTYPE[T]``.

There is no CPU fallback: importing works anywhere, but every object that
touches the GPU loads libewt.so and raises if it is missing or unbuilt.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libewt.so")

EWT_OK = 0
STATUS = {0: "EWT_OK", -1: "EWT_ERR_INVALID_ARGUMENT",
          -2: "EWT_ERR_OUT_OF_MEMORY", -3: "EWT_ERR_CUDA",
          -4: "EWT_ERR_ALPHABET", -5: "EWT_ERR_QUERY",
          -6: "EWT_ERR_UNSUPPORTED", -7: "EWT_ERR_TIMEOUT",
          -8: "EWT_ERR_TOO_LARGE"}
Q_ACCESS, Q_RANK, Q_SELECT = 0, 1, 2

EXP = dict(COUNTS=1, LEVEL_WORDS=2, L1=3, L2=4, SAMPLES0=5, SAMPLES1=6,
           TOTAL_ONES=7, LEVEL_SIZES=8, NODE_RANKS=9, NODE_INFOS=10, CODES=11,
           NODES_AT_LEVEL=12, ALPHABET=13, NUM_LAST_L2=14)
EXP_DTYPE = {1: np.uint64, 2: np.uint32, 3: np.uint64, 4: np.uint16,
             5: np.uint64, 6: np.uint64, 7: np.uint64, 8: np.uint64,
             9: np.uint64, 10: np.uint64, 11: np.uint64, 12: np.uint64,
             13: np.uint64, 14: np.uint64}

SYMBOL_DTYPES = (np.uint8, np.uint16, np.uint32, np.uint64)


def query_dtype(sym_dtype) -> np.dtype:
    """numpy layout of ecl::RankSelectQuery<T>: {uint64 index_; T symbol_;}."""
    return np.dtype({"names": ["index", "symbol"],
                     "formats": [np.uint64, np.dtype(sym_dtype)],
                     "offsets": [0, 8], "itemsize": 16})


QUERY_DTYPE = {np.dtype(t): query_dtype(t) for t in SYMBOL_DTYPES}


class EwtError(RuntimeError):
    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        super().__init__("%s: %s (%d)%s" % (where, STATUS.get(status, "?"),
                                            status,
                                            ": " + message if message else ""))


class Info(C.Structure):
    _fields_ = [("n", C.c_uint64), ("sigma", C.c_uint64),
                ("num_ranks", C.c_uint64), ("codes_start", C.c_uint64),
                ("num_codes", C.c_uint64),
                ("num_nodes_until_last_level", C.c_uint64),
                ("levels", C.c_uint32), ("elem_size", C.c_uint32),
                ("is_min_alphabet", C.c_uint32), ("is_pow2", C.c_uint32),
                ("device_bytes", C.c_uint64)]


class Tuning(C.Structure):
    """Launch shapes chosen by ewt_autotune per query kind (access, rank,
    select, mixed) and the probe rates they gave."""
    _fields_ = [("threads", C.c_uint32 * 4), ("blocks_per_sm", C.c_uint32 * 4),
                ("select_sample_rate", C.c_uint32), ("reserved", C.c_uint32),
                ("default_mq_s", C.c_double * 4), ("tuned_mq_s", C.c_double * 4)]


# Every symbol libewt.so exports, with its ctypes signature.
_U64P = C.POINTER(C.c_uint64)
SIGNATURES = {
    "ewt_build": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p,
                            C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]),
    "ewt_build_u8": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                               C.c_uint32, C.POINTER(C.c_void_p)]),
    "ewt_build_u16": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                C.c_uint32, C.POINTER(C.c_void_p)]),
    "ewt_build_u32": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                C.c_uint32, C.POINTER(C.c_void_p)]),
    "ewt_build_u64": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                C.c_uint32, C.POINTER(C.c_void_p)]),
    "ewt_free": (C.c_int, [C.c_void_p]),
    "ewt_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "ewt_export": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                             C.c_uint64, _U64P]),
    "ewt_access": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ewt_rank": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ewt_select": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ewt_mixed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                            C.c_void_p]),
    "ewt_access_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64,
                                    C.c_void_p, C.c_void_p]),
    "ewt_rank_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64,
                                  C.c_void_p, C.c_void_p]),
    "ewt_select_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64,
                                    C.c_void_p, C.c_void_p]),
    "ewt_mixed_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_uint64, C.c_void_p, C.c_void_p]),
    "ewt_query_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ewt_mixed_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_uint64, C.c_void_p]),
    "ewt_get_device_view": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "ewt_rs_build": (C.c_int, [C.c_void_p, _U64P, C.c_uint32, C.c_int,
                               C.POINTER(C.c_void_p)]),
    "ewt_rs_free": (C.c_int, [C.c_void_p]),
    "ewt_rs_export": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                C.c_uint64, _U64P]),
    "ewt_rs_rank": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                              C.c_uint64, C.c_void_p]),
    "ewt_rs_select": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                C.c_uint64, C.c_void_p]),
    "ewt_rs_get_device_view": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "ewt_last_error": (C.c_char_p, []),
    "ewt_abi_version": (C.c_int, []),
    "ewt_bitarray_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int,
                                      C.c_int, C.POINTER(C.c_void_p)]),
    "ewt_rs_build_in_place": (C.c_int, [C.c_void_p]),
    "ewt_needed_memory": (C.c_int, [C.c_int, C.c_uint64, C.c_uint32,
                                    C.c_uint64, C.POINTER(C.c_uint64)]),
    "ewt_minimal_codes": (C.c_int, [C.c_uint64, C.c_void_p, C.c_void_p,
                                    C.c_uint64, C.POINTER(C.c_uint64)]),
    "ewt_set_work_queue": (None, [C.c_int]),
    "ewt_binary_version": (C.c_int, [C.c_int, C.POINTER(C.c_int)]),
    "ewt_release_cached_memory": (C.c_int, [C.c_int]),
    "ewt_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ewt_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "ewt_build_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                  C.c_void_p]),
    "ewt_mixed_multi": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_uint64,
                                  C.c_void_p]),
    "ewt_mixed_multi_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_uint64,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "ewt_autotune": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Tuning)]),
    "ewt_set_select_samples": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ewt_probe_random_reads": (C.c_int, [C.c_int, C.c_uint64, C.c_uint32,
                                         C.c_uint64, C.POINTER(C.c_double)]),
    "ewt_rs_set_select_samples": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ewt_launch_count": (C.c_uint64, []),
    "ewt_set_timing": (None, [C.c_int]),
    "ewt_get_timing": (None, [C.c_void_p, C.c_int]),
}

PHASES = ["hist", "fill", "rs_counts", "split", "node_ranks", "samples",
          "query", "h2d", "quad"]


class PhaseTimes(C.Structure):
    _fields_ = [("ms", C.c_double * len(PHASES)),
                ("launches", C.c_uint64 * len(PHASES))]


def set_timing(enable: bool):
    """Per-phase device timing with CUDA events on the launching streams."""
    lib().ewt_set_timing(1 if enable else 0)


def get_timing(reset: bool = True) -> dict:
    t = PhaseTimes()
    lib().ewt_get_timing(C.byref(t), 1 if reset else 0)
    return {p: (t.ms[i], int(t.launches[i])) for i, p in enumerate(PHASES)}

_lib = None


def build(verbose: bool = False) -> str:
    """Compiles libewt.so for sm_103a (see buildlib.py)."""
    from . import buildlib as _b
    return _b.build(verbose=verbose)


def lib():
    """Loads libewt.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libewt.so is not built (run ecl_wavelet_gb300.build() or "
                "__graft_entry__.build()); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st: int, where: str):
    if st != EWT_OK:
        msg = lib().ewt_last_error()
        raise EwtError(st, where, msg.decode() if msg else "")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def launch_count() -> int:
    return int(lib().ewt_launch_count())


def probe_random_reads(bytes_: int = 8 << 30, depth: int = 4,
                       chains: int = 1 << 25, gpu_index: int = 0) -> float:
    """Dependent random 32-byte reads per second (ewt_probe_random_reads):
    the random-access roofline of the query walks."""
    r = C.c_double()
    _check(lib().ewt_probe_random_reads(gpu_index, bytes_, depth, chains,
                                        C.byref(r)), "probe_random_reads")
    return r.value


def set_work_queue(enable: bool):
    """Device work queue (default) or fixed-stride chunks for batched
    query launches (ewt_set_work_queue)."""
    lib().ewt_set_work_queue(1 if enable else 0)


def release_cached_memory(gpu_index: int = 0):
    """Returns the library pool's unused device memory to the driver."""
    _check(lib().ewt_release_cached_memory(gpu_index), "release_cached_memory")


_ELEM_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def build_batch(texts, alphabets=None, gpu_index: int = 0):
    """Builds many texts concurrently (ewt_build_batch); returns one
    WaveletTree per text.  All texts share one symbol type; ``alphabets`` is
    None (detect every alphabet) or one sorted alphabet per text."""
    if all(hasattr(t, "data_ptr") for t in texts):  # torch tensors
        dt = np.dtype(str(texts[0].dtype).replace("torch.", ""))
        ptrs = [t.data_ptr() for t in texts]
        sizes = [t.numel() for t in texts]
    else:
        texts = [np.ascontiguousarray(t) for t in texts]
        dt = texts[0].dtype
        if any(t.dtype != dt for t in texts):
            raise TypeError("texts must share one symbol type")
        ptrs = [_ptr(t) for t in texts]
        sizes = [t.size for t in texts]
    if dt not in SYMBOL_DTYPES:
        raise TypeError("texts must hold unsigned 8/16/32/64-bit symbols")
    count = len(texts)
    tp = (C.c_void_p * count)(*ptrs)
    lens = np.array(sizes, dtype=np.uint64)
    ap = sp = None
    if alphabets is not None:
        al = [np.ascontiguousarray(a, dtype=dt) for a in alphabets]
        ap = (C.c_void_p * count)(*[_ptr(a) for a in al])
        sig = np.array([a.size for a in al], dtype=np.uint64)
        sp = _ptr(sig)
    out = (C.c_void_p * count)()
    st = np.zeros(count, dtype=np.int32)
    rc = lib().ewt_build_batch(tp, _ptr(lens), count, dt.itemsize, ap, sp,
                               gpu_index, out, _ptr(st))
    trees = [WaveletTree(None, _handle=h) if h else None for h in out]
    if rc != 0:
        for t in trees:
            if t is not None:
                t.close()
        _check(rc, "build_batch")
    return trees


def mixed_multi(trees, tree_of, types, queries) -> np.ndarray:
    """Mixed queries over several trees in one launch (ewt_mixed_multi):
    query i goes to trees[tree_of[i]]; records as WaveletTree.make_queries."""
    count = len(trees)
    hp = (C.c_void_p * count)(*[t._h.value for t in trees])
    tree_of = np.ascontiguousarray(tree_of, dtype=np.uint32)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    queries = np.ascontiguousarray(queries)
    out = np.empty(types.size, dtype=np.uint64)
    _check(lib().ewt_mixed_multi(hp, count, _ptr(tree_of), _ptr(types),
                                 _ptr(queries), types.size, _ptr(out)),
           "mixed_multi")
    return out


class WaveletTree:
    """ecl::WaveletTree<T> over a numpy text (uint8/16/32/64).

    ``alphabet`` — sorted distinct symbols, or None/empty to detect them.
    ``text`` may also be a torch CUDA tensor (built from device memory).
    """

    def __init__(self, text, alphabet=None, gpu_index: int = 0, _handle=None):
        L = lib()
        self._h = C.c_void_p()
        if _handle is not None:  # adopt a tree built by build_batch
            self._h = C.c_void_p(_handle)
            self._keep = None
            self.info = Info()
            _check(L.ewt_get_info(self._h, C.byref(self.info)), "get_info")
            self.dtype = np.dtype(_ELEM_DTYPE[int(self.info.elem_size)])
            self.qdtype = QUERY_DTYPE[self.dtype]
            return
        if hasattr(text, "data_ptr"):  # torch tensor (host or device)
            dt = np.dtype(str(text.dtype).replace("torch.", ""))
            ptr, n = text.data_ptr(), text.numel()
            self._keep = text
        else:
            text = np.ascontiguousarray(text)
            dt = text.dtype
            ptr, n = _ptr(text), text.size
            self._keep = text
        if dt not in SYMBOL_DTYPES:
            raise TypeError("text must hold unsigned 8/16/32/64-bit symbols")
        self.dtype = np.dtype(dt)
        if alphabet is None or len(alphabet) == 0:
            a_ptr, sigma = None, 0
        else:
            self._alpha = np.ascontiguousarray(alphabet, dtype=self.dtype)
            a_ptr, sigma = _ptr(self._alpha), self._alpha.size
        st = L.ewt_build(ptr, n, self.dtype.itemsize, a_ptr, sigma, gpu_index,
                         C.byref(self._h))
        if st == -2:
            raise EwtError(st, "WaveletTree",
                           "Not enough memory available for the wavelet tree.")
        _check(st, "WaveletTree")
        self._keep = None
        self.info = Info()
        _check(L.ewt_get_info(self._h, C.byref(self.info)), "get_info")
        self.qdtype = QUERY_DTYPE[self.dtype]

    def save(self, path: str):
        """Writes the index to `path` (ewt_save)."""
        _check(lib().ewt_save(self._h, os.fsencode(path)), "save")

    @classmethod
    def load(cls, path: str, gpu_index: int = 0) -> "WaveletTree":
        """Reads an index written by save() onto a GPU (ewt_load)."""
        h = C.c_void_p()
        _check(lib().ewt_load(os.fsencode(path), gpu_index, C.byref(h)), "load")
        return cls(None, _handle=h.value)

    def autotune(self, probe_queries: int = 1 << 22) -> dict:
        """Times the query kernels on `probe_queries` device-generated valid
        queries for candidate dense select-sample rates and, per kind, launch
        shapes, and keeps the fastest for every later query on this tree
        (ewt_autotune).  Returns, per kind, the chosen threads per CTA,
        resident CTAs per SM (0 = as many as fit) and the default and tuned
        rates in million queries/s, and under "select_sample_rate" the dense
        sample rate kept (0: reference-format samples only)."""
        tu = Tuning()
        _check(lib().ewt_autotune(self._h, probe_queries, C.byref(tu)), "autotune")
        res = {kind: {"threads": tu.threads[i],
                      "blocks_per_sm": tu.blocks_per_sm[i],
                      "default_mq_s": tu.default_mq_s[i],
                      "tuned_mq_s": tu.tuned_mq_s[i]}
               for i, kind in enumerate(("access", "rank", "select", "mixed"))}
        res["select_sample_rate"] = tu.select_sample_rate
        return res

    def set_select_samples(self, rate: int):
        """Dense select samples every `rate` zeros / ones (0: none; a power
        of two in [32, 65536]) (ewt_set_select_samples)."""
        _check(lib().ewt_set_select_samples(self._h, rate), "set_select_samples")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ewt_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- getters (wavelet_tree.cuh:2165-2282) ---------------------------
    def getAlphabetSize(self) -> int:
        return int(self.info.sigma)

    def getNumLevels(self) -> int:
        return int(self.info.levels)

    def isMinAlphabet(self) -> bool:
        return bool(self.info.is_min_alphabet)

    def getCodesStart(self) -> int:
        return int(self.info.codes_start)

    def getAlphabet(self) -> np.ndarray:
        return self.export("ALPHABET").astype(self.dtype)

    def getCounts(self, i: int) -> int:
        return int(self.export("COUNTS")[i])

    def getTotalAppearances(self, i: int) -> int:
        c = self.export("COUNTS")
        end = int(self.info.n) if i == len(c) - 1 else int(c[i + 1])
        return end - int(c[i])

    @property
    def handle(self) -> int:
        return self._h.value

    # ---- batch queries ---------------------------------------------------
    def make_queries(self, index, symbol) -> np.ndarray:
        q = np.zeros(len(index), dtype=self.qdtype)
        q["index"] = index
        q["symbol"] = symbol
        return q

    def access(self, indices) -> np.ndarray:
        idx = np.ascontiguousarray(indices, dtype=np.uint64)
        out = np.zeros(idx.size, dtype=self.dtype)
        _check(lib().ewt_access(self._h, _ptr(idx), idx.size, _ptr(out)),
               "access")
        return out

    def rank(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=self.qdtype)
        out = np.zeros(q.size, dtype=np.uint64)
        _check(lib().ewt_rank(self._h, _ptr(q), q.size, _ptr(out)), "rank")
        return out

    def select(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=self.qdtype)
        out = np.zeros(q.size, dtype=np.uint64)
        _check(lib().ewt_select(self._h, _ptr(q), q.size, _ptr(out)), "select")
        return out

    def mixed(self, types, queries) -> np.ndarray:
        t = np.ascontiguousarray(types, dtype=np.uint8)
        q = np.ascontiguousarray(queries, dtype=self.qdtype)
        out = np.zeros(q.size, dtype=np.uint64)
        _check(lib().ewt_mixed(self._h, _ptr(t), _ptr(q), q.size, _ptr(out)),
               "mixed")
        return out

    def try_rank(self, queries):
        """rank returning (results, status) instead of raising."""
        q = np.ascontiguousarray(queries, dtype=self.qdtype)
        out = np.zeros(q.size, dtype=np.uint64)
        st = lib().ewt_rank(self._h, _ptr(q), q.size, _ptr(out))
        return out, st

    def try_select(self, queries):
        q = np.ascontiguousarray(queries, dtype=self.qdtype)
        out = np.zeros(q.size, dtype=np.uint64)
        st = lib().ewt_select(self._h, _ptr(q), q.size, _ptr(out))
        return out, st

    # ---- device-resident batches (pointers from torch tensors) ----------
    def access_device(self, d_idx: int, m: int, d_out: int, stream: int = 0):
        _check(lib().ewt_access_device(self._h, d_idx, m, d_out, stream),
               "access_device")

    def rank_device(self, d_q: int, m: int, d_out: int, stream: int = 0):
        _check(lib().ewt_rank_device(self._h, d_q, m, d_out, stream),
               "rank_device")

    def select_device(self, d_q: int, m: int, d_out: int, stream: int = 0):
        _check(lib().ewt_select_device(self._h, d_q, m, d_out, stream),
               "select_device")

    def mixed_device(self, d_types: int, d_q: int, m: int, d_out: int,
                     stream: int = 0):
        _check(lib().ewt_mixed_device(self._h, d_types, d_q, m, d_out, stream),
               "mixed_device")

    def query_status(self, stream: int = 0) -> int:
        return lib().ewt_query_status(self._h, stream)

    # ---- exports ---------------------------------------------------------
    def export(self, comp: str, level: int = 0) -> np.ndarray:
        cid = EXP[comp]
        size = C.c_uint64()
        _check(lib().ewt_export(self._h, cid, level, None, 0, C.byref(size)),
               "export")
        dt = EXP_DTYPE[cid]
        out = np.zeros(size.value // np.dtype(dt).itemsize, dtype=dt)
        _check(lib().ewt_export(self._h, cid, level, _ptr(out), size.value,
                                C.byref(size)), "export")
        return out


class RankSelect:
    """ecl::RankSelect over caller-given bit arrays (BitArray + RankSelect)."""

    def __init__(self, words_per_array, bits, gpu_index: int = 0):
        bits = np.ascontiguousarray(bits, dtype=np.uint64)
        words = np.concatenate([np.asarray(w, dtype=np.uint32)
                                for w in words_per_array]).astype(np.uint32)
        self._h = C.c_void_p()
        _check(lib().ewt_rs_build(_ptr(words), bits.ctypes.data_as(_U64P),
                                  bits.size, gpu_index, C.byref(self._h)),
               "RankSelect")
        self.bits = bits

    def set_select_samples(self, rate: int):
        """As WaveletTree.set_select_samples (ewt_rs_set_select_samples)."""
        _check(lib().ewt_rs_set_select_samples(self._h, rate), "set_select_samples")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ewt_rs_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def export(self, comp: str, array: int = 0) -> np.ndarray:
        cid = EXP[comp]
        size = C.c_uint64()
        _check(lib().ewt_rs_export(self._h, cid, array, None, 0,
                                   C.byref(size)), "export")
        dt = EXP_DTYPE[cid]
        out = np.zeros(size.value // np.dtype(dt).itemsize, dtype=dt)
        _check(lib().ewt_rs_export(self._h, cid, array, _ptr(out), size.value,
                                   C.byref(size)), "export")
        return out

    def rank(self, array: int, value: int, pos, out=None) -> np.ndarray:
        """rank_value of every position; `out` (uint64, reused when given)
        receives the results."""
        p = np.ascontiguousarray(pos, dtype=np.uint64)
        if out is None:
            out = np.zeros(p.size, dtype=np.uint64)
        _check(lib().ewt_rs_rank(self._h, array, value, _ptr(p), p.size,
                                 _ptr(out)), "rs_rank")
        return out

    def select(self, array: int, value: int, i, out=None) -> np.ndarray:
        """select_value of every index (1-based); `out` as for rank()."""
        p = np.ascontiguousarray(i, dtype=np.uint64)
        if out is None:
            out = np.zeros(p.size, dtype=np.uint64)
        _check(lib().ewt_rs_select(self._h, array, value, _ptr(p), p.size,
                                   _ptr(out)), "rs_select")
        return out
