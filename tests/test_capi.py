"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point include/ewt.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("ewt.h", "ewt_sched.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(ewt_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("ewt_build", "ewt_access", "ewt_rank", "ewt_select",
                 "ewt_mixed", "ewt_export", "ewt_free", "ewt_rs_build"):
        assert must in names


def test_library_exports_every_declared_symbol(ewt):
    lib = ctypes.CDLL(ewt.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.ewt_abi_version() == 1


def test_python_binding_covers_header(ewt):
    from ecl_wavelet_gb300 import serving
    bound = (set(ewt.SIGNATURES) | set(serving.SIGNATURES_SERVER)
             | set(serving.SIGNATURES_SCHED))
    assert set(declared_functions()) <= bound


def test_library_builds_for_sm103a_only():
    from ecl_wavelet_gb300 import buildlib
    assert buildlib.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.gpu
def test_kernels_run_as_sm103a_code(ewt):
    v = ctypes.c_int(0)
    assert ewt.lib().ewt_binary_version(0, ctypes.byref(v)) == 0
    assert v.value == 103


def test_errors_without_gpu_are_statuses(ewt):
    import numpy as np
    lib = ewt.lib()
    h = ctypes.c_void_p()
    st = lib.ewt_build(None, 0, 1, None, 0, 0, ctypes.byref(h))
    assert st == -1  # invalid argument, checked before touching a device
    assert b"non-empty" in lib.ewt_last_error()
    assert lib.ewt_free(None) == 0
    st = lib.ewt_build(np.zeros(4, np.uint8).ctypes.data, 4, 3, None, 0, 0,
                       ctypes.byref(h))
    assert st == -1


def test_minimal_codes_entry_matches_oracle(ewt, oracle):
    """ewt_minimal_codes (what WaveletTree::createMinimalCodes returns) gives
    the codes of the oracle's restatement, which the known answers pin."""
    lib = ctypes.CDLL(ewt.LIB_PATH)
    import numpy as np
    for sigma in (3, 5, 10, 63, 72, 75, 255, 1000, 65535, 256):
        cnt = ctypes.c_uint64()
        assert lib.ewt_minimal_codes(ctypes.c_uint64(sigma), None, None,
                                     ctypes.c_uint64(0), ctypes.byref(cnt)) == 0
        lens = np.zeros(cnt.value, np.uint64)
        codes = np.zeros(cnt.value, np.uint64)
        assert lib.ewt_minimal_codes(ctypes.c_uint64(sigma),
                                     lens.ctypes.data_as(ctypes.c_void_p),
                                     codes.ctypes.data_as(ctypes.c_void_p),
                                     ctypes.c_uint64(cnt.value),
                                     ctypes.byref(cnt)) == 0
        got = [(int(l), int(c)) for l, c in zip(lens, codes)]
        assert got == oracle.minimal_codes(sigma), sigma


def test_needed_memory_entry(ewt):
    lib = ewt.lib()
    b = ctypes.c_uint64()
    assert lib.ewt_needed_memory(0, 1 << 20, 3, 0, ctypes.byref(b)) == 0
    ba = b.value
    assert ba >= 3 * (1 << 20) // 8
    assert lib.ewt_needed_memory(1, 1 << 20, 3, 0, ctypes.byref(b)) == 0
    assert b.value > ba
    assert lib.ewt_needed_memory(2, 1 << 30, 1, 256, ctypes.byref(b)) == 0
    assert b.value > (1 << 30)
    assert lib.ewt_needed_memory(2, 1 << 30, 3, 256, ctypes.byref(b)) == -1
    assert lib.ewt_needed_memory(7, 1, 1, 1, ctypes.byref(b)) == -1
