"""ewt_mixed_noalloc — the mixed batch for callers that cannot allocate.

Serving loops whose own arena or caching allocator owns all free device
memory, hosts that fix each component's device budget in advance, and
latency paths that cannot take an allocation or cudaFree's device-wide
synchronisation use ewt_mixed_noalloc: it stages the batch in a fixed array
inside libewt.so instead of growing device scratch.  These tests call it
through the C ABI and check that it answers exactly as ewt_mixed does and as
the oracle's plain scan does (integer results, zero tolerance), on two calls
in a row (the array keeps the previous call's contents), that a call after
the first one leaves the device's free memory unchanged, and that batches
above its 262144-query limit are refused.  The file is named to run last.
"""
import numpy as np
import pytest

from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu

MAX_QUERIES = 1 << 18


def mixed_batch(tree, text, alphabet, m, seed):
    rng = np.random.default_rng(seed)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    return types, index, sym, tree.make_queries(index, sym)


def call(lib, fn, tree, types, q):
    out = np.full(q.size, 7, dtype=np.uint64)
    st = getattr(lib, fn)(tree.handle, types.ctypes.data, q.ctypes.data,
                          q.size, out.ctypes.data)
    return st, out


def scan_answers(ot, types, index, sym):
    """The oracle's plain-scan answers of a mixed batch."""
    want = np.zeros(types.size, np.uint64)
    a, r, s = types == 0, types == 1, types == 2
    want[a] = ot.scan_access(index[a])
    want[r] = ot.scan_rank(index[r], sym[r])[0]
    want[s] = ot.scan_select(index[s], sym[s])[0]
    return want


def free_device_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


@pytest.mark.parametrize("dtype,sigma,minimal", [(np.uint8, 256, True),
                                                 (np.uint16, 1000, False)])
def test_noalloc_matches_mixed_and_oracle_twice(ewt, oracle, dtype, sigma,
                                                minimal):
    lib = ewt.lib()
    rng = np.random.default_rng(sigma)
    text, alphabet = random_text(rng, 1_500_000, sigma, dtype, minimal=minimal)
    tree = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    # first calls on a fresh tree, before any ewt_mixed grew its scratch
    for seed, m in ((1, MAX_QUERIES), (2, 70_001)):
        types, index, sym, q = mixed_batch(tree, text, alphabet, m, seed)
        st, got = call(lib, "ewt_mixed_noalloc", tree, types, q)
        assert st == 0
        assert np.array_equal(got, scan_answers(ot, types, index, sym))
    for seed, m in ((3, MAX_QUERIES), (4, 70_001)):
        types, index, sym, q = mixed_batch(tree, text, alphabet, m, seed)
        st_ref, want = call(lib, "ewt_mixed", tree, types, q)
        st, got = call(lib, "ewt_mixed_noalloc", tree, types, q)
        assert st_ref == 0 and st == 0
        assert np.array_equal(got, want)
        assert np.array_equal(got, scan_answers(ot, types, index, sym))
    tree.close()


def test_noalloc_call_allocates_no_device_memory(ewt):
    lib = ewt.lib()
    rng = np.random.default_rng(5)
    text, alphabet = random_text(rng, 2_000_000, 64, np.uint8)
    tree = ewt.WaveletTree(text, alphabet)
    types, _, _, q = mixed_batch(tree, text, alphabet, MAX_QUERIES, 6)
    st, first = call(lib, "ewt_mixed_noalloc", tree, types, q)  # set-up call
    assert st == 0
    ewt.release_cached_memory(0)
    before = free_device_bytes()
    for _ in range(2):
        st, got = call(lib, "ewt_mixed_noalloc", tree, types, q)
        assert st == 0 and np.array_equal(got, first)
    assert free_device_bytes() == before
    tree.close()


def test_noalloc_reports_invalid_queries_and_limit(ewt):
    lib = ewt.lib()
    text = np.array([1, 2, 3, 1, 2, 3], np.uint16)
    tree = ewt.WaveletTree(text, [1, 2, 3])
    types = np.array([1, 2, 0], np.uint8)
    q = tree.make_queries([7, 0, 2], [1, 1, 0])  # index > n, k == 0
    st, got = call(lib, "ewt_mixed_noalloc", tree, types, q)
    st_ref, want = call(lib, "ewt_mixed", tree, types, q)
    assert st == st_ref == -5
    assert np.array_equal(got, want)
    # the invalid-query word starts clean on the next call
    types = np.array([1, 2], np.uint8)
    q = tree.make_queries([6, 2], [1, 3])
    st, got = call(lib, "ewt_mixed_noalloc", tree, types, q)
    assert st == 0 and list(got) == [2, 5]
    big = np.zeros(MAX_QUERIES + 1, np.uint8)
    qb = np.zeros(MAX_QUERIES + 1, dtype=tree.qdtype)
    st, _ = call(lib, "ewt_mixed_noalloc", tree, big, qb)
    assert st == -8
    assert b"262144" in lib.ewt_last_error()
