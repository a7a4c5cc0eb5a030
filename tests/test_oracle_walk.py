"""The oracle's structure walk agrees with the plain-scan definition.

Covers every symbol width, minimal and non-minimal alphabets, power-of-two
and shortened-code alphabets, alphabet detection, the edge cases the
reference handles (select past the last occurrence, rank at n, zero-count
symbols) and the invalid-query reports.
"""
import numpy as np
import pytest

from tests.workloads import random_text, random_queries


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
@pytest.mark.parametrize("sigma", [2, 3, 4, 5, 7, 10, 63, 64, 100, 255, 256])
def test_walk_matches_scan(oracle, dtype, sigma):
    if sigma > np.iinfo(dtype).max + 1:
        pytest.skip("alphabet wider than the symbol type")
    rng = np.random.default_rng(sigma * 31 + np.dtype(dtype).itemsize)
    for n in (1, 37, 4097, 70001):
        text, alphabet = random_text(rng, n, sigma, dtype,
                                     minimal=bool(sigma % 2))
        t = oracle.OracleTree(text, alphabet)
        idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, 3000)
        assert (t.access(idx) == t.scan_access(idx)).all()
        a, st1 = t.rank(rk, rs)
        b, st2 = t.scan_rank(rk, rs)
        assert st1 == st2 == 0 and (a == b).all()
        a, st1 = t.select(sk, ss)
        b, st2 = t.scan_select(sk, ss)
        assert st1 == st2 == 0 and (a == b).all()


def test_detected_alphabet(oracle):
    rng = np.random.default_rng(3)
    text = rng.choice(np.array([3, 9, 200, 201, 77], np.uint8), 5000)
    t = oracle.OracleTree(text)
    assert list(t.export("ALPHABET")) == [3, 9, 77, 200, 201]
    assert (t.access(np.arange(5000)) == text).all()


def test_invalid_queries_flagged(oracle):
    text = np.array([1, 2, 3, 1, 2, 3], np.uint16)
    t = oracle.OracleTree(text, [1, 2, 3])
    r, st = t.rank([7], [1])            # index > n
    assert st == -5 and int(r[0]) == 2**64 - 1
    r, st = t.rank([6], [9])            # symbol above the alphabet
    assert st == -5
    s, st = t.select([0], [1])          # k == 0
    assert st == -5
    r, st = t.rank([6, 3], [1, 0])      # rank at n; symbol 0 maps to 1
    assert st == 0 and list(r) == [2, 1]
    s, st = t.select([3], [3])          # past the last occurrence -> n
    assert st == 0 and int(s[0]) == 6


def test_mixed_matches_per_type(oracle):
    rng = np.random.default_rng(11)
    text, alphabet = random_text(rng, 20000, 37, np.uint16, minimal=False)
    t = oracle.OracleTree(text, alphabet)
    m = 5000
    types = rng.integers(0, 3, m).astype(np.uint8)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    got, st = t.mixed(types, index, sym)
    assert st == 0
    want = np.zeros(m, np.uint64)
    want[types == 0] = t.scan_access(index[types == 0])
    want[types == 1] = t.scan_rank(index[types == 1], sym[types == 1])[0]
    want[types == 2] = t.scan_select(index[types == 2], sym[types == 2])[0]
    assert (got == want).all()
