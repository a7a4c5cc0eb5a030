"""The multithreaded CPU build (the CPU baseline and the full-size checker of
the GPU build) against the plain restatement, and the O(n + m log m) batch
scan against the plain-scan answers.  CPU only."""
import numpy as np
import pytest

from tests.workloads import random_queries, random_text

PARTS = ("LEVEL_WORDS", "L1", "L2", "SAMPLES0", "SAMPLES1")
GLOBAL = ("COUNTS", "NODE_RANKS", "TOTAL_ONES", "LEVEL_SIZES", "NUM_LAST_L2",
          "NODE_INFOS", "CODES", "ALPHABET")


def same_structure(a, b, levels):
    for part in GLOBAL:
        assert np.array_equal(a.export(part), b.export(part)), part
    for l in range(levels):
        for part in PARTS:
            assert np.array_equal(a.export(part, l), b.export(part, l)), (part, l)


CASES = [
    # dtype, sigma, minimal, zipf, n
    (np.uint8, 4, True, None, 300_001),
    (np.uint8, 256, True, None, 3 * 65536 + 17),
    (np.uint8, 5, False, None, 200_000),
    (np.uint8, 200, True, 1.3, 500_000),
    (np.uint16, 1000, False, None, 250_000),
    (np.uint16, 1024, True, 1.1, 400_000),
    (np.uint16, 65536, True, None, 600_000),
    (np.uint32, 37, False, None, 100_000),
    (np.uint64, 300, False, 2.0, 100_000),
]


@pytest.mark.parametrize("dtype,sigma,minimal,zipf,n", CASES)
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_mt_build_matches_restatement(oracle, dtype, sigma, minimal, zipf, n,
                                      threads):
    rng = np.random.default_rng(sigma * 7 + threads)
    text, alphabet = random_text(rng, n, sigma, dtype, minimal=minimal,
                                 zipf=zipf)
    ref = oracle.OracleTree(text, alphabet)
    mt = oracle.OracleTree(text, alphabet, threads=threads)
    same_structure(ref, mt, ref.info().levels)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, 3000)
    assert np.array_equal(mt.access(idx), ref.scan_access(idx))
    assert np.array_equal(mt.rank(rk, rs)[0], ref.scan_rank(rk, rs)[0])
    assert np.array_equal(mt.select(sk, ss)[0], ref.scan_select(sk, ss)[0])


def test_mt_detects_alphabet(oracle):
    rng = np.random.default_rng(3)
    text, alphabet = random_text(rng, 100_000, 77, np.uint16, minimal=False)
    ref = oracle.OracleTree(text, alphabet)
    mt = oracle.OracleTree(text, None, threads=4)
    same_structure(ref, mt, ref.info().levels)


def test_mt_edge_texts(oracle):
    # a single node run, sorted and reversed texts, sizes at block edges
    for text in (np.repeat(np.arange(8, dtype=np.uint8), 65536),
                 np.arange(65536 * 2 + 5, dtype=np.uint64).astype(np.uint8)[::-1].copy(),
                 np.array([0, 1] * 4096, np.uint8),
                 np.array([1, 0], np.uint8)):
        ref = oracle.OracleTree(text, None)
        mt = oracle.OracleTree(text, None, threads=5)
        same_structure(ref, mt, ref.info().levels)


@pytest.mark.parametrize("dtype,sigma,zipf", [(np.uint8, 4, None),
                                              (np.uint8, 256, None),
                                              (np.uint16, 1024, 1.1),
                                              (np.uint16, 65536, None)])
def test_scan_batch_matches_plain_scan(oracle, dtype, sigma, zipf):
    rng = np.random.default_rng(sigma)
    text, alphabet = random_text(rng, 700_000, sigma, dtype, zipf=zipf)
    ref = oracle.OracleTree(text, alphabet)
    m = 20_000
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    index[:3] = [text.size, 0, text.size]  # rank at n, select past the end
    types[:3] = [1, 1, 2]
    got, st = oracle.scan_batch(text, sigma, types, index, sym, threads=6)
    assert st == 0
    want = np.zeros(m, np.uint64)
    a, r, s = types == 0, types == 1, types == 2
    want[a] = ref.scan_access(index[a])
    want[r] = ref.scan_rank(index[r], sym[r])[0]
    want[s] = ref.scan_select(index[s], sym[s])[0]
    assert np.array_equal(got, want)


def test_scan_batch_flags_invalid(oracle):
    text = np.array([0, 1, 2, 1], np.uint8)
    types = np.array([1, 2, 1, 0], np.uint8)
    got, st = oracle.scan_batch(text, 3, types, [5, 0, 1, 9], [1, 1, 7, 0])
    assert st == -5
    assert list(got) == [2**64 - 1, 2**64 - 1, 2**64 - 1, 0]
