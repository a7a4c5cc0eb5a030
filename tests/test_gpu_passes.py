"""GPU parity of the multi-level build passes (power-of-two alphabets, 1- and
2-byte symbols) against the CPU oracle, on the shapes that stress their
bookkeeping: every level count L = 1..8 for uint8 and several for uint16,
text lengths at tile (4096) and chunk (65536) boundaries, tiny texts, texts
where most nodes are empty (one symbol, Zipf), and sorted / periodic texts
whose tiles sit inside one class at every level.  Integer results: every
exported structure byte-identical, every query equal to the plain scan.
"""
import numpy as np
import pytest

from tests.test_gpu_parity import assert_same_tree, check_queries

pytestmark = pytest.mark.gpu


def build_both(ewt, oracle, text, sigma):
    alphabet = np.arange(sigma)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    assert_same_tree(gt, ot)
    return gt, ot, alphabet.astype(np.uint64)


@pytest.mark.parametrize("L", range(1, 9))
def test_u8_every_level_count(ewt, oracle, L):
    sigma = 1 << L
    n = 2 * 65536 + 4097
    rng = np.random.default_rng(L)
    text = rng.integers(0, sigma, n, dtype=np.uint64).astype(np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 5_000, seed=L)


@pytest.mark.parametrize("n", [1, 2, 15, 16, 17, 4095, 4096, 4097, 65535,
                               65536, 65537, 3 * 65536 + 4096])
def test_u8_boundary_lengths(ewt, oracle, n):
    rng = np.random.default_rng(n)
    text = rng.integers(0, 256, n, dtype=np.uint64).astype(np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, 256)
    check_queries(gt, ot, text, al, 2_000, seed=n)


# Group query levels: octal superblocks hold 21,504 digits (512 blocks of
# 42), the routing pass works on 32,768-position superblocks, quad
# superblocks hold 49,152 digits.  Lengths at those boundaries, for trees of
# one octal group (sigma 8), octal + quad (32), two octal (64), and octal +
# two quad (128: 3 + 2 + 2).
@pytest.mark.parametrize("sigma", [8, 32, 64, 128])
@pytest.mark.parametrize("n", [41, 42, 43, 21_503, 21_504, 21_505, 32_768 + 1,
                               2 * 49_152 + 95, 5 * 21_504 + 7 * 42])
def test_group_level_boundaries(ewt, oracle, sigma, n):
    rng = np.random.default_rng(sigma * 1_000_003 + n)
    text = rng.integers(0, sigma, n, dtype=np.uint64).astype(np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 2_000, seed=n)


@pytest.mark.parametrize("sigma", [8, 64, 512])
def test_group_levels_sorted_runs(ewt, oracle, sigma):
    # every node boundary of every level falls inside some superblock
    n = 300_000
    rng = np.random.default_rng(sigma)
    text = np.sort(rng.integers(0, sigma, n, dtype=np.uint64))
    text = text.astype(np.uint16 if sigma > 256 else np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 5_000, seed=sigma)


@pytest.mark.parametrize("L", [1, 5, 9, 13, 16])
def test_u16_level_counts(ewt, oracle, L):
    sigma = 1 << L
    n = 200_003
    rng = np.random.default_rng(100 + L)
    text = rng.integers(0, sigma, n, dtype=np.uint64).astype(np.uint16)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 5_000, seed=L)


@pytest.mark.parametrize("dtype,sigma", [(np.uint8, 256), (np.uint16, 65536)])
def test_mostly_empty_nodes(ewt, oracle, dtype, sigma):
    """Zipf(2) over the alphabet: deep nodes are empty or a few symbols."""
    rng = np.random.default_rng(sigma)
    w = 1.0 / np.arange(1, sigma + 1) ** 2.0
    ids = rng.choice(sigma, 300_000, p=w / w.sum())
    perm = rng.permutation(sigma)  # spread the frequent symbols over nodes
    text = perm[ids].astype(dtype)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 5_000, seed=3)


def test_single_symbol_text(ewt, oracle):
    text = np.full(150_000, 200, np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, 256)
    check_queries(gt, ot, text, al, 2_000, seed=4)


@pytest.mark.parametrize("shape", ["sorted", "reversed", "periodic"])
def test_structured_texts(ewt, oracle, shape):
    n, sigma = 5 * 65536 + 123, 64
    rng = np.random.default_rng(7)
    base = rng.integers(0, sigma, n, dtype=np.uint64)
    if shape == "sorted":
        text = np.sort(base)
    elif shape == "reversed":
        text = np.sort(base)[::-1].copy()
    else:
        text = np.arange(n, dtype=np.uint64) % sigma
    text = text.astype(np.uint8)
    gt, ot, al = build_both(ewt, oracle, text, sigma)
    check_queries(gt, ot, text, al, 2_000, seed=5)


def test_pool_reuse_and_release(ewt, oracle):
    """Trees built after others were freed (their memory reused from the
    library pool) and after the pool was trimmed are still exact."""
    rng = np.random.default_rng(11)
    text = rng.integers(0, 256, 300_000, dtype=np.uint64).astype(np.uint8)
    ot = oracle.OracleTree(text, np.arange(256))
    for i in range(3):
        gt = ewt.WaveletTree(text, np.arange(256))
        assert_same_tree(gt, ot)
        gt.close()
        if i == 1:
            ewt.release_cached_memory(0)


@pytest.mark.parametrize("dtype,sigma,minimal", [(np.uint8, 256, True),
                                                 (np.uint16, 1000, False),
                                                 (np.uint64, 12, False)])
def test_save_load_round_trip(ewt, oracle, tmp_path, dtype, sigma, minimal):
    """An index written by save() and read back by load() exports the same
    structures and answers the same queries without a rebuild."""
    from tests.workloads import random_text
    rng = np.random.default_rng(sigma)
    text, alphabet = random_text(rng, 250_000, sigma, dtype, minimal=minimal)
    gt = ewt.WaveletTree(text, alphabet)
    path = str(tmp_path / "index.ewt")
    gt.save(path)
    lt = ewt.WaveletTree.load(path)
    ot = oracle.OracleTree(text, alphabet)
    assert_same_tree(lt, ot)
    al = np.asarray(alphabet, dtype=np.uint64)
    check_queries(lt, ot, text, al, 5_000, seed=4)
    lt.close()
    with open(path, "r+b") as f:  # a damaged file is refused, not loaded
        f.write(b"NOTANIDX")
    with pytest.raises(ewt.EwtError):
        ewt.WaveletTree.load(path)


@pytest.mark.parametrize("dtype,sigma", [(np.uint32, 40_000), (np.uint64, 300)])
def test_detected_wide_alphabet(ewt, oracle, dtype, sigma):
    """Alphabets of 4- and 8-byte texts detected on the GPU (hash set) equal
    the oracle's, including the extreme values 0 and the type's maximum."""
    rng = np.random.default_rng(sigma)
    info = np.iinfo(dtype)
    vals = np.unique(rng.integers(0, info.max, sigma * 2, dtype=np.uint64).astype(dtype))
    vals = vals[:sigma - 2]
    vals = np.unique(np.concatenate([vals, np.array([0, info.max], dtype=dtype)]))
    text = vals[rng.integers(0, vals.size, 400_000)]
    text[:vals.size] = vals  # every symbol present
    gt = ewt.WaveletTree(text)  # alphabet detected
    ot = oracle.OracleTree(text)
    assert np.array_equal(gt.getAlphabet(), np.sort(vals))
    assert_same_tree(gt, ot)
    check_queries(gt, ot, text, np.sort(vals).astype(np.uint64), 3_000, seed=6)


@pytest.mark.parametrize("dtype,sigma,minimal", [(np.uint8, 256, True),
                                                 (np.uint16, 3000, False),
                                                 (np.uint32, 77, False)])
def test_autotuned_queries_exact(ewt, oracle, dtype, sigma, minimal):
    """After ewt_autotune picked a launch shape per query kind, every kind
    still answers exactly as the plain scan (the shape changes speed only)."""
    from tests.workloads import random_text
    rng = np.random.default_rng(sigma + 1)
    text, alphabet = random_text(rng, 300_000, sigma, dtype, minimal=minimal)
    gt = ewt.WaveletTree(text, alphabet)
    tuning = gt.autotune(1 << 14)
    assert set(tuning) == {"access", "rank", "select", "mixed",
                           "select_sample_rate"}
    assert tuning["select_sample_rate"] in (0, 64, 128, 256, 512, 1024)
    for kind in ("access", "rank", "select", "mixed"):
        r = tuning[kind]
        assert r["threads"] in (128, 256), (kind, r)
        assert r["blocks_per_sm"] in (0, 2, 4, 6, 8), (kind, r)
        assert r["tuned_mq_s"] >= r["default_mq_s"] > 0, (kind, r)
    ot = oracle.OracleTree(text, alphabet)
    al = np.asarray(alphabet, dtype=np.uint64)
    check_queries(gt, ot, text, al, 20_000, seed=9)
    with pytest.raises(ewt.EwtError):
        gt.autotune(10)  # below the probe minimum


@pytest.mark.parametrize("rate", [0, 32, 64, 512, 65536])
def test_select_sample_rates_exact(ewt, oracle, rate):
    """Select through dense samples at every rate (and through the
    reference-format samples alone, rate 0) equals the plain scan, on a
    Zipf text whose deep levels hold long runs of one bit value (wide
    sample brackets, the binary-search path) next to dense ones."""
    from tests.workloads import random_text
    rng = np.random.default_rng(rate + 3)
    text, alphabet = random_text(rng, 400_000, 200, np.uint8, minimal=False,
                                 zipf=1.6)
    gt = ewt.WaveletTree(text, alphabet)
    gt.set_select_samples(rate)
    ot = oracle.OracleTree(text, alphabet)
    check_queries(gt, ot, text, np.asarray(alphabet, dtype=np.uint64), 20_000,
                  seed=rate)
    with pytest.raises(ewt.EwtError):
        gt.set_select_samples(48)  # not a power of two


@pytest.mark.parametrize("rate", [0, 32, 128, 4096])
def test_rs_select_sample_rates_exact(ewt, oracle, rate):
    """Standalone RankSelect: select0/select1 at every dense sample rate on
    iid, sparse (a few ones in a million bits), dense and empty arrays."""
    rng = np.random.default_rng(rate + 11)
    sizes = [1_000_003, 999_999, 777_777, 600_000, 4_095, 1]
    words = [rng.integers(0, 2**32, (s + 31) // 32, dtype=np.uint64).astype(np.uint32)
             for s in sizes]
    words[1][:] = 0
    words[1][rng.integers(0, words[1].size, 40)] = np.uint32(1 << 7)
    words[2] |= np.uint32(0xFFFFFFFE)
    words[3][:] = 0
    g = ewt.RankSelect(words, sizes)
    g.set_select_samples(rate)
    o = oracle.OracleRS(words, sizes)
    ones = g.export("TOTAL_ONES").astype(np.int64)
    for a, bits in enumerate(sizes):
        for v in (0, 1):
            tot = int(ones[a]) if v else bits - int(ones[a])
            ks = np.concatenate([rng.integers(1, tot + 1, 3000) if tot else
                                 np.array([], np.int64),
                                 np.array([1, max(tot, 1), tot + 1])])
            assert np.array_equal(g.select(a, v, ks),
                                  o.select_batch(a, ks, v)), (a, v)
