"""GPU parity: libewt.so (called through its C ABI) against the CPU oracle.

Every exported structure — level bit words, L1/L2 counts, select samples,
count table, node-start ranks, codes — must be byte-identical to the
oracle's restatement of the reference, and every query answer must equal
the plain-scan definition.  Integer work: the tolerance is zero.
"""
import json
import os

import numpy as np
import pytest

from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "kats.json")))
TREE_PARTS = ["COUNTS", "LEVEL_SIZES", "TOTAL_ONES", "NUM_LAST_L2",
              "NODE_RANKS", "NODE_INFOS", "CODES", "NODES_AT_LEVEL",
              "ALPHABET"]
LEVEL_PARTS = ["LEVEL_WORDS", "L1", "L2", "SAMPLES0", "SAMPLES1"]


def bits_of(words, n):
    return [(int(words[i // 32]) >> (i % 32)) & 1 for i in range(n)]


def assert_same_tree(gt, ot):
    for p in TREE_PARTS:
        a, b = gt.export(p), ot.export(p)
        assert a.dtype == b.dtype and np.array_equal(a, b), p
    for l in range(gt.getNumLevels()):
        for p in LEVEL_PARTS:
            a, b = gt.export(p, l), ot.export(p, l)
            assert np.array_equal(a, b), (p, l)


def check_queries(gt, ot, text, alphabet, m, seed):
    rng = np.random.default_rng(seed)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    assert np.array_equal(gt.access(idx).astype(np.uint64), ot.scan_access(idx))
    want, st = ot.scan_rank(rk, rs)
    assert st == 0
    assert np.array_equal(gt.rank(gt.make_queries(rk, rs)), want)
    want, st = ot.scan_select(sk, ss)
    assert st == 0
    assert np.array_equal(gt.select(gt.make_queries(sk, ss)), want)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    want, st = ot.mixed(types, index, sym)
    assert st == 0
    assert np.array_equal(gt.mixed(types, gt.make_queries(index, sym)), want)


# ---- known answers of the reference test suite --------------------------

@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
@pytest.mark.parametrize("case", ["sigma10", "sigma5"])
def test_structure_kats(ewt, dtype, case):
    c = KATS["structure"][case]
    t = ewt.WaveletTree(np.array(c["data"], dtype=dtype), c["alphabet"])
    sizes = t.export("LEVEL_SIZES")
    for l, want in enumerate(c["levels"]):
        assert int(sizes[l]) == len(want)
        assert bits_of(t.export("LEVEL_WORDS", l), len(want)) == want


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
@pytest.mark.parametrize("mod", KATS["modulo"], ids=lambda m: "s%d" % m["sigma"])
def test_modulo_kats(ewt, dtype, mod):
    sigma, n = mod["sigma"], mod["n"]
    if sigma > np.iinfo(dtype).max + 1:
        pytest.skip("alphabet wider than the type")
    data = (np.arange(n) % sigma).astype(dtype)
    t = ewt.WaveletTree(data, np.arange(sigma))
    # every prefix length, as the reference's access test does
    for m in (1, 2, 7, n // 2, n - 1):
        assert np.array_equal(t.access(np.arange(m)), data[:m])
    r = t.rank(t.make_queries(mod["rank_index"], mod["rank_symbol"]))
    assert list(r) == mod["rank_result"]
    s = t.select(t.make_queries(mod["select_k"], mod["select_symbol"]))
    assert list(s) == mod["select_result"]
    s = t.select(t.make_queries([mod["missing_k"]], [0]))
    assert int(s[0]) == mod["missing_result"]


def test_rs_index_sizes(ewt):
    k = KATS["index_sizes"]
    words = [np.zeros((s + 31) // 32, np.uint32) for s in k["sizes"]]
    rs = ewt.RankSelect(words, k["sizes"])
    for a in range(len(k["sizes"])):
        assert len(rs.export("L1", a)) == k["num_l1"][a]
        assert len(rs.export("L2", a)) == k["num_l2"][a]
        assert not rs.export("L1", a).any() and not rs.export("L2", a).any()
    assert list(rs.export("NUM_LAST_L2")) == k["num_last_l2"]


@pytest.mark.parametrize("value", [0, 1])
def test_rs_uniform_content(ewt, value):
    k = KATS["uniform"]
    fill = 0xFFFFFFFF if value else 0
    arrs = k["arrays"]
    words = [np.full((a["bits"] + 31) // 32, fill, np.uint32) for a in arrs]
    rs = ewt.RankSelect(words, [a["bits"] for a in arrs])
    for i, a in enumerate(arrs):
        l1 = rs.export("L1", i).astype(np.int64)
        l2 = rs.export("L2", i).astype(np.int64)
        if value:
            assert list(l1) == a["l1_ones"] and list(l2) == a["l2_ones"]
        else:
            assert not l1.any() and not l2.any()
    sm = k["samples"]
    words = [np.full((a["bits"] + 31) // 32, fill, np.uint32) for a in sm]
    rs = ewt.RankSelect(words, [a["bits"] for a in sm])
    ones = rs.export("TOTAL_ONES")
    for i, a in enumerate(sm):
        assert int(ones[i]) == (a["bits"] if value else 0)
        got = rs.export("SAMPLES1" if value else "SAMPLES0", i)
        assert list(got) == a["samples"]
        # closed-form rank/select of a uniform array (test_rank_select.cu
        # :557-663): rank(pos) == pos, select(i) == i - 1, select past the
        # end == size
        bits = a["bits"]
        pos = np.unique(np.array([0, 1, bits // 2, bits - 1, bits]))
        assert np.array_equal(rs.rank(i, value, pos), pos)
        assert np.array_equal(rs.rank(i, 1 - value, pos), np.zeros_like(pos))
        ks = np.unique(np.array([1, max(1, bits // 3), bits]))
        assert np.array_equal(rs.select(i, value, ks), ks - 1)
        assert int(rs.select(i, 1 - value, [1])[0]) == bits


def test_rs_half_words(ewt):
    k = KATS["half_words"]
    cases = k["cases"]
    words = [np.full((c["bits"] + 31) // 32, k["word"], np.uint32)
             for c in cases]
    rs = ewt.RankSelect(words, [c["bits"] for c in cases])
    for a, c in enumerate(cases):
        assert list(rs.rank(a, 1, c["pos"])) == c["rank1"]
        assert list(rs.rank(a, 0, c["pos"])) == c["rank0"]
        s1 = np.array(c["select1"])
        assert np.array_equal(rs.select(a, 1, s1[:, 0]), s1[:, 1])
        s0 = np.array(c["select0"])
        assert np.array_equal(rs.select(a, 0, s0[:, 0]), s0[:, 1])


# ---- random parity --------------------------------------------------------

def test_rs_random_arrays(ewt, oracle):
    rng = np.random.default_rng(2024)
    for trial in range(4):
        sizes = rng.integers(200, 1_000_000, 10)
        words = [rng.integers(0, 2**32, (s + 31) // 32, dtype=np.uint64)
                 .astype(np.uint32) for s in sizes]
        if trial == 1:  # sparse and dense arrays stress the samples
            words = [w & rng.integers(0, 2**32, w.size, dtype=np.uint64)
                     .astype(np.uint32) & np.uint32(0x01010101) for w in words]
        if trial == 2:
            words = [w | np.uint32(0xFEFEFEFE) for w in words]
        g = ewt.RankSelect(words, sizes)
        o = oracle.OracleRS(words, sizes)
        for p in ("TOTAL_ONES", "LEVEL_SIZES", "NUM_LAST_L2"):
            assert np.array_equal(g.export(p), o.export(p)), p
        for a in range(len(sizes)):
            for p in LEVEL_PARTS:
                assert np.array_equal(g.export(p, a), o.export(p, a)), (p, a)
            bits = int(sizes[a])
            pos = rng.integers(0, bits + 1, 500)
            ones = int(g.export("TOTAL_ONES")[a])
            for v in (0, 1):
                want = [o.rank(a, int(p), v) for p in pos]
                assert list(g.rank(a, v, pos)) == want
                tot = ones if v else bits - ones
                ks = rng.integers(1, tot + 2, 500) if tot else np.array([1])
                want = [o.select(a, int(k), v) for k in ks]
                assert list(g.select(a, v, ks)) == want


CASES = [
    (np.uint8, 2, True, 1), (np.uint8, 4, True, 100_000),
    (np.uint8, 5, True, 65_536 * 3 + 17), (np.uint8, 10, False, 4_097),
    (np.uint8, 64, True, 300_001), (np.uint8, 255, False, 200_000),
    (np.uint8, 256, True, 1_000_003), (np.uint16, 3, True, 70_000),
    (np.uint16, 1000, False, 500_000), (np.uint16, 1024, True, 262_144),
    (np.uint16, 65535, True, 600_000), (np.uint16, 65536, True, 700_000),
    (np.uint32, 7, False, 90_000), (np.uint32, 100_000, False, 400_000),
    (np.uint64, 12, False, 50_000), (np.uint64, 4096, True, 300_000),
]


@pytest.mark.parametrize("dtype,sigma,minimal,n", CASES,
                         ids=lambda v: str(getattr(v, "__name__", v)))
def test_tree_parity(ewt, oracle, dtype, sigma, minimal, n):
    rng = np.random.default_rng(sigma * 7 + n)
    text, alphabet = random_text(rng, n, sigma, dtype, minimal=minimal)
    if n >= sigma:  # make every symbol occur at least once
        text[:sigma] = alphabet.astype(dtype)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    assert_same_tree(gt, ot)
    check_queries(gt, ot, text, alphabet, 20_000, seed=n)


def test_detected_alphabet_and_zipf(ewt, oracle):
    rng = np.random.default_rng(5)
    text, alphabet = random_text(rng, 400_000, 300, np.uint16, minimal=False,
                                 zipf=1.1)
    gt = ewt.WaveletTree(text)  # alphabet detected on the GPU
    ot = oracle.OracleTree(text)
    assert_same_tree(gt, ot)
    present = np.unique(text).astype(np.uint64)
    check_queries(gt, ot, text, present, 20_000, seed=9)


def test_config_small_dna(ewt, oracle):
    """n = 2^24 uint8 symbols iid over {0,1,2,3}; 2^20 queries of each type."""
    rng = np.random.default_rng(1)
    n, m = 1 << 24, 1 << 20
    text = rng.integers(0, 4, n, dtype=np.uint8)
    alphabet = np.arange(4)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    assert_same_tree(gt, ot)
    check_queries(gt, ot, text, alphabet.astype(np.uint64), m, seed=2)


def test_invalid_queries_report(ewt):
    text = np.array([1, 2, 3, 1, 2, 3], np.uint16)
    t = ewt.WaveletTree(text, [1, 2, 3])
    out, st = t.try_rank(t.make_queries([7, 2], [1, 1]))  # index > n
    assert st == -5 and int(out[0]) == 2**64 - 1 and int(out[1]) == 1
    out, st = t.try_select(t.make_queries([0, 1], [1, 1]))  # k == 0
    assert st == -5 and int(out[0]) == 2**64 - 1 and int(out[1]) == 0
    out, st = t.try_rank(t.make_queries([6], [9]))  # above the alphabet
    assert st == -5
    # a later valid batch is clean again
    assert list(t.rank(t.make_queries([6, 3], [1, 0]))) == [2, 1]
    assert list(t.select(t.make_queries([3], [3]))) == [6]
    assert list(t.access([0, 5, 6, 100])) == [1, 3, 0, 0]


def test_build_rejects_bad_alphabets(ewt):
    with pytest.raises(ewt.EwtError) as e:
        ewt.WaveletTree(np.array([1, 2, 9], np.uint8), [1, 2, 3])
    assert e.value.status == -4
    with pytest.raises(ewt.EwtError) as e:
        ewt.WaveletTree(np.array([1, 2], np.uint8), [2, 1])
    assert e.value.status == -4
    with pytest.raises(ewt.EwtError) as e:
        ewt.WaveletTree(np.array([5, 5, 5], np.uint8))
    assert e.value.status == -4


def test_device_resident_batches(ewt, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(8)
    text, alphabet = random_text(rng, 300_000, 50, np.uint8, minimal=False)
    dtext = torch.from_numpy(text).cuda()
    gt = ewt.WaveletTree(dtext, alphabet)  # built from device memory
    ot = oracle.OracleTree(text, alphabet)
    assert_same_tree(gt, ot)
    m = 50_000
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    d_idx = torch.from_numpy(idx.view(np.int64)).cuda()
    d_out = torch.zeros(m, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    gt.access_device(d_idx.data_ptr(), m, d_out.data_ptr(), s)
    q = gt.make_queries(rk, rs)
    d_q = torch.from_numpy(q.view(np.uint8)).cuda()
    d_r = torch.zeros(m, dtype=torch.int64, device="cuda")
    gt.rank_device(d_q.data_ptr(), m, d_r.data_ptr(), s)
    assert gt.query_status(s) == 0
    assert np.array_equal(d_out.cpu().numpy().astype(np.uint64),
                          ot.scan_access(idx))
    assert np.array_equal(d_r.cpu().numpy().view(np.uint64),
                          ot.scan_rank(rk, rs)[0])


@pytest.mark.parametrize("n,sigma", [((1 << 31) + 12345, 256),
                                     ((1 << 32) + 777, 4),
                                     ((1 << 32) + 96 * 7 + 5, 256)])
def test_large_text_round_trips(ewt, n, sigma):
    """n > 2^31 exercises 64-bit positions, n > 2^32 also level arrays
    longer than 2^24 rank blocks (their counts need the high-count table);
    size-independent properties: rank answers (rank blocks) agree with
    select answers (L1/L2 counts and samples) and with the text itself."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(3)
    dtext = torch.randint(0, sigma, (n,), dtype=torch.uint8, device="cuda",
                          generator=g)
    t = ewt.WaveletTree(dtext, np.arange(sigma))
    counts = t.export("COUNTS").astype(np.int64)
    occ = np.diff(np.append(counts, n))
    hist = torch.bincount(dtext.to(torch.int32), minlength=sigma).cpu().numpy()
    assert np.array_equal(occ, hist)
    # level 0 holds the top code bit of every symbol in text order
    w0 = t.export("LEVEL_WORDS", 0)
    assert int(np.unpackbits(w0.view(np.uint8)).sum()) == int(hist[sigma // 2:].sum())
    rng = np.random.default_rng(4)
    m = 200_000
    sym = rng.integers(0, sigma, m).astype(np.uint64)
    k = (rng.random(m) * occ[sym]).astype(np.uint64) + 1
    pos = t.select(t.make_queries(k, sym))
    assert (pos < n).all()
    assert np.array_equal(t.access(pos).astype(np.uint64), sym)
    assert np.array_equal(t.rank(t.make_queries(pos, sym)), k - 1)
    idx = rng.integers(0, n, m).astype(np.uint64)
    edge = 224 << 24  # first bit covered by the second high-count entry
    near = np.arange(edge - 300, edge + 300, dtype=np.uint64)
    idx = np.concatenate([idx, near[near < n]])
    c = t.access(idx).astype(np.uint64)
    assert np.array_equal(c, dtext[torch.from_numpy(idx.view(np.int64)).cuda()]
                          .cpu().numpy())
    r = t.rank(t.make_queries(idx, c))
    assert np.array_equal(t.select(t.make_queries(r + 1, c)), idx)
    assert np.array_equal(t.rank(t.make_queries(np.full(sigma, n), np.arange(sigma))),
                          occ.astype(np.uint64))


@pytest.mark.parametrize("dtype,sigma", [(np.uint8, 256), (np.uint16, 1000)])
def test_pipelined_host_batches(ewt, oracle, dtype, sigma):
    """Host batches of 2^21 queries and more run pipelined (queries copied
    in and results copied out chunk by chunk while other chunks are
    answered); every answer equals the oracle's walk, including a ragged
    last chunk."""
    from tests.workloads import random_queries, random_text
    rng = np.random.default_rng(sigma)
    text, alphabet = random_text(rng, 1 << 22, sigma, dtype, minimal=sigma == 256)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    m = (1 << 21) + 4097
    idx, rk, rs, sk, ss = random_queries(rng, text, np.asarray(alphabet, np.uint64), m)
    assert np.array_equal(gt.access(idx).astype(np.uint64), ot.access(idx))
    want, st = ot.rank(rk, rs)
    assert st == 0
    assert np.array_equal(gt.rank(gt.make_queries(rk, rs)), want)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    want, st = ot.mixed(types, index, sym)
    assert st == 0
    assert np.array_equal(gt.mixed(types, gt.make_queries(index, sym)), want)
