"""Pins the CPU oracle to the reference test suite's known answers.

The fixtures in tests/golden/kats.json restate closed-form expectations of
mfranzreb/ECL_wavelet's gtest suites (see make_golden.py for the file:line
of each); these tests check the oracle against every one of them.
"""
import json
import os

import numpy as np
import pytest

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "kats.json")))


def bits_of(words, n):
    return [(int(words[i // 32]) >> (i % 32)) & 1 for i in range(n)]


def test_minimal_codes(oracle):
    k = KATS["minimal_codes"]
    for s in ("72", "63", "75"):
        assert [list(c) for c in oracle.minimal_codes(int(s))] == k[s]
    for s in k["pow2_empty"]:
        assert oracle.minimal_codes(s) == []


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
@pytest.mark.parametrize("case", ["sigma10", "sigma5"])
def test_structure_levels(oracle, dtype, case):
    c = KATS["structure"][case]
    t = oracle.OracleTree(np.array(c["data"], dtype=dtype), c["alphabet"])
    sizes = t.export("LEVEL_SIZES")
    for l, want in enumerate(c["levels"]):
        assert int(sizes[l]) == len(want)
        assert bits_of(t.export("LEVEL_WORDS", l), len(want)) == want


@pytest.mark.parametrize("mod", KATS["modulo"], ids=lambda m: "s%d" % m["sigma"])
def test_modulo_queries(oracle, mod):
    sigma, n = mod["sigma"], mod["n"]
    data = (np.arange(n) % sigma).astype(np.uint8 if sigma <= 256 else np.uint16)
    t = oracle.OracleTree(data, np.arange(sigma))
    idx = np.arange(n)
    assert (t.access(idx) == data).all()
    r, st = t.rank(mod["rank_index"], mod["rank_symbol"])
    assert st == 0 and list(r) == mod["rank_result"]
    s, st = t.select(mod["select_k"], mod["select_symbol"])
    assert st == 0 and list(s) == mod["select_result"]
    s, _ = t.select([mod["missing_k"]], [0])
    assert int(s[0]) == mod["missing_result"]


def test_index_sizes(oracle):
    k = KATS["index_sizes"]
    words = [np.zeros((s + 31) // 32, np.uint32) for s in k["sizes"]]
    rs = oracle.OracleRS(words, k["sizes"])
    for a in range(len(k["sizes"])):
        assert len(rs.export("L1", a)) == k["num_l1"][a]
        assert len(rs.export("L2", a)) == k["num_l2"][a]
    assert list(rs.export("NUM_LAST_L2")) == k["num_last_l2"]


@pytest.mark.parametrize("value", [0, 1])
def test_uniform_content(oracle, value):
    k = KATS["uniform"]
    fill = 0xFFFFFFFF if value else 0
    arrs = k["arrays"]
    words = [np.full((a["bits"] + 31) // 32, fill, np.uint32) for a in arrs]
    rs = oracle.OracleRS(words, [a["bits"] for a in arrs])
    for i, a in enumerate(arrs):
        l1 = rs.export("L1", i).astype(np.int64)
        l2 = rs.export("L2", i).astype(np.int64)
        if value:
            assert list(l1) == a["l1_ones"] and list(l2) == a["l2_ones"]
        else:
            assert not l1.any() and not l2.any()
    sm = k["samples"]
    words = [np.full((a["bits"] + 31) // 32, fill, np.uint32) for a in sm]
    rs = oracle.OracleRS(words, [a["bits"] for a in sm])
    ones = rs.export("TOTAL_ONES")
    for i, a in enumerate(sm):
        assert int(ones[i]) == (a["bits"] if value else 0)
        got = rs.export("SAMPLES1" if value else "SAMPLES0", i)
        assert list(got) == a["samples"]
        assert len(rs.export("SAMPLES0" if value else "SAMPLES1", i)) == 0


def test_half_words(oracle):
    k = KATS["half_words"]
    cases = k["cases"]
    words = [np.full((c["bits"] + 31) // 32, k["word"], np.uint32)
             for c in cases]
    rs = oracle.OracleRS(words, [c["bits"] for c in cases])
    for a, c in enumerate(cases):
        for p, r1, r0 in zip(c["pos"], c["rank1"], c["rank0"]):
            assert rs.rank(a, p, 1) == r1
            assert rs.rank(a, p, 0) == r0
        for i, want in c["select1"]:
            assert rs.select(a, i, 1) == want
        for i, want in c["select0"]:
            assert rs.select(a, i, 0) == want
        # reference edge cases: rank at 0 and at size; select past the end
        assert rs.rank(a, 0, 1) == 0
        assert rs.rank(a, c["bits"], 1) + rs.rank(a, c["bits"], 0) == c["bits"]
        total1 = rs.rank(a, c["bits"], 1)
        assert rs.select(a, total1 + 1, 1) == c["bits"]


def test_utils_tables(oracle):
    u = KATS["utils"]
    for i, want in enumerate(u["prev_pow2"]):
        assert oracle.prev_pow2(i) == want
    for i, want in enumerate(u["ceil_log2"]):
        if want is not None:
            assert oracle.ceil_log2(i) == want


def test_node_positions_enumerate_levels(oracle):
    # tests/test_wavelet_tree.cu:219-259: getNodePosAtLevel numbers the node
    # starts of each level 0, 1, 2, ... in getNodeInfos order.
    rng = np.random.default_rng(7)
    for sigma in list(rng.integers(2, 65535, 40)) + [3, 5, 9, 12, 256, 1000]:
        sigma = int(sigma)
        nodes = oracle.node_infos(sigma)
        counter, prev_level = 0, None
        for start, level in nodes:
            if level != prev_level:
                counter, prev_level = 0, level
            assert oracle.node_pos(sigma, start, level) == counter
            counter += 1
