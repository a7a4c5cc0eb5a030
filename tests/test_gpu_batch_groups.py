"""The segmented group build of a batch's short texts (ewt_build_batch):
texts below 2^22 symbols with a given power-of-two alphabet 0..sigma-1 are
built together as one tree per alphabet size whose top levels are the text
number, then cut into one tree per text over a shared store.  Every tree
must export exactly the oracle's structure and answer every query as the
plain scan (integer results: zero tolerance), whatever the group's size
(including groups split at the pass pipeline's node limit), the texts'
lengths (1 symbol, not multiples of 32 or 65536), their symbol size, the
order the trees are freed in, and after an index file round trip."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

from tests.test_gpu_parity import assert_same_tree
from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu


def check_queries(tree, ot, text, alphabet, m, seed):
    rng = np.random.default_rng(seed)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    want, st = ot.mixed(types, index, sym)
    assert st == 0
    assert np.array_equal(tree.mixed(types, tree.make_queries(index, sym)), want)


@pytest.mark.parametrize("dtype,sigmas", [(np.uint8, [4, 16, 64, 256]),
                                          (np.uint16, [8, 1024, 4096])])
def test_group_build_matches_oracle(ewt, oracle, dtype, sigmas):
    rng = np.random.default_rng(len(sigmas) * 11)
    lens = [1, 31, 32, 33, 1000, 65536, 65537, 3 * 65536 + 5, 200_000,
            1_000_003]
    texts, alph = [], []
    for i, n in enumerate(lens * 2):
        sigma = sigmas[i % len(sigmas)]
        t, a = random_text(rng, n, sigma, dtype)
        texts.append(t)
        alph.append(a)
    trees = ewt.build_batch(texts, alph)
    for i, (t, a, gt) in enumerate(zip(texts, alph, trees)):
        ot = oracle.OracleTree(t, a)
        assert_same_tree(gt, ot)
        check_queries(gt, ot, t, a, 2000, i)
    # free in a scrambled order: the shared store outlives all but the last
    for j in rng.permutation(len(trees)):
        trees[j].close()


def test_large_group_is_split(ewt, oracle):
    """600 texts of one alphabet: more than one group tree (the pass
    pipeline starts at most at level 12)."""
    rng = np.random.default_rng(5)
    texts, alph = [], []
    for i in range(600):
        t, a = random_text(rng, int(rng.integers(1, 3000)), 256, np.uint8)
        texts.append(t)
        alph.append(a)
    trees = ewt.build_batch(texts, alph)
    for i in range(0, 600, 37):
        ot = oracle.OracleTree(texts[i], alph[i])
        assert_same_tree(trees[i], ot)
        check_queries(trees[i], ot, texts[i], alph[i], 500, i)
    for t in trees:
        t.close()


def test_group_trees_round_trip_and_tuning(ewt, oracle):
    rng = np.random.default_rng(9)
    texts, alph = [], []
    for n in (50_000, 70_000, 123_457):
        t, a = random_text(rng, n, 64, np.uint8)
        texts.append(t)
        alph.append(a)
    trees = ewt.build_batch(texts, alph)
    ot = oracle.OracleTree(texts[1], alph[1])
    # the shared store keeps its sample rate; launch shapes still tune
    assert ewt.lib().ewt_set_select_samples(trees[1].handle, 128) == -6
    trees[1].autotune(1 << 12)
    check_queries(trees[1], ot, texts[1], alph[1], 3000, 1)
    assert 0 < trees[1].info.device_bytes < 64 * texts[1].size
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.ewt")
        trees[1].save(path)
        for t in trees:
            t.close()  # the loaded copy owns its own buffers
        back = ewt.WaveletTree.load(path)
        assert_same_tree(back, ot)
        check_queries(back, ot, texts[1], alph[1], 3000, 2)
        back.close()


def test_group_reports_bad_symbols_per_text(ewt):
    rng = np.random.default_rng(3)
    good, a = random_text(rng, 5000, 16, np.uint8)
    bad = good.copy()
    bad[17] = 200  # above the alphabet 0..15
    texts = [good, bad, good]
    lens = np.array([t.size for t in texts], np.uint64)
    tp = (C.c_void_p * 3)(*[t.ctypes.data for t in texts])
    al = np.arange(16, dtype=np.uint8)
    ap = (C.c_void_p * 3)(*[al.ctypes.data] * 3)
    sg = np.full(3, 16, np.uint64)
    out = (C.c_void_p * 3)()
    st = np.zeros(3, np.int32)
    rc = ewt.lib().ewt_build_batch(tp, lens.ctypes.data, 3, 1, ap,
                                   sg.ctypes.data, 0, out, st.ctypes.data)
    assert rc == -4 and list(st) == [0, -4, 0]
    assert out[1] is None and out[0] and out[2]
    for h in (out[0], out[2]):
        assert ewt.lib().ewt_free(h) == 0
