"""Many trees at once, through the C ABI: ewt_build_batch (texts built
concurrently) must give trees byte-identical to the oracle's, and
ewt_mixed_multi (one launch over interleaved queries of many trees) must
answer every query exactly as the plain scan of its own text.  Integer
results: zero tolerance.
"""
import ctypes as C

import numpy as np
import pytest

from tests.test_gpu_parity import assert_same_tree
from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu


def make_texts(rng, count, dtype=np.uint8):
    texts, alphabets = [], []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 18))))
        sigma = int(rng.choice([2, 4, 5, 16, 64, 100, 256]))
        t, a = random_text(rng, n, sigma, dtype, minimal=bool(i % 3))
        texts.append(t)
        alphabets.append(a)
    return texts, alphabets


def interleaved_queries(rng, trees, texts, alphabets, per_tree):
    tree_of, types, index, sym = [], [], [], []
    for i, (t, a) in enumerate(zip(texts, alphabets)):
        idx, rk, rs, sk, ss = random_queries(rng, t, a, per_tree)
        ty = rng.integers(0, 3, per_tree).astype(np.uint8)
        tree_of.append(np.full(per_tree, i, np.uint32))
        types.append(ty)
        index.append(np.where(ty == 0, idx, np.where(ty == 1, rk, sk)))
        sym.append(np.where(ty == 1, rs, ss))
    perm = rng.permutation(per_tree * len(trees))
    cat = lambda xs: np.concatenate(xs)[perm]
    return cat(tree_of), cat(types), cat(index), cat(sym)


def test_build_batch_matches_oracle(ewt, oracle):
    rng = np.random.default_rng(21)
    texts, alphabets = make_texts(rng, 24)
    trees = ewt.build_batch(texts, alphabets)
    for t, a, gt in zip(texts, alphabets, trees):
        assert_same_tree(gt, oracle.OracleTree(t, a))
    detected = ewt.build_batch(texts[:5])  # alphabets detected per text
    for t, gt in zip(texts[:5], detected):
        assert_same_tree(gt, oracle.OracleTree(t))


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_mixed_multi_matches_scan(ewt, oracle, dtype):
    rng = np.random.default_rng(22)
    texts, alphabets = make_texts(rng, 12, dtype)
    trees = ewt.build_batch(texts, alphabets)
    tree_of, types, index, sym = interleaved_queries(rng, trees, texts,
                                                     alphabets, 3000)
    q = trees[0].make_queries(index, sym)
    got = ewt.mixed_multi(trees, tree_of, types, q)
    for i, (t, a) in enumerate(zip(texts, alphabets)):
        sel = tree_of == i
        want, st = oracle.OracleTree(t, a).mixed(types[sel], index[sel], sym[sel])
        assert st == 0
        assert np.array_equal(got[sel], want), i


def test_mixed_multi_unknown_tree_and_device_form(ewt, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(23)
    texts, alphabets = make_texts(rng, 4)
    trees = ewt.build_batch(texts, alphabets)
    tree_of, types, index, sym = interleaved_queries(rng, trees, texts,
                                                     alphabets, 500)
    q = trees[0].make_queries(index, sym)
    bad = tree_of.copy()
    bad[7] = 4  # names no tree
    with pytest.raises(ewt.EwtError) as ex:
        ewt.mixed_multi(trees, bad, types, q)
    assert ex.value.status == -5
    # device buffers on a caller stream
    lib = ewt.lib()
    dev = torch.device("cuda", 0)
    d_tree = torch.from_numpy(tree_of.astype(np.int32)).to(dev)
    d_types = torch.from_numpy(types).to(dev)
    d_q = torch.from_numpy(q.view(np.uint8)).to(dev)
    d_out = torch.empty(types.size, dtype=torch.int64, device=dev)
    d_err = torch.zeros(1, dtype=torch.int32, device=dev)
    hp = (C.c_void_p * len(trees))(*[t.handle for t in trees])
    s = torch.cuda.current_stream()
    st = lib.ewt_mixed_multi_device(hp, len(trees), d_tree.data_ptr(),
                                    d_types.data_ptr(), d_q.data_ptr(),
                                    types.size, d_out.data_ptr(),
                                    d_err.data_ptr(), s.cuda_stream)
    assert st == 0
    s.synchronize()
    assert int(d_err.item()) == 0
    got = d_out.cpu().numpy().view(np.uint64)
    assert np.array_equal(got, ewt.mixed_multi(trees, tree_of, types, q))


def test_mixed_multi_many_trees(ewt, oracle):
    """More trees than the shared-memory grouping holds (4,096): the batch is
    grouped with global atomics instead and still answers every query as the
    plain scan of its own text."""
    rng = np.random.default_rng(24)
    count = 4200
    texts = [rng.integers(0, 4, int(rng.integers(50, 300)), dtype=np.uint64)
             .astype(np.uint8) for _ in range(count)]
    alphabets = [np.arange(4)] * count
    trees = ewt.build_batch(texts, alphabets)
    tree_of, types, index, sym = interleaved_queries(rng, trees, texts,
                                                     alphabets, 20)
    q = trees[0].make_queries(index, sym)
    got = ewt.mixed_multi(trees, tree_of, types, q)
    for i in range(0, count, 97):  # a spread of trees checked on the CPU
        sel = tree_of == i
        want, st = oracle.OracleTree(texts[i], alphabets[i]).mixed(
            types[sel], index[sel], sym[sel])
        assert st == 0
        assert np.array_equal(got[sel], want), i
    for t in trees:
        t.close()
