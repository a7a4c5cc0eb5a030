"""Batched query launches hand chunks to CTAs from a device work queue (an
atomic chunk counter that the last CTA resets).  The answers must not
depend on it: with the queue and with a fixed stride, for launches that
overlap on several streams of one tree (each takes its own counter pair),
and for multi-tree batches, every result equals the oracle's plain scan
(integer results: zero tolerance)."""
import numpy as np
import pytest

from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu


def batch(gt, text, alphabet, m, seed):
    rng = np.random.default_rng(seed)
    idx, rk, rs, sk, ss = random_queries(rng, text, alphabet, m)
    types = rng.integers(0, 3, m).astype(np.uint8)
    index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
    sym = np.where(types == 1, rs, ss)
    return types, index, sym


@pytest.mark.parametrize("queue", [True, False])
def test_mixed_with_and_without_queue(ewt, oracle, queue):
    rng = np.random.default_rng(31)
    text, alphabet = random_text(rng, 900_000, 65536, np.uint16, zipf=1.1)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    try:
        ewt.set_work_queue(queue)
        for seed, m in ((1, 300_001), (2, 5000), (3, 2048)):
            types, index, sym = batch(gt, text, alphabet, m, seed)
            want, st = ot.mixed(types, index, sym)
            assert st == 0
            assert np.array_equal(gt.mixed(types, gt.make_queries(index, sym)), want)
    finally:
        ewt.set_work_queue(True)
    gt.close()


def test_overlapping_launches_on_streams(ewt, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    text, alphabet = random_text(rng, 2_000_000, 256, np.uint8)
    gt = ewt.WaveletTree(text, alphabet)
    ot = oracle.OracleTree(text, alphabet)
    dev = torch.device("cuda", 0)
    m, S = 200_000, 4
    jobs = []
    for s in range(S):
        types, index, sym = batch(gt, text, alphabet, m, 50 + s)
        q = gt.make_queries(index, sym)
        d_t = torch.from_numpy(types).to(dev)
        d_q = torch.from_numpy(q.view(np.uint8)).to(dev)
        d_o = torch.zeros(m, dtype=torch.int64, device=dev)
        jobs.append((types, index, sym, d_t, d_q, d_o, torch.cuda.Stream()))
    torch.cuda.synchronize()
    for rep in range(3):
        for (_, _, _, d_t, d_q, d_o, st) in jobs:
            gt.mixed_device(d_t.data_ptr(), d_q.data_ptr(), m, d_o.data_ptr(),
                            st.cuda_stream)
        torch.cuda.synchronize()
        assert gt.query_status() == 0
        for (types, index, sym, _, _, d_o, _) in jobs:
            want, st_ = ot.mixed(types, index, sym)
            assert st_ == 0
            assert np.array_equal(d_o.cpu().numpy().view(np.uint64), want), rep
    gt.close()


@pytest.mark.parametrize("queue", [True, False])
def test_multi_tree_with_and_without_queue(ewt, oracle, queue):
    rng = np.random.default_rng(19)
    trees, oracles, texts = [], [], []
    for k in range(6):
        sigma = int(rng.choice([4, 16, 256]))
        text, alphabet = random_text(rng, int(rng.integers(20_000, 300_000)),
                                     sigma, np.uint8)
        trees.append(ewt.WaveletTree(text, alphabet))
        oracles.append(oracle.OracleTree(text, alphabet))
        texts.append((text, alphabet))
    m = 120_000
    tree_of = rng.integers(0, len(trees), m).astype(np.uint32)
    types = np.zeros(m, np.uint8)
    index = np.zeros(m, np.uint64)
    sym = np.zeros(m, np.uint64)
    for k, (text, alphabet) in enumerate(texts):
        sel = np.flatnonzero(tree_of == k)
        ty, ix, sy = batch(trees[k], text, alphabet, sel.size, 70 + k)
        types[sel], index[sel], sym[sel] = ty, ix, sy
    q = trees[0].make_queries(index, sym)
    try:
        ewt.set_work_queue(queue)
        got = ewt.mixed_multi(trees, tree_of, types, q)
    finally:
        ewt.set_work_queue(True)
    for k in range(len(trees)):
        sel = np.flatnonzero(tree_of == k)
        want, st = oracles[k].mixed(types[sel], index[sel], sym[sel])
        assert st == 0
        assert np.array_equal(got[sel], want), k
    for t in trees:
        t.close()
