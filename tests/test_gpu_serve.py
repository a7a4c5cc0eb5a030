"""The serving engine on the GPU: every request's results are the same when
it is served alone and when it is served in a mix of concurrently submitted
requests over several trees (continuous batching packs them into shared
launches), and equal to the plain scan.  Invalid queries fail only their own
request, an oversized request is refused, and a build submitted to the
server yields a tree that serves queries.  (Cancellation is covered on the
CPU by tests/test_sched.py.)  Integer results: zero
tolerance."""
import threading

import numpy as np
import pytest

from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu


def make_requests(rng, trees, texts, alphabets, count):
    reqs = []
    for _ in range(count):
        k = int(rng.integers(0, len(trees)))
        m = int(np.exp(rng.uniform(0, np.log(5000))))
        idx, rk, rs, sk, ss = random_queries(rng, texts[k], alphabets[k], m)
        ty = rng.integers(0, 3, m).astype(np.uint8)
        index = np.where(ty == 0, idx, np.where(ty == 1, rk, sk))
        sym = np.where(ty == 1, rs, ss)
        reqs.append((k, ty, trees[k].make_queries(index, sym), index, sym))
    return reqs


@pytest.mark.parametrize("staging", [False, True])
def test_alone_equals_mix(ewt, oracle, staging):
    from ecl_wavelet_gb300.serving import Server
    rng = np.random.default_rng(31)
    texts, alphabets, trees = [], [], []
    for sigma, n in ((256, 400_000), (4, 300_000), (100, 200_000)):
        t, a = random_text(rng, n, sigma, np.uint8, minimal=sigma != 100)
        texts.append(t)
        alphabets.append(a)
        trees.append(ewt.WaveletTree(t, a))
    srv = Server(batch_queries=1 << 14, batch_requests=64, inflight=2,
                 elem_size=1, force_staging=staging)
    ids = [srv.add_tree(t) for t in trees]
    reqs = make_requests(rng, trees, texts, alphabets, 120)
    alone = []
    for k, ty, q, _, _ in reqs:
        rid, out = srv.submit(ids[k], ty, q)
        st, _, _ = srv.wait(rid)
        assert st == 0
        alone.append(out.copy())
    # the mix: four threads submit interleaved, then all are awaited
    handles = [None] * len(reqs)

    def feed(part):
        for i in part:
            k, ty, q, _, _ = reqs[i]
            handles[i] = srv.submit(ids[k], ty, q)

    th = [threading.Thread(target=feed, args=(range(j, len(reqs), 4),))
          for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, (rid, out) in enumerate(handles):
        st, ms, _ = srv.wait(rid)
        assert st == 0 and ms >= 0
        assert np.array_equal(out, alone[i]), i
    # and both equal the plain scan
    for i in range(0, len(reqs), 7):
        k, ty, _, index, sym = reqs[i]
        want, st = oracle.OracleTree(texts[k], alphabets[k]).mixed(ty, index, sym)
        assert st == 0 and np.array_equal(alone[i], want)
    stats = srv.stats()
    assert stats["completed"] == 2 * len(reqs)
    assert stats["batches"] < 2 * len(reqs)  # some requests shared a launch
    srv.close()


@pytest.mark.parametrize("staging", [False, True])
def test_invalid_cancel_and_build(ewt, oracle, staging):
    from ecl_wavelet_gb300.serving import Server
    rng = np.random.default_rng(32)
    t, a = random_text(rng, 100_000, 16, np.uint8)
    tree = ewt.WaveletTree(t, a)
    srv = Server(batch_queries=1 << 12, batch_requests=8, inflight=1, elem_size=1,
                 force_staging=staging)
    tid = srv.add_tree(tree)
    good_ty = np.array([1, 2, 0], np.uint8)
    good_q = tree.make_queries([5, 1, 7], [3, 3, 0])
    bad_q = tree.make_queries([5, 0, 7], [3, 3, 0])   # select k == 0
    r_bad, out_bad = srv.submit(tid, good_ty, bad_q)
    r_good, out_good = srv.submit(tid, good_ty, good_q)
    assert srv.wait(r_bad)[0] == -5
    assert out_bad[1] == np.iinfo(np.uint64).max
    assert srv.wait(r_good)[0] == 0
    ot = oracle.OracleTree(t, a)
    want, _ = ot.mixed(good_ty, [5, 1, 7], [3, 3, 0])
    assert np.array_equal(out_good, want)
    # a request larger than a batch is refused
    big = np.zeros(1 << 13, np.uint8)
    with pytest.raises(ewt.EwtError):
        srv.submit(tid, big, tree.make_queries(np.zeros(big.size), np.zeros(big.size)))
    # build through the server, then query the new tree
    t2, a2 = random_text(rng, 50_000, 4, np.uint8)
    rb = srv.submit_build(t2, a2)
    st, _, new_id = srv.wait(rb)
    assert st == 0
    ty = np.array([0, 1, 2], np.uint8)
    rid, out = srv.submit(new_id, ty, tree.make_queries([3, 100, 2], [0, 1, 2]))
    assert srv.wait(rid)[0] == 0
    want, _ = oracle.OracleTree(t2, a2).mixed(ty, [3, 100, 2], [0, 1, 2])
    assert np.array_equal(out, want)
    srv.close()
