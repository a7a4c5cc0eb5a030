"""Query launches captured in a CUDA graph.  The device entry points
(ewt_access_device ... ewt_mixed_device) enqueue kernel launches on the
caller's stream and nothing else, so a caller captures them once and replays
the graph over new query contents written into the same buffers.  Every
replay must answer exactly as the plain scan (integer results: zero
tolerance), before and after the launch shapes were autotuned.
"""
import numpy as np
import pytest

from tests.workloads import random_queries, random_text

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,sigma,tuned", [(np.uint8, 256, False),
                                               (np.uint16, 1024, True),
                                               (np.uint32, 300, False)])
def test_captured_queries_replay_exact(ewt, oracle, dtype, sigma, tuned):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(sigma + 5)
    text, alphabet = random_text(rng, 400_000, sigma, dtype, minimal=False)
    gt = ewt.WaveletTree(text, alphabet)
    if tuned:
        gt.autotune(1 << 14)
    ot = oracle.OracleTree(text, alphabet)
    m = 40_000
    es = np.dtype(dtype).itemsize
    dev = torch.device("cuda", 0)
    d_idx = torch.empty(m, dtype=torch.int64, device=dev)
    d_rq = torch.empty(m * 16, dtype=torch.uint8, device=dev)
    d_sq = torch.empty(m * 16, dtype=torch.uint8, device=dev)
    d_mq = torch.empty(m * 16, dtype=torch.uint8, device=dev)
    d_types = torch.empty(m, dtype=torch.uint8, device=dev)
    o_acc = torch.empty(m * es, dtype=torch.uint8, device=dev)
    o_rank = torch.empty(m, dtype=torch.int64, device=dev)
    o_sel = torch.empty(m, dtype=torch.int64, device=dev)
    o_mix = torch.empty(m, dtype=torch.int64, device=dev)

    def enqueue(sp):
        gt.access_device(d_idx.data_ptr(), m, o_acc.data_ptr(), sp)
        gt.rank_device(d_rq.data_ptr(), m, o_rank.data_ptr(), sp)
        gt.select_device(d_sq.data_ptr(), m, o_sel.data_ptr(), sp)
        gt.mixed_device(d_types.data_ptr(), d_mq.data_ptr(), m,
                        o_mix.data_ptr(), sp)

    def fill(rep):  # seeded valid queries written into the same buffers
        qrng = np.random.default_rng(100 * sigma + rep)
        idx, rk, rs, sk, ss = random_queries(qrng, text, alphabet, m)
        types = qrng.integers(0, 3, m).astype(np.uint8)
        index = np.where(types == 0, idx, np.where(types == 1, rk, sk))
        sym = np.where(types == 1, rs, ss)
        d_idx.copy_(torch.from_numpy(idx.view(np.int64)))
        d_rq.copy_(torch.from_numpy(gt.make_queries(rk, rs).view(np.uint8)))
        d_sq.copy_(torch.from_numpy(gt.make_queries(sk, ss).view(np.uint8)))
        d_mq.copy_(torch.from_numpy(gt.make_queries(index, sym).view(np.uint8)))
        d_types.copy_(torch.from_numpy(types))
        torch.cuda.synchronize()
        return idx, rk, rs, sk, ss, types, index, sym

    fill(99)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        enqueue(side.cuda_stream)  # warm-up outside the capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    assert gt.query_status() == 0
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        enqueue(torch.cuda.current_stream().cuda_stream)

    for rep in range(3):  # new queries in the same buffers, then replay
        idx, rk, rs, sk, ss, types, index, sym = fill(rep)
        graph.replay()
        torch.cuda.synchronize()
        assert gt.query_status() == 0
        got = o_acc.cpu().numpy().view(dtype).astype(np.uint64)
        assert np.array_equal(got, ot.scan_access(idx)), rep
        want, st = ot.scan_rank(rk, rs)
        assert st == 0
        assert np.array_equal(o_rank.cpu().numpy().view(np.uint64), want), rep
        want, st = ot.scan_select(sk, ss)
        assert st == 0
        assert np.array_equal(o_sel.cpu().numpy().view(np.uint64), want), rep
        want, st = ot.mixed(types, index, sym)
        assert st == 0
        assert np.array_equal(o_mix.cpu().numpy().view(np.uint64), want), rep
