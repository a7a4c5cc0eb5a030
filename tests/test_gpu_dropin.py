"""The C++ drop-in API (ecl::WaveletTree<T> from include/ecl_wavelet) works
as the reference's does: host batches and a user kernel that receives the
tree by value and calls deviceAccess / deviceRank / deviceSelect."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,sigma", [(100_000, 4), (300_001, 37), (70_000, 256)])
def test_dropin_example(ewt, oracle, tmp_path, n, sigma):
    from ecl_wavelet_gb300 import dropin
    exe = dropin.build_example()
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(n), str(sigma), "12345", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    hdr = np.frombuffer(raw[:24], np.uint64)
    n_, s_, m = (int(v) for v in hdr)
    assert (n_, s_) == (n, sigma)
    off = 24
    text = np.frombuffer(raw[off:off + n], np.uint8); off += n
    idx = np.frombuffer(raw[off:off + 8 * m], np.uint64); off += 8 * m
    qdt = ewt.QUERY_DTYPE[np.dtype(np.uint8)]
    rq = np.frombuffer(raw[off:off + 16 * m], qdt); off += 16 * m
    sq = np.frombuffer(raw[off:off + 16 * m], qdt); off += 16 * m
    host = np.frombuffer(raw[off:off + 24 * m], np.uint64).reshape(3, m)
    off += 24 * m
    dev = np.frombuffer(raw[off:off + 32 * m], np.uint64).reshape(m, 4)
    ot = oracle.OracleTree(text)  # alphabet detected, as in the example
    alpha = ot.export("ALPHABET")
    want_a = ot.scan_access(idx)
    want_r = ot.scan_rank(rq["index"], rq["symbol"].astype(np.uint64))[0]
    want_s = ot.scan_select(sq["index"], sq["symbol"].astype(np.uint64))[0]
    assert np.array_equal(host[0], want_a)
    assert np.array_equal(host[1], want_r)
    assert np.array_equal(host[2], want_s)
    # device calls answer in the minimal alphabet; here the detected
    # alphabet is 0..sigma-1 (every symbol occurs), so they coincide
    assert list(alpha) == list(range(sigma))
    assert np.array_equal(dev[:, 0], want_a)
    assert np.array_equal(dev[:, 1], want_r)
    assert np.array_equal(dev[:, 2], want_s)
    lvl0 = ot.export("LEVEL_WORDS", 0)
    bits = np.unpackbits(lvl0.view(np.uint8), bitorder="little")
    csum = np.concatenate([[0], np.cumsum(bits, dtype=np.uint64)])
    assert np.array_equal(dev[:, 3], csum[idx.astype(np.int64)])


@pytest.mark.parametrize("init", [0, 1])
def test_bitarray_filled_by_user_kernel(ewt, oracle, tmp_path, init):
    """BitArray(sizes[, init]) filled by a user kernel (writeWord /
    writeWordAtBit), moved into RankSelect(BitArray&&, gpu), queried by a
    user kernel: every rank (both values, with the bit) and select answer,
    and the total ones, equal the oracle's restatement of the reference's
    RankSelect over the same words."""
    from ecl_wavelet_gb300 import dropin
    exe = dropin.build_example("bitarray_example")
    out = tmp_path / "ba.bin"
    r = subprocess.run([exe, str(init), "4242", str(out)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    A, m, init_, need_ba, need_rs = (int(v) for v in np.frombuffer(raw[:40], np.uint64))
    assert init_ == init
    off = 40
    sizes = np.frombuffer(raw[off:off + 8 * A], np.uint64).astype(np.int64)
    off += 8 * A
    assert need_rs > need_ba >= int(sizes.sum()) // 8
    words, queries = [], []
    for a in range(A):
        nw = (int(sizes[a]) + 31) // 32
        words.append(np.frombuffer(raw[off:off + 4 * nw], np.uint32))
        off += 4 * nw
        pos = np.frombuffer(raw[off:off + 8 * m], np.uint64); off += 8 * m
        k1 = np.frombuffer(raw[off:off + 8 * m], np.uint64); off += 8 * m
        k0 = np.frombuffer(raw[off:off + 8 * m], np.uint64); off += 8 * m
        res = np.frombuffer(raw[off:off + 48 * m], np.uint64).reshape(m, 6)
        off += 48 * m
        queries.append((pos, k1, k0, res))
    ors = oracle.OracleRS(words, sizes)
    ones = ors.export("TOTAL_ONES")
    for a, (pos, k1, k0, res) in enumerate(queries):
        r1 = ors.rank_batch(a, pos, 1)
        assert np.array_equal(res[:, 0], r1), a
        assert np.array_equal(res[:, 1], pos - r1), a
        w = words[a]
        p = pos.astype(np.int64)
        inside = p < int(sizes[a])
        bit = np.zeros(m, np.uint64)
        bit[inside] = (w[p[inside] // 32] >> (p[inside] % 32).astype(np.uint32)) & 1
        assert np.array_equal(res[:, 2], bit), a
        assert np.array_equal(res[:, 3], ors.select_batch(a, k1, 1)), a
        assert np.array_equal(res[:, 4], ors.select_batch(a, k0, 0)), a
        assert np.all(res[:, 5] == ones[a]), a


@pytest.mark.parametrize("seed", [7, 2024])
def test_cooperative_rank_select(ewt, seed):
    """RankSelect::rank<NumThreads, ...> / select<Value, NumThreads> with
    2, 4, 8, 16 and 32 lanes per query give the single-lane answers (which
    the tests above check against the oracle), on a tree's levels (rank
    blocks, dense samples) and on standalone arrays (reference-format
    samples; sparse arrays make select's brackets span many L1 blocks)."""
    from ecl_wavelet_gb300 import dropin
    exe = dropin.build_example("coop_rank_select")
    r = subprocess.run([exe, str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if "differences" in l]
    assert len(lines) == 2 and all(l.endswith(" 0 differences") for l in lines), r.stdout


def test_needed_memory_bounds_built_trees(ewt):
    """WaveletTree::getNeededGPUMemory's figure (ewt_needed_memory) bounds the
    device bytes of the finished trees it describes."""
    import ctypes
    rng = np.random.default_rng(8)
    for dtype, sigma, n in ((np.uint8, 256, 3_000_000), (np.uint8, 5, 2_000_000),
                            (np.uint16, 1000, 1_000_000),
                            (np.uint32, 70_000, 500_000)):
        text = rng.integers(0, sigma, n).astype(dtype)
        t = ewt.WaveletTree(text, np.arange(sigma))
        b = ctypes.c_uint64()
        assert ewt.lib().ewt_needed_memory(2, n, np.dtype(dtype).itemsize,
                                           sigma, ctypes.byref(b)) == 0
        assert t.info.device_bytes <= b.value, (dtype, sigma)
        t.close()
