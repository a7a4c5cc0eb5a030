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
