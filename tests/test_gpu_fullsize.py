"""Parity of the GPU build at the benchmark's full sizes.

The 6 * 2^30-symbol uint8 construction configuration (sigma 256, the timed
workload, and sigma 4) and the 3 * 2^30-symbol uint16 configurations
(sigma 65536 Zipf(1.1), sigma 1024 uniform) are built on the GPU and,
independently, by the oracle's multithreaded CPU build of the reference's
structure on all host cores.  Every export — each level's bit words, L1
and L2 counts, both select-sample arrays, the count table, total ones,
level sizes, node ranks — must be byte-identical, and 2^22 mixed queries
answered on the GPU must equal the oracle's plain scan of the text.
Integer work: zero tolerance.
"""
import numpy as np
import pytest

from tests.workloads import device_text, host_view, mixed_queries_from_counts

pytestmark = pytest.mark.gpu

GIB = 1 << 30
TREE_PARTS = ["COUNTS", "LEVEL_SIZES", "TOTAL_ONES", "NUM_LAST_L2",
              "NODE_RANKS", "NODE_INFOS", "CODES", "NODES_AT_LEVEL",
              "ALPHABET"]
LEVEL_PARTS = ["LEVEL_WORDS", "L1", "L2", "SAMPLES0", "SAMPLES1"]

CONFIGS = [
    # n, elem_size, sigma, zipf
    pytest.param(6 * GIB, 1, 256, None, id="6Gi_u8_sigma256"),
    pytest.param(6 * GIB, 1, 4, None, id="6Gi_u8_sigma4"),
    pytest.param(3 * GIB, 2, 65536, 1.1, id="3Gi_u16_sigma65536_zipf1.1"),
    pytest.param(3 * GIB, 2, 1024, None, id="3Gi_u16_sigma1024"),
]


@pytest.mark.parametrize("n,es,sigma,zipf", CONFIGS)
def test_full_size_build_and_queries(ewt, oracle, n, es, sigma, zipf):
    torch = pytest.importorskip("torch")
    import ctypes
    dtext = device_text(torch, n, sigma, es, zipf=zipf, seed=sigma + es)
    alphabet = np.arange(sigma, dtype=np.uint64)
    symbols = alphabet.astype(np.uint8 if es == 1 else np.uint16)
    h = ctypes.c_void_p()
    torch.cuda.synchronize()
    st = ewt.lib().ewt_build(dtext.data_ptr(), n, es, symbols.ctypes.data,
                             sigma, 0, ctypes.byref(h))
    assert st == 0, ewt.lib().ewt_last_error()
    gt = ewt.WaveletTree(None, _handle=h.value)
    text = host_view(dtext)
    del dtext
    torch.cuda.empty_cache()
    ot = oracle.OracleTree(text, alphabet, threads=0)
    for p in TREE_PARTS:
        a, b = gt.export(p), ot.export(p)
        assert a.dtype == b.dtype and np.array_equal(a, b), p
    for l in range(gt.getNumLevels()):
        for p in LEVEL_PARTS:
            assert np.array_equal(gt.export(p, l), ot.export(p, l)), (p, l)
    del ot
    counts = gt.export("COUNTS").astype(np.int64)
    occ = np.diff(np.append(counts, n))
    rng = np.random.default_rng(n + sigma)
    types, index, sym = mixed_queries_from_counts(rng, n, occ, 1 << 22)
    got = gt.mixed(types, gt.make_queries(index, sym))
    want, st = oracle.scan_batch(text, sigma, types, index, sym)
    assert st == 0
    assert np.array_equal(got, want)
    gt.close()
