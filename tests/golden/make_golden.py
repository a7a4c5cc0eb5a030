"""Writes tests/golden/kats.json: known answers of the reference test suite.

Every entry restates, as explicit numbers, an expectation that
mfranzreb/ECL_wavelet's own gtest suites state in closed form (paths are
inside that project).  Nothing here runs the reference; the values follow
from the formulas and literals of those tests, so they pin the oracle and
the GPU library to the reference's behaviour.

    python tests/golden/make_golden.py
"""
import json
import os

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kats.json")

L1_BITS, L2_BITS, L2_PER_L1, SAMPLE = 65536, 512, 128, 4096


def minimal_codes():
    # tests/test_wavelet_tree.cu:174-217 (createMinimalCodes)
    out = {}
    out["72"] = [[4, 64 + 8 * k] for k in range(8)]
    out["63"] = [[5, 62]]
    out["75"] = ([[5, 64 + 4 * k] for k in range(8)]
                 + [[4, 96], [4, 104], [3, 112]])
    out["pow2_empty"] = [4, 8, 16, 32]
    return out


def structure():
    # tests/test_wavelet_tree.cu:446-518: sigma=10, data i % 10, n = 100.
    s10 = {"data": [i % 10 for i in range(100)], "alphabet": list(range(10)),
           "levels": []}
    s10["levels"].append([0 if i % 10 < 8 else 1 for i in range(100)])
    s10["levels"].append([0 if i % 8 < 4 else 1 for i in range(80)]
                         + [i % 2 for i in range(80, 100)])
    s10["levels"].append([0 if i % 4 < 2 else 1 for i in range(80)])
    s10["levels"].append([i % 2 for i in range(80)])
    # tests/test_wavelet_tree.cu:520-564: sigma=5 fixed sequence; the bit
    # strings are the comments at :526, :539, :553.
    s5 = {"data": [4, 1, 1, 2, 1, 1, 3, 4, 4, 0, 0, 2, 3, 2, 4, 2, 4, 1, 3, 2],
          "alphabet": [0, 1, 2, 3, 4],
          "levels": [[int(c) for c in "10000001100000101000"],
                     [int(c) for c in "001001001111011"],
                     [int(c) for c in "111100101010010"]]}
    return {"sigma10": s10, "sigma5": s5}


def modulo_queries(sigma, n):
    # tests/test_wavelet_tree.cu:567-707: data i % sigma; access = data,
    # rank(c, j) for c = data[j] is j // sigma, select(j // sigma + 1,
    # data[j]) = j; the (count+1)-th occurrence of 0 yields n.
    data = [i % sigma for i in range(n)]
    return {"sigma": sigma, "n": n,
            "rank_index": list(range(n)), "rank_symbol": data,
            "rank_result": [j // sigma for j in range(n)],
            "select_k": [j // sigma + 1 for j in range(n)],
            "select_symbol": data, "select_result": list(range(n)),
            "missing_k": (n + sigma - 1) // sigma + 1,
            "missing_result": n}


def index_sizes():
    # tests/test_rank_select.cu:190-253
    sizes = [1, L2_BITS - 1, L2_BITS + 1, 2 * L2_BITS - 1, L1_BITS - 1,
             L1_BITS + 1, 2 * L1_BITS - 1]
    return {"sizes": sizes,
            "num_l1": [1, 1, 1, 1, 1, 2, 2],
            "num_l2": [1, 1, 2, 2, L2_PER_L1, L2_PER_L1 + 1, 2 * L2_PER_L1],
            "num_last_l2": [1, 1, 2, 2, L2_PER_L1, 1, L2_PER_L1]}


def uniform_content():
    # tests/test_rank_select.cu:309-403: all-ones / all-zeros arrays.
    sizes = [1, L2_BITS + 1, 2 * L2_BITS - 1, L1_BITS - 1, L1_BITS + 1,
             2 * L1_BITS - 1, 2 * L1_BITS + 1]
    sample_sizes = [1, SAMPLE - 1, SAMPLE, SAMPLE + 1, 2 * SAMPLE - 1,
                    2 * SAMPLE, 2 * SAMPLE + 1, 6 * SAMPLE,
                    6 * L2_BITS + L2_BITS // 5]
    arrays = []
    for s in sizes:
        nl1 = (s + L1_BITS - 1) // L1_BITS
        nl2 = (s + L2_BITS - 1) // L2_BITS
        arrays.append({"bits": s,
                       "l1_ones": [j * L1_BITS for j in range(nl1)],
                       "l2_ones": [(j % L2_PER_L1) * L2_BITS
                                   for j in range(nl2)]})
    samples = [{"bits": s,
                "samples": [j * SAMPLE - 1 for j in range(1, s // SAMPLE + 1)]}
               for s in sample_sizes]
    return {"arrays": arrays, "samples": samples}


def half_words():
    # tests/test_rank_select.cu:665-761: every word 0xFFFF0000; closed forms
    # for rank1/select1/rank0/select0 at every position of each array.
    sizes = [L2_BITS + 1, 2 * L2_BITS - 1, L1_BITS - 1, L1_BITS + 1,
             2 * L1_BITS - 1, 2 * L1_BITS + 1]
    cases = []
    for s in sizes:
        # a spread of positions incl. both ends of every block kind
        pos = sorted({1, 2, 15, 16, 17, 31, 32, 33, 48, 63, 64, 511, 512, 513,
                      s // 3, s // 2, s - 2, s - 1} & set(range(1, s)))
        r1, s1, r0, s0 = [], [], [], []
        for p in pos:
            sb = p % 32 - 16
            nw = p // 32
            rank1 = 32 * nw // 2 + (sb if sb > 0 else 0)
            rank0 = 32 * nw // 2 + min(16, p % 32)
            r1.append(rank1)
            r0.append(rank0)
            if rank1:
                sel1 = 32 * (rank1 // 16) - 1
                if rank1 % 16:
                    sel1 += 16 + rank1 % 16
                s1.append([rank1, sel1])
            if rank0:
                sel0 = 32 * (rank0 // 16) - 1
                if rank0 % 16:
                    sel0 += min(16, rank0 % 16)
                else:
                    sel0 -= 16
                s0.append([rank0, sel0])
        cases.append({"bits": s, "pos": pos, "rank1": r1, "rank0": r0,
                      "select1": s1, "select0": s0})
    return {"word": 0xFFFF0000, "cases": cases}


def utils_tables():
    # tests/test_utils.cu:30-57: getPrevPowTwo and ceilLog2 for 0..1023.
    prev, exp = [], 0
    for i in range(1024):
        prev.append(exp)
        if i & (i - 1) == 0:
            exp = i
    clog, e = [None], 0
    for i in range(1, 1024):
        clog.append(e)
        if i & (i - 1) == 0:
            e += 1
    return {"prev_pow2": prev, "ceil_log2": clog}


def main():
    kats = {"minimal_codes": minimal_codes(), "structure": structure(),
            "modulo": [modulo_queries(10, 100), modulo_queries(256, 1280)],
            "index_sizes": index_sizes(), "uniform": uniform_content(),
            "half_words": half_words(), "utils": utils_tables()}
    with open(OUT, "w") as f:
        json.dump(kats, f, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
