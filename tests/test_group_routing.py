"""The construction identity behind the group query levels, on the CPU.

A group level of width w at binary level l holds, in level-l order, each
symbol's bits l .. l+w-1 (from the top).  The GPU builds it without the
level-l order of the symbols: a level-l node's zeros go, in order, to its left
child on level l+1 and its ones to its right child, so the level-(l+1) bit at
the child position of every level-l position is obtained by routing the two
child runs of level l+1 by the level-l bits ("route" below); level l+2 routed
into level-(l+1) order gives the octal digit's lowest bit the same way.

These tests restate that routing with numpy over the oracle's exported binary
levels and compare the digits with the symbols' own bits in level-l order
(a stable sort by their top l bits), for every group of the level plan: octal
(3-bit) groups first, then one or two quad (2-bit) groups covering all L
levels.  No GPU; the CUDA kernels are compared with the oracle's query answers
in the GPU parity tests.
"""
import numpy as np
import pytest

from bench import group_levels


def group_widths(L):
    """Widths of the group levels of an L-level power-of-two tree, top down."""
    if L < 2:
        return []
    quads = 0 if L % 3 == 0 else (1 if L % 3 == 2 else 2)
    return [3] * ((L - 2 * quads) // 3) + [2] * quads


def level_bits(tree, l, n):
    words = tree.export("LEVEL_WORDS", l).astype(np.uint32)
    return np.unpackbits(words.view(np.uint8), bitorder="little")[:n]


def route(h, plane, counts, l, L):
    """plane (indexed by level-(l+1) positions) read at the child position of
    every level-l position, h = the level-l bits."""
    n = h.size
    out = np.zeros(n, np.uint8)
    sh = L - l
    nodes = 1 << l
    for g in range(nodes):
        s = int(counts[g << sh])
        e = int(counts[(g + 1) << sh]) if g + 1 < nodes else n
        hb = h[s:e]
        zeros = int((hb == 0).sum())
        seg = np.empty(e - s, np.uint8)
        seg[hb == 0] = plane[s:s + zeros]   # left child, in order
        seg[hb == 1] = plane[s + zeros:e]   # right child, in order
        out[s:e] = seg
    return out


def digits_by_sort(text, l, w, L):
    order = np.argsort(text.astype(np.int64) >> (L - l), kind="stable")
    return (text[order].astype(np.int64) >> (L - l - w)) & ((1 << w) - 1)


@pytest.mark.parametrize("L", [2, 3, 4, 5, 6, 7, 8, 10])
def test_plan_covers_every_level(L):
    w = group_widths(L)
    assert sum(w) == L and w == sorted(w, reverse=True)
    assert len(w) == group_levels(L)  # the bench's read model uses the same plan


@pytest.mark.parametrize("L", [3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("shape", ["uniform", "sorted", "skewed"])
def test_routed_digits_match_sorted_symbols(oracle, L, shape):
    sigma = 1 << L
    n = 20_011
    rng = np.random.default_rng(L * 7 + len(shape))
    if shape == "skewed":  # most nodes small or empty
        text = np.minimum(rng.geometric(0.05, n) - 1, sigma - 1)
    else:
        text = rng.integers(0, sigma, n)
    if shape == "sorted":
        text = np.sort(text)
    text = text.astype(np.uint8 if sigma <= 256 else np.uint16)
    tree = oracle.OracleTree(text, np.arange(sigma))
    counts = np.append(tree.export("COUNTS").astype(np.int64), n)
    bits = [level_bits(tree, l, n) for l in range(L)]
    l = 0
    for w in group_widths(L):
        h = bits[l]
        mid = route(h, bits[l + 1], counts, l, L)
        if w == 2:
            got = 2 * h.astype(np.int64) + mid
        else:
            plane = route(bits[l + 1], bits[l + 2], counts, l + 1, L)  # level l+2 in level-(l+1) order
            low = route(h, plane, counts, l, L)
            got = 4 * h.astype(np.int64) + 2 * mid + low
        want = digits_by_sort(text, l, w, L)
        assert np.array_equal(got, want), (L, l, w)
        l += w
