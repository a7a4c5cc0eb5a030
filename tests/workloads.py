"""Seeded synthetic texts and query batches shared by tests and bench.py.

The reference measures on uniform random texts (README.md:12-13 of
mfranzreb/ECL_wavelet); these generators reproduce those shapes: iid
uniform or Zipf(s) symbols over a minimal or scattered alphabet, access
positions uniform in [0, n), rank positions uniform in [0, n], select k
uniform in [1, count(c)] (plus a share past the last occurrence).
"""
import numpy as np


def random_alphabet(rng, sigma, dtype, minimal=True):
    if minimal:
        return np.arange(sigma, dtype=np.uint64)
    hi = np.iinfo(dtype).max
    if sigma > hi // 2:
        return np.arange(sigma, dtype=np.uint64) + np.uint64(hi + 1 - sigma)
    a = np.unique(rng.integers(0, hi, size=sigma * 3, dtype=np.uint64,
                               endpoint=True))
    while a.size < sigma:
        a = np.unique(np.concatenate(
            [a, rng.integers(0, hi, size=sigma, dtype=np.uint64,
                             endpoint=True)]))
    return np.sort(rng.choice(a, sigma, replace=False)).astype(np.uint64)


def random_text(rng, n, sigma, dtype, minimal=True, zipf=None):
    """Text of n symbols drawn iid from a sigma-symbol alphabet."""
    alphabet = random_alphabet(rng, sigma, dtype, minimal)
    if zipf is None:
        ids = rng.integers(0, sigma, n)
    else:
        w = 1.0 / np.arange(1, sigma + 1) ** zipf
        ids = rng.choice(sigma, n, p=w / w.sum())
    text = alphabet[ids].astype(dtype)
    return text, alphabet


def random_queries(rng, text, alphabet, m, past_end=0.05):
    """(access idx, rank idx, rank sym, select k, select sym) in the
    reference's ranges; rank may ask at n, select may ask past the end."""
    n = text.size
    sigma = alphabet.size
    idx = rng.integers(0, n, m).astype(np.uint64)
    rk = rng.integers(0, n + 1, m).astype(np.uint64)
    rs = alphabet[rng.integers(0, sigma, m)].astype(np.uint64)
    counts = np.zeros(sigma, np.int64)
    pos = np.searchsorted(alphabet, text.astype(np.uint64))
    np.add.at(counts, pos, 1)
    sel_ids = rng.integers(0, sigma, m)
    cnt = counts[sel_ids]
    k = (rng.random(m) * np.maximum(cnt, 1)).astype(np.int64) + 1
    extra = rng.random(m) < past_end
    k[extra] = cnt[extra] + 1 + rng.integers(0, 3, int(extra.sum()))
    ss = alphabet[sel_ids].astype(np.uint64)
    return idx, rk, rs, k.astype(np.uint64), ss


def device_text(torch, n, sigma, elem_size, zipf=None, seed=0,
                chunk=1 << 27):
    """Seeded text of n symbols over [0, sigma) generated on cuda:0 (iid
    uniform, or Zipf(zipf) by inverse CDF in float64), as a uint8 (1-byte)
    or int16 (2-byte, symbols in the low 16 bits) tensor."""
    dev = "cuda"
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    dt = torch.uint8 if elem_size == 1 else torch.int16
    text = torch.empty(n, dtype=dt, device=dev)
    cdf = None
    if zipf is not None:
        w = 1.0 / torch.arange(1, sigma + 1, device=dev,
                               dtype=torch.float64) ** zipf
        cdf = torch.cumsum(w, 0) / w.sum()
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        if cdf is None:
            ids = torch.randint(0, sigma, (b - a,), device=dev, generator=gen)
        else:
            u = torch.rand(b - a, device=dev, dtype=torch.float64,
                           generator=gen)
            ids = torch.searchsorted(cdf, u).clamp_(max=sigma - 1)
        text[a:b] = ids.to(torch.int32).to(dt)
    return text


def host_view(torch_text):
    """numpy copy of a device_text tensor with unsigned symbols."""
    a = torch_text.cpu().numpy()
    return a.view(np.uint16) if a.dtype == np.int16 else a


def mixed_queries_from_counts(rng, n, occ, m):
    """m mixed queries (types 40/40/20 interleaved) over a text of n symbols
    with per-symbol occurrence counts occ: access positions in [0, n), rank
    positions in [0, n], select k in [1, occ[c]] for symbols that occur."""
    sigma = occ.size
    u = rng.random(m)
    types = np.where(u < 0.4, 0, np.where(u < 0.8, 1, 2)).astype(np.uint8)
    sym = rng.integers(0, sigma, m).astype(np.uint64)
    present = np.flatnonzero(occ)
    sel = types == 2
    sym[sel] = present[rng.integers(0, present.size, int(sel.sum()))]
    index = np.where(types == 0, rng.integers(0, n, m),
                     rng.integers(0, n + 1, m)).astype(np.uint64)
    cnt = occ[sym[sel].astype(np.int64)]
    index[sel] = (rng.random(int(sel.sum())) * cnt).astype(np.uint64) + 1
    return types, index, sym
