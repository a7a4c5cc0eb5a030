"""Benchmark of the GB300 wavelet tree on the reference's headline workload.

Workload (one step): build the wavelet tree of a 6 * 2^30-symbol uint8 text,
iid uniform over sigma = 256 symbols, already resident in HBM — histogram,
log2(sigma) level bit arrays with stable partition, RankSelect L1/L2 counts
and select samples, node-start ranks.  value = text GB/s (text bytes / step
time), the construction-sweep configuration of the reference.  After the
timed steps the same tree answers 2^26 mixed queries (40 % access, 40 %
rank, 20 % select, types interleaved at random) in the batched one-launch
form and in the plain per-type form, device-resident and end to end from
pinned host memory; the sweep over sigma in {4, 16, 64} is timed once each.
Further sections: 256 uneven texts built and queried together, the serving
loop under Poisson load, the standalone RankSelect, and uint16 texts of
3 * 2^30 symbols over sigma 65536 (Zipf 1.1) and 1024 with autotuned and
graph-replayed query launches.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/, all host cores) on a bounded sample of the same workload.
Multi-GPU runs are independent replicas (one text per GPU, no exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("Mqueries/s (access/rank/select) + build GB/s; batched vs plain, "
          "bit-exact")
GIB = 1 << 30
KINDS = ("access", "rank", "select", "mixed")



def group_levels(L):
    """Query levels of a power-of-two tree with L binary levels: octal (3-bit)
    groups, then one or two quad (2-bit) groups, covering all L levels (the
    library's plan); a one-level tree is walked binary."""
    if L < 2:
        return L
    quads = 0 if L % 3 == 0 else (1 if L % 3 == 2 else 2)
    return (L - 2 * quads) // 3 + quads

def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=6 * GIB)
    p.add_argument("--sigma", type=int, default=256)
    p.add_argument("--queries", type=int, default=1 << 26)
    p.add_argument("--no-sweep", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-multi", action="store_true",
                   help="skip the many-text build and multi-tree queries")
    p.add_argument("--no-serve", action="store_true",
                   help="skip the serving-loop rate sweep")
    p.add_argument("--no-rs", action="store_true",
                   help="skip the standalone RankSelect comparison")
    p.add_argument("--no-large", action="store_true",
                   help="skip the uint16 large-alphabet build and queries")
    p.add_argument("--cpu-sample", type=int, default=6 * GIB,
                   help="symbols of the CPU baseline build in the main arm")
    p.add_argument("--ref-sample", type=int, default=6 * GIB,
                   help="symbols per step of the --impl reference arm (the "
                        "full 6*2^30 config by default: ~5 s per step on 16 "
                        "Grace cores)")
    p.add_argument("--no-ref-gpu", action="store_true",
                   help="skip timing the reference's own GPU build")
    p.add_argument("--only", default="all",
                   choices=["all", "build", "queries", "multi", "serve", "rs",
                            "large"],
                   help="build: stop after the timed builds; queries: also "
                        "time the query batches (for profiling runs)")
    return p.parse_args()


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,"
         "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="ewt_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_tree_baseline(sigma, sample, steps=1, warmup=0, queries=1 << 22,
                      seed=99, text=None):
    """The oracle's multithreaded build of the reference's structure (the
    same levels, L1/L2 counts and samples) on every host core, over an iid
    uniform uint8 text of `sample` symbols, then `queries` mixed queries
    (40/40/20) answered by walking it, one query per loop iteration."""
    from oracle import oracle as O
    O.build_library()
    cores = int(O.lib().ewto_max_threads())
    rng = np.random.default_rng(seed)
    if text is None:
        text = rng.integers(0, sigma, sample, dtype=np.uint8)
    text = text[:sample]
    alphabet = np.arange(sigma)
    for _ in range(warmup):
        O.OracleTree(text, alphabet, threads=0)
    times = []
    t = None
    for _ in range(steps):
        t = None
        t0 = time.perf_counter()
        t = O.OracleTree(text, alphabet, threads=0)
        times.append(time.perf_counter() - t0)
    res = {"build_s": times, "cores": cores,
           "build_GB_s": sample / statistics.mean(times) / 1e9}
    if queries:
        counts = t.export("COUNTS").astype(np.int64)
        occ = np.diff(np.append(counts, sample))
        from tests.workloads import mixed_queries_from_counts
        ty, idx, sy = mixed_queries_from_counts(rng, sample, occ, queries)
        a = time.perf_counter()
        _, st = t.mixed(ty, idx, sy)
        res["mixed_queries_Mq_s"] = queries / (time.perf_counter() - a) / 1e6
        assert st == 0
        for kind, code in (("access", 0), ("rank", 1), ("select", 2)):
            k = ty == code
            a = time.perf_counter()
            t.mixed(ty[k], idx[k], sy[k])
            res[kind + "_Mq_s"] = int(k.sum()) / (time.perf_counter() - a) / 1e6
    return res


def run_reference(args, world, rank):
    """The reference arm: the reference ships no CPU implementation of the
    path, so this times the oracle's multithreaded CPU build of the
    reference's exact structure on all host cores, on a bounded sample of
    the same workload (iid uniform uint8 text, same sigma)."""
    if rank != 0:
        return
    sample = args.ref_sample
    r = cpu_tree_baseline(args.sigma, sample, steps=args.steps,
                          warmup=args.warmup, queries=0)
    ms = 1e3 * statistics.mean(r["build_s"])
    gbs = sample / (ms / 1e3) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": gbs,
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic: iid uniform uint8 text, seed 99",
        "config": {"workload": "wavelet-tree build, uint8 text, sigma=%d, "
                               "%d symbols%s" % (args.sigma, sample,
                                                 "" if sample == 6 * GIB else
                                                 " (a sample of the 6*2^30 config)"),
                   "n": sample,
                   "sigma": args.sigma, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": r["cores"],
                         "kind": "port",
                         "sample": "%d uint8 symbols, sigma=%d: full build of "
                                   "the reference's structure by the "
                                   "multithreaded CPU tree (parallel stable "
                                   "partition per level, popcount L1/L2, "
                                   "samples per L1 block)" % (sample,
                                                              args.sigma)},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def reference_gpu(n, sigma, m, reps=2, timeout=900):
    """The reference's own GPU build (baseline/build_ref.sh, unmodified
    sources) timed on this GPU: its build from pinned host memory and its
    host access / rank / select calls on m pinned queries each, asserts live
    (its default build) and with -DNDEBUG."""
    script = os.path.join(REPO, "baseline", "build_ref.sh")
    r = subprocess.run(["bash", script], capture_output=True, text=True)
    if r.returncode != 0:
        return {"unavailable": (r.stderr.strip().splitlines() or ["build failed"])[-1]}
    out = {}
    for name, key in (("ref_driver", "default_asserts_live"),
                      ("ref_driver_ndebug", "ndebug")):
        exe = os.path.join(REPO, "baseline", "_ref", name)
        try:
            p = subprocess.run([exe, "bench", str(n), "1", str(sigma), str(m),
                                str(reps)], capture_output=True, text=True,
                               timeout=timeout)
        except subprocess.TimeoutExpired:
            out[key] = {"unavailable": "timed out after %d s" % timeout}
            continue
        if p.returncode != 0:
            out[key] = {"unavailable": "exit %d: %s" % (
                p.returncode, p.stderr.strip()[-300:])}
            continue
        out[key] = json.loads(p.stdout.strip().splitlines()[-1])
    return out


def pass_plan(L):
    """Levels emitted by each build pass, as the library plans them: with
    octal group levels at 0 and 3 and at most four levels below level 3
    (L = 6 or 8) a first pass of levels 1-3 and one of the rest (its level-3
    order feeds octal level 3); else the L - 1 levels below level 0 in
    ceil((L - 1) / 4) passes of near-equal size."""
    levels = L - 1
    if levels <= 0:
        return []
    if L in (6, 8):
        return [3, L - 4]
    np_ = (levels + 3) // 4
    return [levels // np_ + (1 if i < levels % np_ else 0) for i in range(np_)]


def pass_bytes_per_launch(n, L):
    """Algorithmic HBM bytes of one pass launch over n uint8 symbols, averaged
    over the passes: read the level order (n), write k levels of bits
    (k * n / 8) and, unless it is the last pass, the next level order (n)."""
    plan = pass_plan(L)
    if not plan:
        return 0.0
    total, a = 0.0, 0
    for k in plan:
        b = a + k
        total += n + k * n / 8.0 + (n if b < L - 1 else 0.0)
        a = b
    return total / len(plan)


def bench_multi_text(torch, E, dev, gen, seed=7):
    """256 uint8 texts, lengths log-uniform in [2^16, 2^26], sigma per text
    from {4, 16, 64, 256}, device-resident: batched build vs one build per
    text, then 2^24 mixed queries (text chosen in proportion to its length)
    in one multi-tree launch vs one launch per text."""
    import ctypes
    rng = np.random.default_rng(seed)
    T = 256
    lens = np.floor(np.exp(rng.uniform(np.log(2 ** 16), np.log(2 ** 26), T))).astype(np.int64)
    sig = rng.choice([4, 16, 64, 256], T)
    texts = [torch.randint(0, int(s_), (int(n_),), dtype=torch.uint8, device=dev,
                           generator=gen) for n_, s_ in zip(lens, sig)]
    alph = [np.arange(int(s_)) for s_ in sig]
    total = int(lens.sum())
    torch.cuda.synchronize()
    # warm-up: the library pool grows to hold every tree of the batch once
    # (as the single-text bench's warm-up builds grow it before timing)
    for t in E.build_batch(texts, alph):
        t.close()
    a = time.perf_counter()
    plain = [E.WaveletTree(t, al) for t, al in zip(texts, alph)]
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - a
    for t in plain:
        t.close()
    a = time.perf_counter()
    trees = E.build_batch(texts, alph)
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - a
    # 2^24 mixed queries, 40/40/20, text in proportion to its length
    m = 1 << 24
    tree_of = rng.choice(T, m, p=lens / lens.sum()).astype(np.uint32)
    ty = rng.choice(3, m, p=[0.4, 0.4, 0.2]).astype(np.uint8)
    n_t = lens[tree_of]
    s_t = sig[tree_of]
    u = rng.random(m)
    c = (rng.random(m) * s_t).astype(np.int64)
    occ = np.zeros((T, 256), np.int64)
    for i, t in enumerate(trees):
        cnt = t.export("COUNTS").astype(np.int64)
        occ[i, :sig[i]] = np.diff(np.append(cnt, lens[i]))
    k = 1 + (u * np.maximum(occ[tree_of, c], 1)).astype(np.int64)
    index = np.where(ty == 0, (u * n_t).astype(np.int64),
                     np.where(ty == 1, (u * (n_t + 1)).astype(np.int64), k))
    rec = np.zeros(m, dtype=trees[0].qdtype)
    rec["index"] = index
    rec["symbol"] = c
    d_tree = torch.from_numpy(tree_of.view(np.int32)).to(dev)
    d_ty = torch.from_numpy(ty).to(dev)
    d_q = torch.from_numpy(rec.view(np.uint8)).to(dev)
    d_out = torch.empty(m, dtype=torch.int64, device=dev)
    d_err = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    hp = (ctypes.c_void_p * T)(*[t.handle for t in trees])
    L = E.lib()

    def multi():
        st = L.ewt_mixed_multi_device(hp, T, d_tree.data_ptr(), d_ty.data_ptr(),
                                      d_q.data_ptr(), m, d_out.data_ptr(),
                                      d_err.data_ptr(), stream.cuda_stream)
        assert st == 0

    # the same queries grouped per text for the plain per-text launches
    order = np.argsort(tree_of, kind="stable")
    bounds = np.searchsorted(tree_of[order], np.arange(T + 1))
    g_ty = torch.from_numpy(ty[order]).to(dev)
    g_q = torch.from_numpy(rec[order].view(np.uint8)).to(dev)
    g_out = torch.empty(m, dtype=torch.int64, device=dev)

    def per_text():
        for i, t in enumerate(trees):
            b0, b1 = int(bounds[i]), int(bounds[i + 1])
            if b1 > b0:
                t.mixed_device(g_ty.data_ptr() + b0, g_q.data_ptr() + 16 * b0,
                               b1 - b0, g_out.data_ptr() + 8 * b0,
                               stream.cuda_stream)

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    multi_ms = timed(multi)
    assert int(d_err.item()) == 0
    plain_ms = timed(per_text)
    # both forms answer identically
    assert torch.equal(d_out[torch.from_numpy(order).to(dev)], g_out)
    for t in trees:
        t.close()
    return {"texts": T, "symbols": total,
            "batched_build_ms": batch_s * 1e3,
            "per_text_build_ms": plain_s * 1e3,
            "batched_build_GB_s": total / batch_s / 1e9,
            "per_text_build_GB_s": total / plain_s / 1e9,
            "queries": m,
            "multi_tree_Mq_s": m / multi_ms / 1e3,
            "per_text_launches_Mq_s": m / plain_ms / 1e3,
            "multi_over_per_text": plain_ms / multi_ms}


def bench_serving(torch, E, dev, gen, big_text):
    """A 6*2^30-symbol sigma-256 index plus 64 sigma-4 texts of 2^26 symbols
    resident; Poisson arrivals of requests of log-uniform 1..2^16 mixed
    queries (40/40/20) at swept rates, served by the engine (continuous
    batching) and, at the lower rates, by the plain per-request path; build
    requests of 2^24-symbol texts arrive every 0.25 s at one rate."""
    from ecl_wavelet_gb300.serving import Server
    big = E.WaveletTree(big_text, np.arange(256))
    small_texts = [torch.randint(0, 4, (1 << 26,), dtype=torch.uint8, device=dev,
                                 generator=gen) for _ in range(64)]
    smalls = E.build_batch(small_texts, [np.arange(4)] * 64)
    srv = Server(batch_queries=1 << 20, batch_requests=1 << 12, inflight=3,
                 memory_budget=200 << 30, elem_size=1)
    srv.add_tree(big)
    for t in smalls:
        srv.add_tree(t)
    srv.run_load(rate=2000, duration_s=0.3, num_trees=65, seed=99)  # warm-up
    srv.run_load(rate=2000, duration_s=0.3, num_trees=65, seed=99, plain=True)
    out = []
    for rate in (1000, 4000, 16000, 64000, 256000):
        e = {"rate_rps": rate,
             "engine": srv.run_load(rate=rate, duration_s=1.0, num_trees=65,
                                    seed=rate,
                                    build_n=(1 << 24) if rate == 16000 else 0,
                                    build_interval_s=0.25)}
        if rate <= 16000:
            e["plain"] = srv.run_load(rate=rate, duration_s=0.5, num_trees=65,
                                      seed=rate, plain=True)
        out.append(e)
    srv.close()
    big.close()
    for t in smalls:
        t.close()
    return {"resident": "1 x 6*2^30 sigma-256 + 64 x 2^26 sigma-4 (uint8)",
            "request_sizes": "log-uniform 1..65536, 40/40/20 access/rank/select",
            "server": {"batch_queries": 1 << 20, "inflight": 3},
            "sweep": out}


def bench_rank_select(torch, E, dev, seed=11):
    """Standalone RankSelect (ecl::RankSelect): one 2^32-bit array of iid
    bits; build from device words and 2^26 rank and select queries (host
    buffers, answered in place) on the GPU, next to the CPU restatement
    (popcount rank / sampled select, one query per iteration on all host
    cores) on 2^24 queries of the same array."""
    import ctypes
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    bits = 1 << 32
    words = rng.integers(0, 1 << 32, bits // 32, dtype=np.uint64).astype(np.uint32)
    d_words = torch.from_numpy(words.view(np.int32)).to(dev)
    bits_arr = np.array([bits], dtype=np.uint64)
    L = E.lib()

    def gpu_build():
        h = ctypes.c_void_p()
        st = L.ewt_rs_build(ctypes.c_void_p(d_words.data_ptr()),
                            bits_arr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                            1, 0, ctypes.byref(h))
        assert st == 0
        return h

    L.ewt_rs_free(gpu_build())
    torch.cuda.synchronize()
    a = time.perf_counter()
    h = gpu_build()
    build_s = time.perf_counter() - a
    rs = E.RankSelect.__new__(E.RankSelect)
    rs._h, rs.bits = h, bits_arr
    ones = int(rs.export("TOTAL_ONES")[0])
    m = 1 << 26
    pos = rng.integers(0, bits + 1, m, dtype=np.uint64)
    ks = rng.integers(1, ones + 1, m, dtype=np.uint64)
    # result buffers written once before timing (allocation, not queries)
    r_gpu = np.zeros(m, dtype=np.uint64)
    s_gpu = np.zeros(m, dtype=np.uint64)
    rs.rank(0, 1, pos, out=r_gpu)
    rs.select(0, 1, ks, out=s_gpu)

    def best_of(fn, reps=3):  # host wall clock: keep the fastest of a few calls
        best = float("inf")
        for _ in range(reps):
            a = time.perf_counter()
            fn()
            best = min(best, time.perf_counter() - a)
        return best

    rank_s = best_of(lambda: rs.rank(0, 1, pos, out=r_gpu))
    sel_s = best_of(lambda: rs.select(0, 1, ks, out=s_gpu))
    # the same call into a freshly allocated result array (the library
    # populates its pages before the GPU writes them)
    a = time.perf_counter()
    fresh = rs.rank(0, 1, pos)
    fresh_s = time.perf_counter() - a
    assert np.array_equal(fresh, r_gpu)
    rs.close()
    a = time.perf_counter()
    ors = O.OracleRS([words], [bits])
    cpu_build_s = time.perf_counter() - a
    mc = 1 << 24
    a = time.perf_counter()
    r_cpu = ors.rank_batch(0, pos[:mc], 1)
    cpu_rank_s = time.perf_counter() - a
    a = time.perf_counter()
    s_cpu = ors.select_batch(0, ks[:mc], 1)
    cpu_sel_s = time.perf_counter() - a
    assert np.array_equal(r_gpu[:mc], r_cpu) and np.array_equal(s_gpu[:mc], s_cpu)
    cores = int(O.lib().ewto_max_threads())
    return {"bits": bits, "queries": m,
            "gpu_build_GB_s": bits / 8 / build_s / 1e9,
            "gpu_rank_Mq_s": m / rank_s / 1e6, "gpu_select_Mq_s": m / sel_s / 1e6,
            "gpu_rank_fresh_output_Mq_s": m / fresh_s / 1e6,
            "cpu_cores": cores, "cpu_build_GB_s": bits / 8 / cpu_build_s / 1e9,
            "cpu_rank_Mq_s": mc / cpu_rank_s / 1e6,
            "cpu_select_Mq_s": mc / cpu_sel_s / 1e6,
            "rank_gpu_over_cpu": (m / rank_s) / (mc / cpu_rank_s),
            "select_gpu_over_cpu": (m / sel_s) / (mc / cpu_sel_s)}


def bench_large_alphabet(torch, E, dev, gen, n=3 * GIB, m=1 << 26):
    """Uint16 texts of 3*2^30 symbols (device-resident): sigma = 65536 with
    Zipf(1.1) symbols and sigma = 1024 uniform.  Each is built once timed,
    then answers 2^26 mixed queries (40/40/20, types interleaved) as plain
    per-type launches, as one batched launch, both again after the library
    autotuned the launch shapes, and as a CUDA graph replay of the tuned
    batched launch."""
    import ctypes
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    L = E.lib()
    res = {}

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for sigma, zipf in ((65536, 1.1), (1024, None)):
        text = torch.empty(n, dtype=torch.int16, device=dev)
        chunk = 1 << 27
        if zipf is None:
            for a in range(0, n, chunk):
                b = min(n, a + chunk)
                text[a:b] = torch.randint(0, sigma, (b - a,), device=dev,
                                          generator=gen).to(torch.int16)
        else:
            w = 1.0 / torch.arange(1, sigma + 1, device=dev,
                                   dtype=torch.float64) ** zipf
            cdf = torch.cumsum(w, 0) / w.sum()
            for a in range(0, n, chunk):
                b = min(n, a + chunk)
                u = torch.rand(b - a, device=dev, dtype=torch.float64,
                               generator=gen)
                ids = torch.searchsorted(cdf, u).clamp_(max=sigma - 1)
                text[a:b] = ids.to(torch.int32).to(torch.int16)  # low 16 bits
            del w, cdf, u, ids
        alph = np.arange(sigma, dtype=np.uint16)

        def build():
            h = ctypes.c_void_p()
            st = L.ewt_build(text.data_ptr(), n, 2, alph.ctypes.data, sigma, 0,
                             ctypes.byref(h))
            assert st == 0, st
            return E.WaveletTree(None, _handle=h.value)

        build().close()
        torch.cuda.synchronize()
        a = time.perf_counter()
        tree = build()
        torch.cuda.synchronize()
        build_s = time.perf_counter() - a
        types, rec = make_mixed_queries(torch, tree, n, sigma, m, gen)
        out = torch.empty(m, dtype=torch.int64, device=dev)
        sel = {t: torch.nonzero(types == t).squeeze(1) for t in (0, 1, 2)}
        acc_idx = rec[sel[0], 0].contiguous()
        rq = rec[sel[1]].contiguous()
        sq = rec[sel[2]].contiguous()
        o_acc = torch.empty(acc_idx.numel(), dtype=torch.int16, device=dev)
        o_r = torch.empty(rq.shape[0], dtype=torch.int64, device=dev)
        o_s = torch.empty(sq.shape[0], dtype=torch.int64, device=dev)

        def mixed():
            tree.mixed_device(types.data_ptr(), rec.data_ptr(), m,
                              out.data_ptr(), sptr)

        def plain():
            return (timed(lambda: tree.access_device(
                        acc_idx.data_ptr(), acc_idx.numel(), o_acc.data_ptr(), sptr))
                    + timed(lambda: tree.rank_device(
                        rq.data_ptr(), rq.shape[0], o_r.data_ptr(), sptr))
                    + timed(lambda: tree.select_device(
                        sq.data_ptr(), sq.shape[0], o_s.data_ptr(), sptr)))

        mixed_ms = timed(mixed)
        E.set_work_queue(False)
        static_ms = timed(mixed)
        E.set_work_queue(True)
        plain_ms = plain()
        assert tree.query_status(sptr) == 0
        want = out.clone()
        tuning = tree.autotune(1 << 22)
        tuned_mixed_ms = timed(mixed)
        tuned_plain_ms = plain()
        assert tree.query_status(sptr) == 0
        assert torch.equal(out, want)  # the launch shape changes no answer
        # the tuned batched launch captured once, replayed
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            tree.mixed_device(types.data_ptr(), rec.data_ptr(), m,
                              out.data_ptr(), side.cuda_stream)
        out.zero_()
        graph_ms = timed(graph.replay)
        assert tree.query_status(sptr) == 0
        assert torch.equal(out, want)
        key = "sigma%d_%s" % (sigma, "zipf1.1" if zipf else "uniform")
        res[key] = {
            "n": n, "sigma": sigma, "levels": int(tree.info.levels),
            "build_GB_s": 2 * n / build_s / 1e9, "build_ms": build_s * 1e3,
            "queries": m,
            "batched_mixed_Mq_s": m / mixed_ms / 1e3,
            "batched_mixed_static_stride_Mq_s": m / static_ms / 1e3,
            "plain_per_type_Mq_s": m / plain_ms / 1e3,
            "autotuned": {"shapes": {k: [v["threads"], v["blocks_per_sm"]]
                                     for k, v in tuning.items() if k in KINDS},
                          "select_sample_rate": tuning["select_sample_rate"],
                          "batched_mixed_Mq_s": m / tuned_mixed_ms / 1e3,
                          "plain_per_type_Mq_s": m / tuned_plain_ms / 1e3,
                          "graph_replay_mixed_Mq_s": m / graph_ms / 1e3},
        }
        del graph, out, want, types, rec, acc_idx, rq, sq, o_acc, o_r, o_s, sel
        tree.close()
        del text
        torch.cuda.empty_cache()
    return res


def make_mixed_queries(torch, tree, n, sigma, m, gen):
    """Device-resident mixed batch: types 40/40/20, RankSelectQuery records."""
    dev = "cuda"
    u = torch.rand(m, device=dev, generator=gen)
    types = torch.where(u < 0.4, 0, torch.where(u < 0.8, 1, 2)).to(torch.uint8)
    counts = torch.from_numpy(tree.export("COUNTS").astype(np.int64)).to(dev)
    occ = torch.diff(torch.cat([counts, torch.tensor([n], device=dev)]))
    sym = torch.randint(0, sigma, (m,), device=dev, generator=gen)
    acc_idx = torch.randint(0, n, (m,), device=dev, generator=gen)
    rank_idx = torch.randint(0, n + 1, (m,), device=dev, generator=gen)
    k = (torch.rand(m, device=dev, generator=gen, dtype=torch.float64)
         * occ[sym].to(torch.float64)).to(torch.int64) + 1
    index = torch.where(types == 0, acc_idx, torch.where(types == 1, rank_idx, k))
    rec = torch.zeros((m, 2), dtype=torch.int64, device=dev)
    rec[:, 0] = index
    rec[:, 1] = sym  # symbol in the low byte(s) of the second word
    return types, rec


def run_ours(args, world, rank, local):
    import torch
    import ecl_wavelet_gb300 as E
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    E.build()
    dev = torch.device("cuda", local)
    n, sigma = args.n, args.sigma
    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    text = torch.randint(0, sigma, (n,), dtype=torch.uint8, device=dev,
                         generator=gen)
    alphabet = np.arange(sigma)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    if args.only in ("multi", "serve", "rs", "large"):
        if args.only == "multi":
            key, part = "many_texts", bench_multi_text(torch, E, dev, gen)
        elif args.only == "serve":
            key, part = "serving", bench_serving(torch, E, dev, gen, text)
        elif args.only == "large":
            del text
            key, part = "large_alphabet_u16", bench_large_alphabet(torch, E, dev, gen)
        else:
            key, part = "rank_select", bench_rank_select(torch, E, dev)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "partial": args.only, key: part}))
        return
    for _ in range(args.warmup):
        E.WaveletTree(text, alphabet, gpu_index=local).close()
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    E.set_timing(True)
    E.get_timing(reset=True)
    launches0 = E.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    tree = None
    ev0.record(stream)
    for s in range(args.steps):
        if tree is not None:
            tree.close()
        tree = E.WaveletTree(text, alphabet, gpu_index=local)
    ev1.record(stream)
    barrier()
    step_ms = ev0.elapsed_time(ev1) / args.steps
    launches = E.launch_count() - launches0
    phases = E.get_timing(reset=True)
    E.set_timing(False)
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([step_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
    value = world * n / (step_ms / 1e3) / 1e9

    # ---- roofline of the dominant build kernel -----------------------------
    peak, peak_kind = measured_peaks()
    build_phases = {k: v for k, v in phases.items() if k not in ("query", "h2d")}
    dom = max(build_phases, key=lambda k: build_phases[k][0])
    dom_ms, dom_launches = build_phases[dom]
    L = int(tree.getNumLevels())
    per_launch_bytes = {
        # split: the multi-level passes (power-of-two alphabet, uint8)
        "split": pass_bytes_per_launch(n, L),
        # fill: read the level order, write one bit per symbol
        "fill": n + n / 8.0,
        # rank/select counts: read one level's bits, write L2 + L1
        "rs_counts": n / 8.0 + 2.0 * n / 512 + 8.0 * n / 65536,
        # digit counts of each pass: read the level order
        "hist": float(n),
        "samples": 2.0 * L * n / 512 + 16.0 * L * n / 4096,
        "node_ranks": 0.0,
    }
    achieved = (per_launch_bytes.get(dom, 0.0)
                / (dom_ms / max(dom_launches, 1) / 1e3) / 1e9)
    traffic = None
    prof = os.path.join(REPO, "profiles", "traffic_per_symbol.json")
    if os.path.exists(prof):
        try:
            tp = json.load(open(prof))
            if dom in tp:
                traffic = tp[dom] * n
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": per_launch_bytes.get(dom)}
    compulsory = n + L * n / 8.0 + L * n * (8 / 65536 + 2 / 512 + 16 / 4096)
    build = {"phases_ms_per_step": {k: v[0] / args.steps for k, v in
                                    phases.items() if v[1]},
             "compulsory_GB": compulsory / 1e9,
             "compulsory_frac_of_peak": (compulsory / (step_ms / 1e3) / 1e9)
             / peak}

    queries, e2e, sweep, cpu = {}, None, {}, None
    if args.only == "build":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "GB/s",
                              "ms_per_step": step_ms, "roofline": roofline,
                              "build": build, "partial": "build only"}))
        return
    # ---- queries on the last tree -----------------------------------------
    m = args.queries
    qgen = torch.Generator(device=dev).manual_seed(77 + rank)
    types, rec = make_mixed_queries(torch, tree, n, sigma, m, qgen)
    out = torch.empty(m, dtype=torch.int64, device=dev)
    sptr = stream.cuda_stream

    def timed(fn, reps=3):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    mixed_ms = timed(lambda: tree.mixed_device(types.data_ptr(), rec.data_ptr(),
                                               m, out.data_ptr(), sptr))
    assert tree.query_status(sptr) == 0
    E.set_work_queue(False)  # the same launch with fixed-stride chunks
    static_mixed_ms = timed(lambda: tree.mixed_device(
        types.data_ptr(), rec.data_ptr(), m, out.data_ptr(), sptr))
    E.set_work_queue(True)
    assert tree.query_status(sptr) == 0
    # plain per-type calls over the same queries
    sel = {t: torch.nonzero(types == t).squeeze(1) for t in (0, 1, 2)}
    acc_idx = rec[sel[0], 0].contiguous()
    rq = rec[sel[1]].contiguous()
    sq = rec[sel[2]].contiguous()
    o_acc = torch.empty(acc_idx.numel(), dtype=torch.uint8, device=dev)
    o_r = torch.empty(rq.shape[0], dtype=torch.int64, device=dev)
    o_s = torch.empty(sq.shape[0], dtype=torch.int64, device=dev)
    acc_ms = timed(lambda: tree.access_device(acc_idx.data_ptr(),
                                              acc_idx.numel(),
                                              o_acc.data_ptr(), sptr))
    rank_ms = timed(lambda: tree.rank_device(rq.data_ptr(), rq.shape[0],
                                             o_r.data_ptr(), sptr))
    sel_ms = timed(lambda: tree.select_device(sq.data_ptr(), sq.shape[0],
                                              o_s.data_ptr(), sptr))
    assert tree.query_status(sptr) == 0
    plain_ms = acc_ms + rank_ms + sel_ms
    # end to end through the host API (pinned host buffers, copies inside)
    h_types = types.cpu().pin_memory().numpy()
    h_rec = rec.cpu().pin_memory().numpy().view(tree.qdtype).reshape(-1)
    h_out = torch.empty(m, dtype=torch.int64).pin_memory().numpy().view(
        np.uint64)
    import ctypes
    L_ = E.lib()

    def host_mixed():
        st = L_.ewt_mixed(tree.handle, h_types.ctypes.data, h_rec.ctypes.data,
                          m, h_out.ctypes.data)
        assert st == 0

    e2e_q_ms = timed(host_mixed, reps=2)
    # the plain per-call host form (the reference's host access / rank /
    # select batch calls): one call per type from pinned host buffers
    h_acc = acc_idx.cpu().pin_memory().numpy().view(np.uint64)
    h_rq = rq.cpu().pin_memory().numpy().view(tree.qdtype).reshape(-1)
    h_sq = sq.cpu().pin_memory().numpy().view(tree.qdtype).reshape(-1)
    h_oa = torch.empty(h_acc.size, dtype=torch.uint8).pin_memory().numpy()
    h_or = torch.empty(h_rq.size, dtype=torch.int64).pin_memory().numpy()
    h_os = torch.empty(h_sq.size, dtype=torch.int64).pin_memory().numpy()

    def host_plain():
        assert L_.ewt_access(tree.handle, h_acc.ctypes.data, h_acc.size,
                             h_oa.ctypes.data) == 0
        assert L_.ewt_rank(tree.handle, h_rq.ctypes.data, h_rq.size,
                           h_or.ctypes.data) == 0
        assert L_.ewt_select(tree.handle, h_sq.ctypes.data, h_sq.size,
                             h_os.ctypes.data) == 0

    host_plain_ms = timed(host_plain, reps=2)
    del h_acc, h_rq, h_sq, h_oa, h_or, h_os
    # launch shapes picked by the library's autotuner, then the same calls
    tuning = tree.autotune(1 << 22)
    tuned_mixed_ms = timed(lambda: tree.mixed_device(
        types.data_ptr(), rec.data_ptr(), m, out.data_ptr(), sptr))
    tuned_plain_ms = (
        timed(lambda: tree.access_device(acc_idx.data_ptr(), acc_idx.numel(),
                                         o_acc.data_ptr(), sptr))
        + timed(lambda: tree.rank_device(rq.data_ptr(), rq.shape[0],
                                         o_r.data_ptr(), sptr))
        + timed(lambda: tree.select_device(sq.data_ptr(), sq.shape[0],
                                           o_s.data_ptr(), sptr)))
    assert tree.query_status(sptr) == 0
    # random-access roofline: dependent random 32-byte reads per second
    probe = E.probe_random_reads(8 * GIB, 4, 1 << 25, local)
    L_ = int(tree.info.levels)
    steps = group_levels(L_)
    reads = {"access": steps, "rank": steps, "select": 2 * steps}
    reads["mixed"] = 0.4 * reads["access"] + 0.4 * reads["rank"] + 0.2 * reads["select"]
    rates = {"access": acc_idx.numel() / acc_ms / 1e3 * 1e6,
             "rank": rq.shape[0] / rank_ms / 1e3 * 1e6,
             "select": sq.shape[0] / sel_ms / 1e3 * 1e6,
             "mixed": m / mixed_ms / 1e3 * 1e6}
    rroof = {"probe_reads_per_s": probe,
             "model": "block reads per query: one per group level (octal or "
                      "quad) for access and rank, a sample and a block per level "
                      "for select (a lower bound: wide brackets read more)",
             "reads_per_query": reads,
             "frac": {k: rates[k] * reads[k] / probe for k in reads}}
    queries = {
        "random_read_roofline": rroof,
        "autotuned": {"shapes": {k: [v["threads"], v["blocks_per_sm"]]
                                 for k, v in tuning.items() if k in KINDS},
                      "select_sample_rate": tuning["select_sample_rate"],
                      "batched_mixed_Mq_s": m / tuned_mixed_ms / 1e3,
                      "plain_per_type_Mq_s": m / tuned_plain_ms / 1e3},
        "n_queries": m, "mix": "40/40/20 access/rank/select, interleaved",
        "batched_mixed_Mq_s": m / mixed_ms / 1e3,
        "batched_mixed_static_stride_Mq_s": m / static_mixed_ms / 1e3,
        "plain_per_type_Mq_s": m / plain_ms / 1e3,
        "batched_over_plain": plain_ms / mixed_ms,
        "access_Mq_s": acc_idx.numel() / acc_ms / 1e3,
        "rank_Mq_s": rq.shape[0] / rank_ms / 1e3,
        "select_Mq_s": sq.shape[0] / sel_ms / 1e3,
        "e2e_mixed_host_Mq_s": m / e2e_q_ms / 1e3,
        "plain_host_per_type_Mq_s": m / host_plain_ms / 1e3,
        "batched_host_over_plain_host": host_plain_ms / e2e_q_ms,
        "ms": {"mixed": mixed_ms, "access": acc_ms, "rank": rank_ms,
               "select": sel_ms, "e2e_mixed": e2e_q_ms,
               "plain_host_per_type": host_plain_ms},
    }
    del out, o_acc, o_r, o_s, rq, sq, acc_idx, rec, types
    if args.only == "queries":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value,
                              "queries": queries, "partial": "build+queries"}))
        return

    # ---- end-to-end build from pinned host memory --------------------------
    h_text = torch.empty(n, dtype=torch.uint8).pin_memory()
    h_text.copy_(text)
    h_np = h_text.numpy()
    tree.close()
    tree = None
    for _ in range(max(args.warmup, 3)):  # warm-up: pool and page tables
        E.WaveletTree(h_np, alphabet, gpu_index=local).close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        tr = E.WaveletTree(h_np, alphabet, gpu_index=local)
        ones = tr.export("TOTAL_ONES")  # result read back to the host
        tr.close()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    e2e = {"value": world * n / (e2e_ms / 1e3) / 1e9, "unit": "GB/s",
           "h2d_bytes_per_step": n, "d2h_bytes_per_step": int(ones.nbytes),
           "ms_per_step": e2e_ms,
           "queries_Mq_s": queries["e2e_mixed_host_Mq_s"],
           "queries_h2d_bytes": m * 17, "queries_d2h_bytes": m * 8}
    del h_text, h_np
    cpu_text = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu_text = text[:min(args.cpu_sample, n)].cpu().numpy()

    # ---- sigma sweep -------------------------------------------------------
    if not args.no_sweep:
        for s in (4, 16, 64, 256):
            if s == sigma:
                sweep[str(s)] = value / world
                continue
            t2 = torch.randint(0, s, (n,), dtype=torch.uint8, device=dev,
                               generator=gen)
            E.WaveletTree(t2, np.arange(s), gpu_index=local).close()
            torch.cuda.synchronize()
            a = time.perf_counter()
            E.WaveletTree(t2, np.arange(s), gpu_index=local).close()
            torch.cuda.synchronize()
            sweep[str(s)] = n / (time.perf_counter() - a) / 1e9
            del t2

    # ---- many texts and serving (one GPU's share) --------------------------
    multi = serve = None
    if not args.no_multi:
        multi = bench_multi_text(torch, E, dev, gen)
    if not args.no_serve:
        serve = bench_serving(torch, E, dev, gen, text)
    rsel = None
    if not args.no_rs and rank == 0 and world == 1:
        rsel = bench_rank_select(torch, E, dev)
    large = None
    if not args.no_large:
        del text
        torch.cuda.empty_cache()
        large = bench_large_alphabet(torch, E, dev, gen)

    # ---- the reference's own GPU build on this GPU (rank 0, N = 1) ---------
    ref_gpu = None
    if rank == 0 and world == 1 and not args.no_ref_gpu:
        torch.cuda.empty_cache()
        ref_gpu = reference_gpu(n, sigma, m)

    # ---- CPU baseline (rank 0, N = 1 only) ---------------------------------
    if rank == 0 and world == 1 and not args.no_cpu:
        sample = min(args.cpu_sample, n)
        r = cpu_tree_baseline(sigma, sample, text=cpu_text)
        del cpu_text
        cpu = {"value": r["build_GB_s"], "unit": "GB/s", "cores": r["cores"],
               "kind": "port",
               "sample": "%d uint8 symbols, sigma=%d: one full build of the "
                         "reference's structure by the multithreaded CPU tree "
                         "on all host cores, then 2^22 mixed queries walked "
                         "one per loop iteration" % (sample, sigma),
               "mixed_queries_Mq_s": r["mixed_queries_Mq_s"],
               "access_Mq_s": r["access_Mq_s"], "rank_Mq_s": r["rank_Mq_s"],
               "select_Mq_s": r["select_Mq_s"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic: iid uniform uint8 text (torch seed %d), "
                    "device-resident" % 1234,
            "config": {"workload": "wavelet-tree build of a 6*2^30-symbol "
                                   "uint8 text, sigma=%d, + %d mixed queries"
                                   % (sigma, m),
                       "n": n, "sigma": sigma,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (6 GiB text)"},
            "gpu_launches": launches,
            "roofline": roofline, "build": build, "queries": queries,
            "sigma_sweep_GB_s": sweep, "e2e": e2e, "cpu_baseline": cpu,
            "reference_gpu": ref_gpu,
            "many_texts": multi, "serving": serve, "rank_select": rsel,
            "large_alphabet_u16": large,
            "clocks": clk,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
