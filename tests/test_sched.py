"""The serving engine's scheduling core on the CPU (libewt_sched.so, no GPU):
FIFO admission into batches bounded by queries and requests, cancellation
only before a request is taken, build admission by memory footprint, and
nearest-rank latency percentiles.  Failures are made on the host: refused
requests, a cancelled request, a failed completion."""
import numpy as np
import pytest

from ecl_wavelet_gb300 import buildlib
from ecl_wavelet_gb300.serving import Sched


@pytest.fixture(scope="module", autouse=True)
def _built():
    buildlib.build_sched()


def test_batches_respect_capacity_and_order():
    s = Sched(batch_queries=100, batch_requests=3, budget=1 << 30)
    ids = [s.submit_query(0, m, 0.0) for m in (40, 40, 30, 10, 5, 90)]
    assert all(ids) and ids == sorted(ids)
    assert s.take_batch(1.0) == ids[:2]          # 40 + 40 + 30 > 100
    assert s.take_batch(2.0) == ids[2:5]         # request limit 3
    assert s.take_batch(3.0) == ids[5:]
    assert s.take_batch(4.0) == []
    st = s.stats()
    assert st["batches"] == 3 and st["batched_requests"] == 6
    assert st["queries"] == 215


def test_refused_requests():
    s = Sched(100, 4, 1000)
    assert s.submit_query(0, 0, 0.0) == 0        # empty
    assert s.submit_query(0, 101, 0.0) == 0      # above the batch size
    assert s.submit_build(1001, 0.0) == 0        # above the budget
    with pytest.raises(ValueError):
        Sched(0, 1, 1)


def test_cancel_only_while_pending():
    s = Sched(100, 8, 1 << 20)
    a = s.submit_query(0, 10, 0.0)
    b = s.submit_query(1, 10, 0.0)
    c = s.submit_query(2, 10, 0.0)
    assert s.cancel(b, 0.5)
    assert s.state(b) == 3
    assert not s.cancel(b, 0.6)                  # already cancelled
    assert s.take_batch(1.0) == [a, c]           # the cancelled one is skipped
    assert not s.cancel(a, 1.1)                  # running
    s.complete(a, 0, 2.0)
    s.complete(c, -5, 2.0)                       # a request that failed
    assert s.state(a) == 2 and s.state(c) == 2
    st = s.stats()
    assert st["cancelled"] == 1 and st["completed"] == 2 and st["failed"] == 1
    assert s.state(12345) == -1


def test_build_admission_by_footprint():
    s = Sched(100, 8, budget=1000)
    s.reserve(300)                               # a resident tree
    b1 = s.submit_build(600, 0.0)
    b2 = s.submit_build(500, 0.0)
    b3 = s.submit_build(50, 0.0)
    assert s.take_build(1.0) == b1               # 300 + 600 <= 1000
    assert s.used() == 900
    assert s.take_build(1.0) == b3               # b2 does not fit, b3 does
    assert s.take_build(1.0) == 0
    s.release(600)                               # b1 done: its scratch back
    assert s.take_build(2.0) == b2
    assert s.used() == 300 + 50 + 500


def test_latency_percentiles_nearest_rank():
    s = Sched(1000, 1000, 1 << 20)
    ids = [s.submit_query(0, 1, 0.0) for _ in range(100)]
    s.take_batch(0.0)
    for i, r in enumerate(ids):                  # latencies 1 .. 100 ms
        s.complete(r, 0, (i + 1) / 1000.0)
    st = s.stats()
    assert st["p50_ms"] == pytest.approx(51.0, abs=1.01)
    assert st["p99_ms"] == pytest.approx(99.0, abs=1.01)
    assert st["max_ms"] == pytest.approx(100.0)
    assert st["mean_ms"] == pytest.approx(50.5)


def test_many_requests_fifo_under_random_sizes():
    rng = np.random.default_rng(3)
    s = Sched(1 << 16, 1 << 12, 1 << 30)
    sizes = rng.integers(1, 1 << 12, 5000)
    ids = [s.submit_query(int(i % 7), int(m), 0.0) for i, m in enumerate(sizes)]
    seen = []
    t = 0.0
    while True:
        b = s.take_batch(t)
        if not b:
            break
        assert sum(int(sizes[ids.index(r)]) for r in b) <= 1 << 16
        seen += b
        t += 1
    assert seen == ids
