"""Host logic of the serving loop (mflib_gb300/serving.py) with a fake
executor: admission under the memory budget, eviction, FIFO order,
concurrency of the worker slots, errors and statistics.  No GPU."""
import threading
import time

import numpy as np
import pytest

from mflib_gb300.serving import DetectionRequest, Server, TemplateBank, latency_stats


class FakeExecutor:
    """Objects of a fixed size per bank; run() sleeps and records overlap."""

    def __init__(self, size=100, delay=0.02):
        self.size, self.delay = size, delay
        self.lock = threading.Lock()
        self.active = self.max_active = 0
        self.alive = set()
        self.order = []

    def estimate_bytes(self, bank, n):
        return self.size * len(bank)

    def create(self, bank, n):
        obj = object()
        with self.lock:
            self.alive.add(id(obj))
        return obj

    def device_bytes(self, obj):
        return self.size * 1

    def run(self, obj, bank, req):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)
            self.order.append(req.id)
        time.sleep(self.delay)
        req.peaks = [np.zeros(0, np.int32)] * len(bank)
        req.lags = len(bank) * bank.valid_lags(req.n)
        with self.lock:
            self.active -= 1

    def destroy(self, obj):
        with self.lock:
            self.alive.discard(id(obj))


def banks():
    return [TemplateBank("a", [np.ones(100)]), TemplateBank("b", [np.ones(200)]), TemplateBank("c", [np.ones(300)])]


def req(bank, n=5000, c=2):
    return DetectionRequest(bank, np.zeros((c, n), np.float32))


def test_budget_and_eviction():
    ex = FakeExecutor(size=100)
    srv = Server(banks(), ex, memory_budget=250, slots=4, buckets=(6000, 12000)).start()
    rs = [srv.submit(req("abc"[i % 3], n=5000 if i % 2 else 9000)) for i in range(30)]
    for r in rs:
        r.wait(10)
    srv.close()
    assert srv.peak_held <= 250
    assert srv.evicted > 0
    assert len(srv.served) == 30 and all(r.error is None for r in rs)
    assert not ex.alive  # close() released every object


def test_fifo_with_one_slot():
    ex = FakeExecutor(delay=0.0)
    srv = Server(banks(), ex, slots=1).start()
    rs = [srv.submit(req("a")) for _ in range(10)]
    for r in rs:
        r.wait(10)
    srv.close()
    assert ex.order == [r.id for r in rs]


def test_slots_overlap():
    ex = FakeExecutor(delay=0.05)
    srv = Server(banks(), ex, slots=4).start()
    t0 = time.perf_counter()
    rs = [srv.submit(req("a")) for _ in range(8)]
    for r in rs:
        r.wait(10)
    el = time.perf_counter() - t0
    srv.close()
    assert ex.max_active == 4
    assert el < 8 * 0.05


def test_request_over_budget_fails_alone():
    ex = FakeExecutor(size=1000)
    srv = Server(banks(), ex, memory_budget=500, slots=2).start()
    bad, good = srv.submit(req("a")), None
    with pytest.raises(MemoryError):
        bad.wait(10)
    srv.close()
    ex2 = FakeExecutor(size=100)
    srv2 = Server(banks(), ex2, memory_budget=500, slots=2).start()
    good = srv2.submit(req("a")).wait(10)
    srv2.close()
    assert good.error is None


def test_validation_and_buckets():
    srv = Server(banks(), FakeExecutor(), buckets=(100, 1000))
    assert srv.bucket(1) == 100 and srv.bucket(100) == 100 and srv.bucket(101) == 1000
    with pytest.raises(ValueError):
        srv.bucket(1001)
    with pytest.raises(ValueError):
        srv.submit(req("zzz"))
    with pytest.raises(ValueError):
        DetectionRequest("a", np.zeros((65, 10)))
    with pytest.raises(ValueError):
        TemplateBank("x", [np.ones(10)], channel_slots=[64])


class FakeRing:
    """Stands in for a SignalRing (channel count and head only)."""

    def __init__(self, n_channels=8, head=5000):
        self.n_channels, self.head = n_channels, head


def test_ring_window_requests():
    ring = FakeRing()
    r = DetectionRequest("a", ring=ring, channels=[2, 5, 7], n=1200)
    assert r.channels == 3 and r.n == 1200 and r.end == 5000 and r.signals is None
    r = DetectionRequest("a", ring=ring, n=300, end=4000)
    assert r.channels == 8 and r.end == 4000
    with pytest.raises(ValueError):
        DetectionRequest("a", np.zeros((2, 10)), ring=ring, n=10)
    with pytest.raises(ValueError):
        DetectionRequest("a", ring=ring, channels=[8], n=10)
    with pytest.raises(ValueError):
        DetectionRequest("a", ring=ring, channels=[0])
    with pytest.raises(ValueError):
        DetectionRequest("a", ring=FakeRing(n_channels=100), n=10)
    # the server buckets and admits a ring request like any other
    ex = FakeExecutor()
    srv = Server(banks(), ex, slots=1).start()
    done = srv.submit(DetectionRequest("a", ring=ring, channels=[1], n=1200)).wait(10)
    srv.close()
    assert done.error is None


def test_latency_stats():
    ex = FakeExecutor(delay=0.01)
    srv = Server(banks(), ex, slots=2).start()
    rs = [srv.submit(req("b", n=1200)) for _ in range(6)]
    for r in rs:
        r.wait(10)
    srv.close()
    st = latency_stats(rs)
    assert st["requests"] == 6
    assert 0 < st["p50_s"] <= st["p99_s"]
    assert st["template_lags"] == 6 * (1200 - 200 + 1)
    assert st["throughput"] > 0


class FailingExecutor(FakeExecutor):
    """run() fails for requests whose signals hold a NaN; destroy() can be
    made to fail."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.destroy_fails = False

    def run(self, obj, bank, req):
        if np.isnan(req.signals).any():
            raise RuntimeError("device error")
        super().run(obj, bank, req)

    def destroy(self, obj):
        super().destroy(obj)
        if self.destroy_fails:
            raise OSError("destroy failed")


def test_failed_request_discards_its_object():
    ex = FailingExecutor(size=100, delay=0.0)
    srv = Server(banks(), ex, memory_budget=1000, slots=1).start()
    bad = req("a")
    bad.signals[0, 0] = np.nan
    rb = srv.submit(bad)
    with pytest.raises(RuntimeError):
        rb.wait(10)
    good = srv.submit(req("a")).wait(10)
    srv.close()
    assert good.error is None
    assert srv.discarded == 1 and srv.created == 2  # the failed object was not reused
    assert not ex.alive


def test_failing_destroy_keeps_no_reservation():
    ex = FailingExecutor(size=100, delay=0.0)
    srv = Server(banks(), ex, memory_budget=150, slots=1).start()
    assert srv.submit(req("a")).wait(10).error is None
    ex.destroy_fails = True  # evicting bank a's idle object for bank b fails
    rb = srv.submit(req("b"))
    with pytest.raises(OSError):
        rb.wait(10)
    ex.destroy_fails = False
    # the budget is whole again: another request is admitted and served
    assert srv.submit(req("c")).wait(10).error is None
    srv.close()
    assert srv._reserved == 0

