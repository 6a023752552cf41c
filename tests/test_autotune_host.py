"""Host logic of MatchedFilter.autotune (mflib_gb300/matched_filter.py) on a
fake object whose plans and apply times come from a known cost table: the
coordinate descent over bucket counts, FFT lengths and organisations finds
the cheapest plan, infeasible candidates are recorded and skipped, and the
object ends initialised with the winner, its signals and peak threshold
loaded again.  No GPU."""
import numpy as np
import pytest

from mflib_gb300.matched_filter import MatchedFilter


class _Tpl:
    def __init__(self, n):
        self.n = n

    def get_signal_length(self):
        return self.n


class FakeFilter(MatchedFilter):
    """Bucket b of a k-bucket plan has automatic FFT length 4096 and
    organisation 1; apply time = sum over buckets of cost(k, b, fft,
    variant), plus tc_cost(templates per group) for the tensor-core plan
    (automatic group 8; groups above 12 do not fit).  Plans with fft 2048
    and organisation 2 do not fit."""

    def __init__(self, lens, dtype=np.float32, cost=None):  # no device object
        self._dtype = dtype
        self._templates = [_Tpl(n) for n in lens]
        self._params = object()
        self._init_kw = dict(template_channels=[0] * len(lens), n_channels=1, fft_length=0, correlator_variant=0,
                             length_buckets=0, bucket_plans=None)
        self.cost = cost
        self.tc_cost = lambda g: 0.0
        self.tcg = 0
        self.oom = None        # a plan whose initialize runs out of memory
        self.fail_at = None    # the initialize call that fails hard
        self.calls = 0
        self.loads = 0
        self.thresholds = []
        self.inits = []
        self.kw = None

    def initialize(self, params, **kw):
        k = max(1, kw.get("length_buckets") or 1)
        plans = [(4096, 1)] * k
        for b, (f, v) in enumerate((kw.get("bucket_plans") or [])[:k]):
            plans[b] = (f or plans[b][0], v or plans[b][1])
        tcg = 0
        if kw.get("correlator_variant") == 4:
            plans = [(4096, 4)]
            tcg = kw.get("tc_group") or 8
            if tcg > 12:
                raise ValueError("tc_group does not fit")
        if any(p == (2048, 2) for p in plans):
            raise ValueError("the plan override does not fit")
        if any(p == self.oom for p in plans):
            raise MemoryError("out of device memory")
        self.calls += 1
        if self.fail_at is not None and self.calls == self.fail_at:
            raise OSError("device lost")
        self.inits.append(kw)
        self.kw = kw
        self.plans = plans
        self.tcg = tcg
        self._init_kw = dict(kw)

    def set_channel_signals(self, x, first_channel=0):
        self.loads += 1

    def set_peak_threshold(self, threshold):
        self.thresholds.append(threshold)
        self._peak_thr = threshold

    def apply(self):
        pass

    def synchronize(self):
        pass

    def last_timings(self):
        k = len(self.plans)
        ms = float(sum(self.cost(k, b, f, v) for b, (f, v) in enumerate(self.plans)))
        return {"xcorr_ms": 0.0, "apply_ms": ms + (self.tc_cost(self.tcg) if self.tcg else 0.0)}

    def get_plan(self):
        return {"fft_length": self.plans[-1][0], "correlator": self.plans[-1][1], "tc_group": self.tcg,
                "bucket_plans": [{"fft_length": f, "correlator": v, "templates": 1, "lags_per_block": f // 2}
                                 for f, v in self.plans]}


def test_autotune_finds_cheapest_mixed():
    # two buckets beat one; in the two-bucket plan, bucket 0 is cheapest at
    # (8192, 2) and bucket 1 at (2048, 1)
    def cost(k, b, f, v):
        if k == 1:
            return 10.0 + (f != 4096) + (v != 1)
        best = {0: (8192, 2), 1: (2048, 1)}[b] if k == 2 else (4096, 1)
        return (3.0 if k == 2 else 4.0) + abs(np.log2(f) - np.log2(best[0])) + (v != best[1])

    f = FakeFilter([200, 900, 3000], cost=cost)
    f.set_peak_threshold(0.6)
    res = f.autotune(np.zeros((1, 10), np.float32), repeats=2, max_buckets=3)
    assert res["config"]["length_buckets"] == 2
    assert res["config"]["bucket_plans"] == [(8192, 2), (2048, 1)]
    assert res["apply_ms"] == 6.0
    ok = [t for t in res["trials"] if t["apply_ms"] is not None]
    assert res["apply_ms"] == min(t["apply_ms"] for t in ok)
    # (2048, 2) does not fit: recorded with its error, never timed
    bad = [t for t in res["trials"] if t["apply_ms"] is None]
    assert bad and all("does not fit" in t["error"] for t in bad)
    # FP32 transforms stop at 8192: no 16384 candidate was tried
    assert all(p[0] <= 8192 for t in res["trials"] for p in (t["config"]["bucket_plans"] or []))
    # left on the winner, signals loaded after every successful initialize,
    # the threshold set before tuning applied again each time
    assert f.kw == res["config"] and f.plans == [(8192, 2), (2048, 1)]
    assert f.loads == len(ok) + 1
    assert f.thresholds[-1] == 0.6 and len(f.thresholds) == f.loads + 1
    # mixed lengths: only the whole-CTA organisations are candidates
    assert {p[1] for t in res["trials"] for p in (t["config"]["bucket_plans"] or [])} <= {1, 2}


def test_autotune_one_length_includes_tensor_cores():
    def cost(k, b, f, v):
        return {4: 1.0, 3: 2.0}.get(v, 5.0) + (f != 4096)

    f = FakeFilter([500] * 8, cost=cost)
    res = f.autotune(np.zeros((1, 10), np.float32), repeats=1)
    tried = {p[1] for t in res["trials"] for p in (t["config"]["bucket_plans"] or [])}
    assert tried == {1, 2, 3, 5}
    assert {t["config"]["length_buckets"] for t in res["trials"]} == {1}
    assert res["config"]["correlator_variant"] == 4 and res["apply_ms"] == 1.0
    # FP64: no tensor-core candidate
    g = FakeFilter([500] * 8, dtype=np.float64, cost=cost)
    res = g.autotune(np.zeros((1, 10), np.float64), repeats=1)
    assert all(t["config"]["correlator_variant"] != 4 for t in res["trials"])
    assert res["config"]["bucket_plans"] == [(4096, 3)]


def test_autotune_searches_tensor_core_tile_shape():
    def cost(k, b, f, v):
        return {4: 1.0, 3: 2.0}.get(v, 5.0) + (f != 4096)

    f = FakeFilter([300] * 8, cost=cost)
    f.tc_cost = lambda g: abs(g - 4) * 0.1  # four templates per group is best
    res = f.autotune(np.zeros((1, 10), np.float32), repeats=1)
    assert res["config"]["correlator_variant"] == 4 and res["config"]["tc_group"] == 4
    assert res["plan"]["tc_group"] == 4 and res["apply_ms"] == 1.0
    tc = [t for t in res["trials"] if t["config"]["correlator_variant"] == 4]
    assert [t["config"]["tc_group"] for t in tc] == [0, 2, 4, 6, 8, 12, 16]
    assert tc[-1]["apply_ms"] is None and "does not fit" in tc[-1]["error"]
    # the FFT candidates never carry a tile shape
    assert all(t["config"]["tc_group"] == 0 for t in res["trials"] if t["config"]["correlator_variant"] != 4)


def test_autotune_restrictions_and_errors():
    f = FakeFilter([200, 900], cost=lambda k, b, fl, v: 1.0)
    with pytest.raises(ValueError):
        f.autotune(np.zeros(10, np.float32))
    res = f.autotune(np.zeros((1, 10), np.float32), repeats=1, max_buckets=1, fft_lengths=[4096], variants=[1])
    assert all(t["config"]["bucket_plans"] in (None, [(4096, 1)]) for t in res["trials"])
    f._params = None
    with pytest.raises(RuntimeError):
        f.autotune(np.zeros((1, 10), np.float32))


def test_autotune_skips_out_of_memory_and_restores_on_failure():
    cost = lambda k, b, fl, v: 2.0 if (fl, v) == (8192, 1) else 3.0
    f = FakeFilter([200, 900], cost=cost)
    f.oom = (8192, 1)
    res = f.autotune(np.zeros((1, 10), np.float32), repeats=1, max_buckets=1)
    assert any("out of device memory" in t.get("error", "") for t in res["trials"])
    assert res["apply_ms"] == 3.0
    # a hard failure mid-search: the object goes back to the plan it had
    g = FakeFilter([200, 900], cost=cost)
    g.initialize(None, **dict(g._init_kw, length_buckets=2))
    start = dict(g._init_kw)
    g.fail_at = 4
    with pytest.raises(OSError):
        g.autotune(np.zeros((1, 10), np.float32), repeats=1, max_buckets=2)
    assert g.kw == start and g.plans == [(4096, 1), (4096, 1)]

