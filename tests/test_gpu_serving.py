"""Serving loop on the GPU (mflib_gb300/serving.py): request windows against
resident banks, checked against the oracle, and every request's result the
same alone and in a concurrent mix."""
import numpy as np
import pytest
from scipy.signal import butter, sosfilt
from scipy.signal.windows import hann

from mflib_gb300.serving import DetectionRequest, GpuExecutor, Server, TemplateBank

pytestmark = pytest.mark.gpu

FS = 100.0


def _bp(x, lo, hi):
    return sosfilt(butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos"), x)


def _template(rng, L):
    lo = rng.uniform(1.0, 7.0)
    return _bp(rng.standard_normal(L), lo, min(lo + rng.uniform(2.0, 8.0), 15.0)) * hann(L)


def _banks():
    rng = np.random.default_rng(41)
    mixed = TemplateBank("mixed", [_template(rng, int(L)) for L in rng.integers(200, 601, 12)])
    equal = TemplateBank("equal", [_template(rng, 300) for _ in range(8)], channel_slots=[3 * t for t in range(8)])
    return [mixed, equal]


def _requests(banks, rng):
    out = []
    for i, (c, n) in enumerate([(1, 3000), (3, 9000), (64, 4500), (5, 14000), (2, 12000), (7, 2500), (64, 10000),
                                (1, 15000)]):
        bank = banks[i % 2]
        x = _bp(rng.standard_normal((c, n)), 1.0, 10.0)
        for _ in range(3):  # injected template copies
            t = int(rng.integers(len(bank)))
            tp = bank.templates[t]
            o = int(rng.integers(0, n - tp.size))
            x[bank.slots[t] % c, o:o + tp.size] += rng.uniform(0.5, 2.0) * np.std(x) * tp / np.std(tp)
        x += rng.uniform(-50, 50, (c, 1))  # DC offsets
        out.append((bank.name, x.astype(np.float32), (0, len(bank) - 1)))
    return out


def _serve(banks, reqs, slots):
    srv = Server(banks, GpuExecutor(threshold=0.5, min_distance=100), memory_budget=8e9, slots=slots,
                 buckets=(5000, 10000, 15000)).start()
    rs = [srv.submit(DetectionRequest(b, x, keep=k)) for b, x, k in reqs]
    for r in rs:
        r.wait(120)
    srv.close()
    return rs


def test_serving_matches_oracle(gpu, oracle):
    banks = _banks()
    reqs = _requests(banks, np.random.default_rng(7))
    rs = _serve(banks, reqs, slots=2)
    by = {b.name: b for b in banks}
    worst = 0.0
    for r, (bname, x, keep) in zip(rs, reqs):
        bank = by[bname]
        nv = r.n - bank.max_length + 1
        assert len(r.peaks) == len(bank) and r.lags == len(bank) * nv
        for t in keep:
            got = r.rho[t].astype(np.float64)
            assert got.size == nv
            lags = np.unique(np.linspace(0, nv - 1, 400).astype(int))
            truth = oracle.pearson_naive(bank.templates[t], x[bank.slots[t] % x.shape[0]].astype(np.float64), lags)
            worst = max(worst, float(np.max(np.abs(got[lags] - truth))))
            # peaks agree with the oracle's PeakFinder on the returned trace
            np.testing.assert_array_equal(r.peaks[t], oracle.peaks(got, 0.5, 100))
    print("\nserving: max|drho| vs oracle %.3g" % worst)
    assert worst < 1e-4


def test_serving_alone_equals_mix(gpu):
    banks = _banks()
    reqs = _requests(banks, np.random.default_rng(8))
    alone = []
    for b, x, k in reqs:
        alone += _serve(banks, [(b, x, k)], slots=1)
    mix = _serve(banks, reqs, slots=4)
    worst = 0.0
    for a, m in zip(alone, mix):
        assert len(a.peaks) == len(m.peaks)
        for pa, pm in zip(a.peaks, m.peaks):
            np.testing.assert_array_equal(pa, pm)
        for t in a.rho:
            worst = max(worst, float(np.max(np.abs(a.rho[t].astype(np.float64) - m.rho[t]))))
    print("\nserving: max|drho| alone vs mix %.3g" % worst)
    assert worst <= 1e-6


def test_serving_under_tight_budget(gpu):
    """A device-memory budget that holds only about one object forces the
    loop to evict idle objects between keys; every result still equals the
    same request served alone with room to spare."""
    banks = _banks()
    reqs = _requests(banks, np.random.default_rng(9))
    ex = GpuExecutor(threshold=0.5, min_distance=100)
    big = max(ex.estimate_bytes(b, 15000) for b in banks)
    tight = Server(banks, ex, memory_budget=1.2 * big, slots=3, buckets=(5000, 10000, 15000)).start()
    rs = [tight.submit(DetectionRequest(b, x, keep=k)) for b, x, k in reqs]
    for r in rs:
        r.wait(120)
    tight.close()
    assert tight.evicted > 0
    assert tight.peak_held <= 1.2 * big + max(ex.estimate_bytes(b, 15000) for b in banks)
    alone = _serve(banks, reqs, slots=1)
    for a, m in zip(alone, rs):
        for pa, pm in zip(a.peaks, m.peaks):
            np.testing.assert_array_equal(pa, pm)
        for t in a.rho:
            np.testing.assert_array_equal(a.rho[t], m.rho[t])
