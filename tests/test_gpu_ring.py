"""Device ring of recent samples (SignalRing, mfgpu_ring_*): a window set
from the ring gives the same coefficients as the same window uploaded from
the host, across the ring's wrap-around, and serving requests that name a
ring window return the same peaks as requests carrying the samples."""
import numpy as np
import pytest
from scipy.signal import butter, sosfilt
from scipy.signal.windows import hann

import mflib_gb300 as mf
from mflib_gb300.serving import DetectionRequest, GpuExecutor, Server, TemplateBank

pytestmark = pytest.mark.gpu

FS = 100.0


def _bp(x, lo=1.0, hi=10.0):
    return sosfilt(butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos"), x, axis=-1)


def _templates(rng, lens):
    return [_bp(rng.standard_normal(int(L)), 2.0, 8.0) * hann(int(L)) for L in lens]


def _filter(tps, nch, n, dtype):
    p = mf.MultiChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(FS)
        p.add_template(wt)
    p.set_signal_size(n)
    f = mf.MultiChannel.MatchedFilter(dtype=dtype)
    f.initialize(p, template_channels=np.arange(len(tps)) % nch, n_channels=nch)
    return f


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ring_window_equals_uploaded_window(gpu, dtype):
    rng = np.random.default_rng(21)
    nch, cap, total = 6, 50_000, 180_000
    data = (_bp(rng.standard_normal((nch, total))) + rng.uniform(-20, 20, (nch, 1))).astype(dtype)
    ring = mf.SignalRing(nch, cap, dtype=dtype)
    assert ring.head == 0
    # appends of ragged sizes; the ring wraps several times
    pos, i = 0, 0
    sizes = [7_000, 1, 23_456, 50_000, 3, 31_000]
    while pos < total:
        k = min(sizes[i % len(sizes)], total - pos)
        ring.append(data[:, pos:pos + k])
        pos += k
        i += 1
    assert ring.head == total
    tps = _templates(rng, [300, 520, 411, 300])
    f = _filter(tps, 4, 30_000, dtype)
    chans = [5, 0, 3, 2]
    for end, n in [(total, 30_000), (total - 12_345, 20_000), (total - cap + 30_000, 30_000), (total, 5_000)]:
        f.set_window_ring(ring, end, n, chans)
        f.apply()
        a = [f.get_matched_filtered_signal(t).copy() for t in range(len(tps))]
        f.set_window(data[chans, end - n:end])
        f.apply()
        for t in range(len(tps)):
            np.testing.assert_array_equal(a[t], f.get_matched_filtered_signal(t))
    ring.close()


def test_ring_errors_and_long_append(gpu):
    rng = np.random.default_rng(22)
    ring = mf.SignalRing(2, 10_000)
    x = rng.standard_normal((2, 25_000)).astype(np.float32)
    ring.append(x)  # longer than the ring: its last 10,000 samples are kept
    assert ring.head == 25_000
    f = _filter(_templates(rng, [200]), 1, 8_000, np.float32)
    f.set_window_ring(ring, 25_000, 8_000, [1])
    f.apply()
    a = f.get_matched_filtered_signal(0).copy()
    f.set_window(x[1:2, 17_000:25_000])
    f.apply()
    np.testing.assert_array_equal(a, f.get_matched_filtered_signal(0))
    with pytest.raises(ValueError):
        f.set_window_ring(ring, 25_001, 8_000, [0])      # past the head
    with pytest.raises(ValueError):
        f.set_window_ring(ring, 22_000, 8_000, [0])      # start overwritten
    with pytest.raises(ValueError):
        f.set_window_ring(ring, 25_000, 8_000, [2])      # no such channel
    with pytest.raises(ValueError):
        f.set_window_ring(ring, 25_000, 9_000, [0])      # longer than the object's signal
    with pytest.raises(ValueError):
        f.set_window_ring(mf.SignalRing(1, 100, dtype=np.float64), 0, 10, [0])
    with pytest.raises(ValueError):
        mf.SignalRing(0, 10)
    with pytest.raises(ValueError):
        ring.append(np.zeros((3, 10), np.float32))


def test_serving_ring_requests_equal_uploaded(gpu):
    rng = np.random.default_rng(23)
    bank = TemplateBank("b", _templates(rng, rng.integers(200, 601, 10)))
    nch, total = 8, 120_000
    data = _bp(rng.standard_normal((nch, total))).astype(np.float32)
    for _ in range(12):  # injected template copies
        t = int(rng.integers(len(bank)))
        o = int(rng.integers(0, total - 700))
        c = int(rng.integers(nch))
        data[c, o:o + bank.templates[t].size] += (2 * np.std(data) * bank.templates[t]
                                                  / np.std(bank.templates[t])).astype(np.float32)
    ring = mf.SignalRing(nch, 100_000)
    for a in range(0, total, 6_000):
        ring.append(data[:, a:a + 6_000])
    srv = Server([bank], GpuExecutor(threshold=0.4, min_distance=100), memory_budget=8e9, slots=3,
                 buckets=(10_000, 20_000)).start()
    specs = [([0], total, 9_000), ([3, 1, 7], total - 4_000, 15_000), (list(range(8)), total - 50_000, 20_000),
             ([6, 2], total - 99_000 + 12_000, 12_000)]
    via_ring = [srv.submit(DetectionRequest("b", ring=ring, channels=ch, n=n, end=e, keep=(0,))) for ch, e, n in specs]
    uploaded = [srv.submit(DetectionRequest("b", data[ch, e - n:e], keep=(0,))) for ch, e, n in specs]
    for a, b in zip(via_ring, uploaded):
        a.wait(120)
        b.wait(120)
        assert len(a.peaks) == len(b.peaks) == len(bank)
        for t in range(len(bank)):
            np.testing.assert_array_equal(a.peaks[t], b.peaks[t])
        np.testing.assert_array_equal(a.rho[0], b.rho[0])
    assert sum(len(r.peaks[t]) for r in via_ring for t in range(len(bank))) > 0
    srv.close()
    ring.close()
