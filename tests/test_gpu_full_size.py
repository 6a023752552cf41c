"""The 24-channel day at its full size (24 channels x 8,640,000 FP32
samples, 192 templates of 500 samples, 8 per channel) through the
properties that hold at any size:

* parity with the FP64 oracle (direct Pearson sums) at sampled lags of one
  template per channel, the first and last lags and both sides of every
  sampled block boundary included, within the metric's 1e-4;
* every coefficient finite and |rho| <= 1 (FP32 rounding aside);
* negating the signals negates every coefficient;
* scaling the signals by 4 (exact in FP32) leaves every coefficient
  unchanged to rounding;
* shifting the signals (circularly, by a count that is no multiple of the
  block length) shifts every coefficient by the same count: the blocks then
  cut the traces at other places.
"""
import numpy as np
import pytest

from test_gpu_configs import _params, _template

pytestmark = pytest.mark.gpu

NCH, N, L, TPC = 24, 8_640_000, 500, 8


@pytest.fixture(scope="module")
def day():
    rng = np.random.default_rng(2026)
    x = rng.standard_normal((NCH, N), dtype=np.float32)
    tps = [_template(4000 + t, L, 1.5 + (t % 5), 8.0 + (t % 5)) for t in range(NCH * TPC)]
    chan = np.repeat(np.arange(NCH), TPC)
    # injected copies, so that the sampled lags include large coefficients
    for t in range(0, NCH * TPC, TPC):
        for o in rng.integers(0, N - L, 20):
            x[chan[t], o:o + L] += (2.0 * tps[t] / np.std(tps[t])).astype(np.float32)
    return x, tps, chan


def _traces(f, ts):
    return np.stack([f.get_matched_filtered_signal(t) for t in ts])


def test_full_day_properties(gpu, oracle, day):
    mf = gpu
    x, tps, chan = day
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, tps, N), template_channels=chan, n_channels=NCH)
    plan = f.get_plan()
    S = plan["lags_per_block"]
    nv = f.get_filtered_signal_length()
    assert nv == N - L + 1
    ts = [TPC * c + c % TPC for c in range(NCH)]  # one template per channel

    f.set_channel_signals(x)
    f.apply()
    r0 = _traces(f, ts)
    assert np.all(np.isfinite(r0))
    assert float(np.max(np.abs(r0))) <= 1.0 + 1e-5

    rng = np.random.default_rng(7)
    worst = 0.0
    for i, t in enumerate(ts):
        b = rng.integers(1, nv // S, 8) * S
        lags = np.unique(np.concatenate([[0, 1, nv - 2, nv - 1], b - 1, b, rng.integers(0, nv, 48)]))
        truth = oracle.pearson_naive(tps[t], x[chan[t]].astype(np.float64), lags)
        worst = max(worst, float(np.max(np.abs(r0[i, lags].astype(np.float64) - truth))))
    print("\nfull day: max|drho| vs the FP64 oracle at sampled lags %.3g" % worst)
    assert worst < 1e-4

    f.set_channel_signals(-x)
    f.apply()
    np.testing.assert_allclose(_traces(f, ts), -r0, rtol=0, atol=1e-6)

    f.set_channel_signals(4.0 * x)
    f.apply()
    np.testing.assert_allclose(_traces(f, ts), r0, rtol=0, atol=1e-6)

    s = 1_234_567
    assert s % S != 0
    f.set_channel_signals(np.roll(x, -s, axis=1))
    f.apply()
    r1 = _traces(f, ts)
    m = nv - s
    np.testing.assert_allclose(r1[:, :m], r0[:, s:s + m], rtol=0, atol=1e-5)
