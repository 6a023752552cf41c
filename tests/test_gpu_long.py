"""Templates longer than any FFT plan takes (FP32 above 8,161 samples, FP64
above 4,065): correlated directly in the time domain (the fix-up kernel's
direct mode, two-pass Pearson per lag) beside the FFT plan of the other
templates.  The reference accepts any template length and sizes its FFT up
to 2^21 (src/matchedFilterParameters.cpp:54-64); its own sizing test uses
4,500-sample templates (testing/matchedFilterParameters.cpp:14-33)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(mf, tps, n, single=False):
    p = mf.SingleChannel.MatchedFilterParameters() if single else mf.MultiChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(100.0)
        p.add_template(wt)
    p.set_signal_size(n)
    return p


def _signal(rng, n, tps, copies=3):
    x = rng.standard_normal(n) + 2.0
    for tp in tps:
        for o in rng.integers(0, n - tp.size, copies):
            x[o:o + tp.size] += 1.5 * tp / np.std(tp)
    return x


def test_fp64_reference_sizing(gpu, oracle, rng):
    """nb = 4,500 against 75,000 samples (the reference's sizing case, FFT
    32,768 / block 28,269), beside a template the FFT plan takes."""
    mf = gpu
    assert oracle.fft_sizes(4500, 75000) == (32768, 28269)
    tps = [rng.standard_normal(4500), rng.standard_normal(700)]
    x = _signal(rng, 75_000, tps)
    f = mf.SingleChannel.MatchedFilter(dtype=np.float64)
    f.initialize(_params(mf, tps, x.size, single=True))
    f.set_signal(x)
    f.apply()
    for t, tp in enumerate(tps):
        got = f.get_valid_matched_filtered_signal(t)
        ref = oracle.pearson_naive(tp, x)
        assert got.size == ref.size
        assert np.max(np.abs(got - ref)) < 1e-11


def test_fp32_long_templates_mixed(gpu, oracle, rng):
    """FP32 templates of 9,000 and 20,000 samples beside FFT-planned ones on
    two channels, every lag against the FP64 oracle on the same samples."""
    mf = gpu
    n = 100_000
    tps = [rng.standard_normal(L) for L in (20_000, 500, 9_000, 1_200)]
    chan = [0, 0, 1, 1]
    sigs = [_signal(rng, n, [tps[i] for i in range(4) if chan[i] == c]).astype(np.float32) for c in range(2)]
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, tps, n), template_channels=chan, n_channels=2)
    f.set_channel_signals(np.stack(sigs))
    f.apply()
    for t, c in enumerate(chan):
        got = f.get_valid_matched_filtered_signal(t).astype(np.float64)
        ref = oracle.pearson_naive(tps[t], sigs[c].astype(np.float64))
        assert got.size == ref.size
        assert np.max(np.abs(got - ref)) < 1e-5, (t, np.max(np.abs(got - ref)))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_only_long_templates_and_peaks(gpu, oracle, rng, dtype):
    """An object whose every template is long (no FFT plan at all), and the
    batched peak finder on its traces."""
    mf = gpu
    L = 9_000 if dtype == np.float32 else 5_000
    tps = [rng.standard_normal(L), rng.standard_normal(L + 333)]
    n = 60_000
    x = _signal(rng, n, tps).astype(dtype)
    f = mf.SingleChannel.MatchedFilter(dtype=dtype)
    f.initialize(_params(mf, tps, n, single=True))
    f.set_signal(x)
    f.apply()
    tol = 1e-5 if dtype == np.float32 else 1e-11
    for t, tp in enumerate(tps):
        rho = f.get_matched_filtered_signal(t).astype(np.float64)
        ref = oracle.pearson_naive(tp, x.astype(np.float64))[: rho.size]
        assert np.max(np.abs(rho - ref)) < tol
        f.find_peaks(0.3, 500)
        np.testing.assert_array_equal(f.get_peaks(t), oracle.peaks(rho, 0.3, 500))


def test_long_template_fused_peaks_and_dead_channel(gpu, oracle, rng):
    """Peak candidates gathered inside the correlator for the FFT templates
    and recounted for the long one give the oracle's peaks; a dead channel's
    long template is all zeros."""
    mf = gpu
    n = 80_000
    tps = [rng.standard_normal(10_000), rng.standard_normal(400), rng.standard_normal(12_000)]
    chan = [0, 0, 1]
    sig0 = _signal(rng, n, tps[:2]).astype(np.float32)
    dead = np.full(n, 3.0, dtype=np.float32)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, tps, n), template_channels=chan, n_channels=2)
    f.set_peak_threshold(0.25)
    f.set_channel_signals(np.stack([sig0, dead]))
    f.apply()
    f.find_peaks(0.25, 300)
    counts, idx = f.get_all_peaks()
    off = 0
    for t in range(3):
        rho = f.get_matched_filtered_signal(t).astype(np.float64)
        np.testing.assert_array_equal(idx[off:off + counts[t]], oracle.peaks(rho, 0.25, 300))
        off += counts[t]
    assert not np.any(f.get_valid_matched_filtered_signal(2))


def test_too_long_for_the_direct_correlator(gpu, rng):
    """Beyond what one warp's shared-memory row holds, initialize refuses."""
    mf = gpu
    n = 40_000
    f = mf.SingleChannel.MatchedFilter(dtype=np.float64)
    with pytest.raises(ValueError):
        f.initialize(_params(mf, [rng.standard_normal(30_000)], n, single=True))
