"""Matched filter on the GPU (through the C ABI) against the CPU oracle and
the reference's own known-answer tests.

Tolerances: FP64 engine at the reference tests' own bounds (1e-13 .. 1e-14
versus the naive two-pass Pearson correlation); FP32 engine within 1e-5
absolute of the FP64 oracle, the bound stated for the FP32 path."""
import numpy as np
import pytest

from test_oracle import damped_case

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def _params(mf, templates, n, mode="multi", fs=1.0):
    p = mf.MultiChannel.MatchedFilterParameters() if mode == "multi" else mf.SingleChannel.MatchedFilterParameters()
    for t in templates:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(fs)
        p.add_template(wt)
    p.set_signal_size(n)
    return p


def test_basic_double(gpu, oracle):
    # testing/matchedFilter.cpp:58-168
    mf = gpu
    x, x2, b, b2 = damped_case()
    f = mf.MultiChannel.MatchedFilter()
    f.initialize(_params(mf, [b], x.size))
    f.set_signal(0, x)
    np.testing.assert_array_equal(f.get_signal(0), x)
    assert not f.have_matched_filtered_signals()
    f.apply()
    assert f.have_matched_filtered_signals()
    r = f.get_matched_filtered_signal(0)
    assert r.size == x.size - b.size + 1
    assert np.max(np.abs(r - oracle.pearson_naive(b, x))) < 1e-13
    f.initialize(_params(mf, [b, b2, b, b2], x.size))
    for i, s in enumerate([x, x2, x, x2]):
        f.set_signal(i, s)
    f.apply()
    for i, (tp, s) in enumerate(zip([b, b2, b, b2], [x, x2, x, x2])):
        assert np.max(np.abs(f.get_matched_filtered_signal(i) - oracle.pearson_naive(tp, s))) < 1e-13


def test_basic_float(gpu, oracle):
    # testing/matchedFilter.cpp:172-271 (< 2e-6)
    mf = gpu
    x, x2, b, b2 = damped_case()
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, [b, b2, b, b2], x.size))
    for i, s in enumerate([x, x2, x, x2]):
        f.set_signal(i, s.astype(np.float32))
    f.apply()
    for i, (tp, s) in enumerate(zip([b, b2, b, b2], [x, x2, x, x2])):
        ref = oracle.pearson_naive(tp.astype(np.float32), s.astype(np.float32))
        assert np.max(np.abs(f.get_matched_filtered_signal(i).astype(np.float64) - ref)) < 2e-6


def test_shift_and_stack(gpu, oracle):
    # testing/matchedFilter.cpp:275-465
    mf = gpu
    df = 100.0
    dt = 1 / df
    n = int(120 / dt + 0.5) + 1
    tsz = int(4 / dt + 0.5) + 1
    toffs = [1.0, 2.0, 1.5]
    extras = [int(t / dt + 0.5) for t in toffs]
    tts = [20.0, 40.0, 80.0]
    amps = [(2.0, 1.0), (1.5, 1.5), (1.2, 2.5)]
    sigs = []
    tps = []
    base = np.where(np.arange(n) % 2 == 0, -0.001, 0.001)
    t = np.arange(tsz) * dt
    for (a, d), ex, tt in zip(amps, extras, tts):
        w = a * np.exp(-d * t) * np.sin(2 * np.pi * t / 4.0)
        w[0] = 0
        w[-1] = 0
        tp = np.zeros(tsz + ex)
        tp[ex:] = w
        s = base.copy()
        i0 = int((8.0 + tt) / dt + 0.5)
        s[i0:i0 + tsz] = w
        tps.append(tp)
        sigs.append(s)
    p = mf.MultiChannel.MatchedFilterParameters()
    for tp, to, tt in zip(tps, toffs, tts):
        wt = mf.WaveformTemplate()
        wt.set_signal(tp)
        wt.set_sampling_rate(df)
        wt.set_phase_travel_time(tt)
        wt.set_phase_onset_time_in_signal(to)
        p.add_template(wt)
    p.set_signal_size(n)
    f = mf.MultiChannel.MatchedFilter()
    f.initialize(p)
    for i, s in enumerate(sigs):
        f.set_signal(i, s)
    f.apply()
    for i in range(3):
        r = f.get_matched_filtered_signal(i)
        ref = oracle.pearson_naive(tps[i], sigs[i])[: r.size]
        assert np.max(np.abs(r - ref)) <= 1e-11
    stack = f.shift_and_stack()
    imax = int(np.argmax(stack))
    assert abs(stack[imax] - 1.0) < 1e-3
    assert abs(imax / df - 8.0) <= 1 / df / 2
    # the same stack from the oracle's restatement of shiftAndStack
    rows = [f.get_matched_filtered_signal(i) for i in range(3)]
    shifts = [int((tt - to) * df + 0.5) for tt, to in zip(tts, toffs)]
    ref_stack = oracle.shift_and_stack(rows, rows[0].size, shifts, [1, 1, 1])
    assert np.max(np.abs(stack - ref_stack)) < 1e-14


def test_single_channel_double(gpu, oracle, rng):
    # testing/singleChannel.cpp:104-160 (< 1e-12)
    mf = gpu
    wave = rng.uniform(2, 3, 4000)
    tps = [wave[25:155], wave[1124:1264], wave[3601:3726]]
    f = mf.SingleChannel.MatchedFilter()
    f.initialize(_params(mf, tps, wave.size, mode="single"))
    f.set_signal(wave)
    np.testing.assert_array_equal(f.get_signal(), wave)
    f.apply()
    for i, tp in enumerate(tps):
        r = f.get_matched_filtered_signal(i)
        ref = oracle.pearson_naive(tp, wave)[: r.size]
        assert np.max(np.abs(r - ref)) < 1e-12


def test_pymflib_multichannel(gpu, oracle):
    # python/unit_tests.py:198-246 (< 1e-14)
    mf = gpu
    n = 3000
    tmax = 8
    f0 = 4 / tmax
    dt = tmax / (n - 1)
    times = np.linspace(0, tmax, n, endpoint=False)
    s1 = np.exp(-0.1 * times) * np.sin(2 * np.pi * f0 * times)
    s2 = np.exp(-0.15 * times) * np.cos(2 * np.pi * f0 * times)
    nb = int(2 / dt + 0.5)
    tt = np.linspace(0, 2, nb, endpoint=False)
    t1 = np.sin(2 * np.pi * f0 * tt)
    t2 = np.cos(2 * np.pi * f0 * tt)
    f = mf.MultiChannel.MatchedFilter()
    f.initialize(_params(mf, [t1, t2], n, fs=1 / dt))
    f.set_signal(0, s1)
    f.set_signal(1, s2)
    f.apply()
    assert np.max(np.abs(f.get_matched_filtered_signal(0) - oracle.pearson_naive(t1, s1))) < 1e-14
    assert np.max(np.abs(f.get_matched_filtered_signal(1) - oracle.pearson_naive(t2, s2))) < 1e-14


def test_pymflib_single_channel(gpu, oracle, rng):
    # python/unit_tests.py:250-299 (< 1e-14)
    mf = gpu
    fs = 100.0
    n = int(fs * 60 * 3) + 1
    L = int(fs * 10) + 1
    sig = rng.uniform(-3, 4, n)
    tps = [sig[int(n * a):int(n * a) + L] for a in (0.25, 0.05, 0.8)]
    f = mf.SingleChannel.MatchedFilter()
    f.initialize(_params(mf, tps, n, mode="single", fs=fs))
    f.set_signal(sig)
    f.apply()
    lags = rng.integers(0, n - L + 1, 3000)
    for i, tp in enumerate(tps):
        r = f.get_matched_filtered_signal(i)
        ref = oracle.pearson_naive(tp, sig, lags)
        assert np.max(np.abs(r[lags] - ref)) < 1e-14


@pytest.mark.parametrize("mode", ["multi", "single"])
@pytest.mark.parametrize("lens", [(400,), (200, 200, 200), (37, 500, 130, 999)])
def test_fp32_vs_fp64_oracle(gpu, oracle, rng, mode, lens):
    mf = gpu
    n = 50_000
    nsig = len(lens) if mode == "multi" else 1
    sigs = [(rng.standard_normal(n) * 2 + 3).astype(np.float32) for _ in range(nsig)]
    tps = [rng.standard_normal(L) for L in lens]
    f = mf.MatchedFilter(dtype=np.float32)
    p = mf.MatchedFilterParameters(0 if mode == "single" else 1)
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(100.0)
        p.add_template(wt)
    p.set_signal_size(n)
    f.initialize(p)
    for i, s in enumerate(sigs):
        f.set_signal(i, s)
    f.apply()
    ref = oracle.matched_filter(tps, sigs, multi=(mode == "multi"), fp64_from_f32=True)
    for i in range(len(tps)):
        r = f.get_valid_matched_filtered_signal(i).astype(np.float64)
        assert r.size == ref[i].size
        assert np.max(np.abs(r - ref[i])) < FP32_TOL
        short = f.get_matched_filtered_signal(i)
        assert short.size == n - max(lens) + 1
        np.testing.assert_array_equal(short, r[: short.size].astype(np.float32))


@pytest.mark.parametrize("fft_length", [1024, 2048, 4096, 8192])
def test_forced_fft_lengths(gpu, oracle, rng, fft_length):
    mf = gpu
    n = 30_001
    sig = rng.standard_normal(n).astype(np.float32)
    tps = [rng.standard_normal(300), rng.standard_normal(300)]
    p = _params(mf, tps, n, mode="single")
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, fft_length=fft_length)
    assert f.get_plan()["fft_length"] == fft_length
    f.set_signal(sig)
    f.apply()
    ref = oracle.matched_filter(tps, [sig], multi=False, fp64_from_f32=True)
    for i in range(2):
        assert np.max(np.abs(f.get_valid_matched_filtered_signal(i) - ref[i])) < FP32_TOL


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("variant", [1, 2, 3, 5])
@pytest.mark.parametrize("fft_length", [0, 256, 2048, 4096])
@pytest.mark.parametrize("ntpl", [1, 2, 5])
def test_correlator_variants(gpu, oracle, rng, dtype, variant, fft_length, ntpl):
    """Every correlator organisation (whole CTA, whole CTA with the next
    spectrum prefetched, two teams of 128 threads reading precomputed
    normalisation rows or normalising inside the CTA) gives the oracle's
    coefficients; 5 templates on one channel leave one team a template
    short in the last round."""
    mf = gpu
    if dtype == np.float64 and fft_length > 4096:
        pytest.skip("FP64 correlator stops at N = 4096")
    n = 20_011
    L = 100
    chans = [rng.standard_normal(n) + 3.0 for _ in range(2)]
    assign = [0] * ntpl + [1] * ntpl
    tps = [rng.standard_normal(L) for _ in assign]
    p = _params(mf, tps, n)
    f = mf.MultiChannel.MatchedFilter(dtype=dtype)
    f.initialize(p, template_channels=assign, n_channels=2, fft_length=fft_length, correlator_variant=variant)
    if fft_length:
        assert f.get_plan()["fft_length"] == fft_length
    assert f.get_plan()["correlator"] == variant
    for c, s in enumerate(chans):
        f.set_channel_signal(c, s.astype(dtype))
    f.apply()
    sig = [chans[c].astype(dtype) for c in assign]
    ref = oracle.matched_filter(tps, sig, multi=True, fp64_from_f32=dtype == np.float32)
    tol = FP32_TOL if dtype == np.float32 else 1e-11
    for i in range(len(assign)):
        a = f.get_valid_matched_filtered_signal(i)
        assert a.size == ref[i].size
        assert np.max(np.abs(a - ref[i])) < tol, (i, np.max(np.abs(a - ref[i])))


def test_correlator_variant_errors(gpu, rng):
    mf = gpu
    n = 5000
    p = _params(mf, [rng.standard_normal(100), rng.standard_normal(120)], n)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    with pytest.raises(ValueError):
        f.initialize(p, correlator_variant=3)  # teams need one template length
    with pytest.raises(ValueError):
        f.initialize(p, correlator_variant=5)
    with pytest.raises(ValueError):
        f.initialize(p, correlator_variant=4)
    with pytest.raises(ValueError):
        f.initialize(p, correlator_variant=7)
    f.initialize(p, correlator_variant=2)
    assert f.is_initialized()
    # two 256-thread teams: FP32 and templates of several lengths only
    f.initialize(p, correlator_variant=6)
    assert f.get_plan()["correlator"] == 6
    with pytest.raises(ValueError):
        mf.MultiChannel.MatchedFilter(dtype=np.float64).initialize(p, correlator_variant=6)
    with pytest.raises(ValueError):
        f.initialize(_params(mf, [rng.standard_normal(100)] * 2, n), correlator_variant=6)


def test_shared_channels_extension(gpu, oracle, rng):
    """Several templates reading one channel (template_channels) give the
    same coefficients as one signal copy per template."""
    mf = gpu
    n = 40_000
    chans = [rng.standard_normal(n).astype(np.float32) for _ in range(3)]
    assign = [0, 0, 1, 2, 2, 2]
    tps = [rng.standard_normal(250) for _ in assign]
    p = _params(mf, tps, n)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, template_channels=assign, n_channels=3)
    for c, s in enumerate(chans):
        f.set_channel_signal(c, s)
    f.apply()
    g = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    g.initialize(p)
    for i, c in enumerate(assign):
        g.set_signal(i, chans[c])
    g.apply()
    ref = oracle.matched_filter(tps, [chans[c] for c in assign], multi=True, fp64_from_f32=True)
    for i in range(len(assign)):
        a = f.get_matched_filtered_signal(i)
        np.testing.assert_array_equal(a, g.get_matched_filtered_signal(i))
        assert np.max(np.abs(a - ref[i][: a.size])) < FP32_TOL


def test_dc_offset_fp32(gpu, oracle, rng):
    """A large DC offset (1e4) barely moves the FP32 engine's error: the
    block mean is removed before the FFT and the sliding sums."""
    mf = gpu
    n = 60_000
    sig = (rng.standard_normal(n) + 1e4).astype(np.float32)
    tp = rng.standard_normal(500)
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, [tp], n, mode="single"))
    f.set_signal(sig)
    f.apply()
    lags = rng.integers(0, n - 500 + 1, 2000)
    ref = oracle.pearson_naive(tp, sig.astype(np.float64), lags)
    r = f.get_matched_filtered_signal(0)
    assert np.max(np.abs(r[lags] - ref)) < 5e-4


def test_dead_and_zero_signals(gpu, rng):
    mf = gpu
    n = 5000
    tps = [rng.standard_normal(100), rng.standard_normal(100)]
    f = mf.MultiChannel.MatchedFilter()
    f.initialize(_params(mf, tps, n))
    f.set_signal(0, np.full(n, 3.0))        # dead: |min| == |max|
    f.set_signal(1, rng.standard_normal(n))
    f.apply()
    assert np.all(f.get_matched_filtered_signal(0) == 0)
    assert np.any(f.get_matched_filtered_signal(1) != 0)
    f.zero_signal(1)
    f.apply()
    assert np.all(f.get_matched_filtered_signal(1) == 0)
    np.testing.assert_array_equal(f.get_signal(1), np.zeros(n))
    # a live-looking signal whose extremes are +-5 is dead by the reference's
    # rule too (|min| == |max|, src/matchedFilter.cpp:882-894); one sample
    # less extreme makes it live again
    x = np.clip(rng.standard_normal(n), -4, 4)
    x[10], x[4000] = 5.0, -5.0
    for dtype in (np.float64, np.float32):
        g = mf.MultiChannel.MatchedFilter(dtype=dtype)
        g.initialize(_params(mf, tps, n))
        g.set_signal(0, x.astype(dtype))
        x2 = x.copy()
        x2[4000] = -4.5
        g.set_signal(1, x2.astype(dtype))
        g.apply()
        assert np.all(g.get_matched_filtered_signal(0) == 0)
        assert np.any(g.get_matched_filtered_signal(1) != 0)


def test_errors(gpu, rng):
    mf = gpu
    f = mf.MultiChannel.MatchedFilter()
    with pytest.raises(RuntimeError):
        f.apply()
    assert f.get_number_of_templates() == 0  # pymflib: 0 before initialize
    tps = [rng.standard_normal(50)]
    f.initialize(_params(mf, tps, 1000))
    with pytest.raises(ValueError):
        f.set_signal(1, np.zeros(1000))
    with pytest.raises(ValueError):
        f.set_signal(0, np.zeros(999))
    with pytest.raises(RuntimeError):
        f.get_matched_filtered_signal(0)
    with pytest.raises(RuntimeError):
        f.shift_and_stack()
    p = mf.MultiChannel.MatchedFilterParameters()
    with pytest.raises(ValueError):
        f.initialize(p)


def test_short_signal_edge(gpu, oracle, rng):
    """Signal shorter than the longest template: the common filtered length
    is empty; shorter templates keep their valid lags."""
    mf = gpu
    n = 300
    tps = [rng.standard_normal(40), rng.standard_normal(400)]
    f = mf.SingleChannel.MatchedFilter()
    f.initialize(_params(mf, tps, n, mode="single"))
    sig = rng.standard_normal(n)
    f.set_signal(sig)
    f.apply()
    assert f.get_matched_filtered_signal(0).size == 0
    r = f.get_valid_matched_filtered_signal(0)
    assert r.size == n - 40 + 1
    assert np.max(np.abs(r - oracle.pearson_naive(tps[0], sig))) < 1e-12
    assert f.get_valid_matched_filtered_signal(1).size == 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("mode", ["multi", "single"])
def test_signal_as_long_as_the_template(gpu, oracle, rng, dtype, mode):
    """A signal as long as the longest template (one valid lag) or one
    sample longer (two): the reference sizes its FFT from (L, n + L - 1)
    (src/matchedFilter.cpp:519-525), so both are legal; coefficients equal
    the two-pass Pearson correlation."""
    mf = gpu
    tol = 1e-12 if dtype == np.float64 else 2e-5
    for L in (2, 37, 500, 3000):
        for extra in (0, 1):
            n = L + extra
            tp = rng.standard_normal(L)
            sig = rng.standard_normal(n) + 3.0
            f = mf.SingleChannel.MatchedFilter(dtype=dtype) if mode == "single" else \
                mf.MultiChannel.MatchedFilter(dtype=dtype)
            f.initialize(_params(mf, [tp], n, mode=mode))
            if mode == "single":
                f.set_signal(sig.astype(dtype))
            else:
                f.set_signal(0, sig.astype(dtype))
            f.apply()
            r = f.get_matched_filtered_signal(0)
            assert r.size == extra + 1
            ref = oracle.pearson_naive(tp, sig.astype(dtype).astype(np.float64))
            assert np.max(np.abs(r - ref)) < tol, (L, n)


def test_spectra_of_template(gpu, rng):
    """getSpectraOfTemplate is the reference's rfft of the reversed,
    demeaned, unit-norm template at its own FFT length."""
    mf = gpu
    tp = rng.standard_normal(120)
    f = mf.MultiChannel.MatchedFilter()
    f.initialize(_params(mf, [tp], 2000))
    spec = f.get_spectra_of_template(0)
    nfft, _ = mf.compute_optimal_fft_and_block_length(120, 2000 + 119)
    b = tp - tp.mean()
    b = b[::-1] / np.linalg.norm(b)
    ref = np.fft.rfft(b, nfft)
    assert np.max(np.abs(spec - ref)) < 1e-12


def test_repeat_apply_and_reinitialize(gpu, oracle, rng):
    mf = gpu
    n = 20_000
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    for L in (64, 700, 2500):
        tp = rng.standard_normal(L)
        f.initialize(_params(mf, [tp], n, mode="single"))
        for _ in range(2):
            sig = rng.standard_normal(n).astype(np.float32)
            f.set_signal(sig)
            f.apply()
            ref = oracle.matched_filter([tp], [sig], multi=False, fp64_from_f32=True)[0]
            assert np.max(np.abs(f.get_matched_filtered_signal(0) - ref)) < FP32_TOL


def test_batched_channel_upload(gpu, rng):
    """set_channel_signals (one copy, one dead-trace pass) stores the same
    samples and dead flags as one set_channel_signal per channel, for
    contiguous and strided rows and a channel sub-range."""
    mf = gpu
    n = 33_333
    x = rng.standard_normal((5, n)).astype(np.float32)
    x[3] = 0.0                       # dead channel
    x[1, :] = 2.0
    x[1, 7] = -2.0                   # |min| == |max|: dead as well
    assign = [0, 1, 2, 3, 4, 0]
    tps = [rng.standard_normal(64) for _ in assign]
    p = _params(mf, tps, n)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, template_channels=assign, n_channels=5)
    g = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    g.initialize(p, template_channels=assign, n_channels=5)
    wide = np.zeros((5, n + 17), dtype=np.float32)
    wide[:, :n] = x
    f.set_channel_signals(x[:2])
    f.set_channel_signals(wide[2:, :n], first_channel=2)
    for c in range(5):
        g.set_channel_signal(c, x[c])
    for h in (f, g):
        h.apply()
    for i in range(len(assign)):
        np.testing.assert_array_equal(f.get_signal(i), x[assign[i]])
        np.testing.assert_array_equal(f.get_matched_filtered_signal(i), g.get_matched_filtered_signal(i))
    assert not np.any(f.get_matched_filtered_signal(3))
    assert not np.any(f.get_matched_filtered_signal(1))
    with pytest.raises(ValueError):
        f.set_channel_signals(x, first_channel=1)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("L", [32, 33, 95, 511, 1024, 4097, 6000])
@pytest.mark.parametrize("variant", [0, 5])
def test_shared_length_normalisation(gpu, oracle, rng, dtype, L, variant):
    """Templates of one length: the planner's choice (variant 0) or the
    in-CTA normalisation (variant 5), for window lengths
    with L mod 32 = 0, 1, 31 and lengths that need two or three 32-sample
    runs per thread; the signals carry an offset and a slow drift of several
    standard deviations."""
    mf = gpu
    if dtype == np.float64 and L > 4065:
        pytest.skip("the FP64 correlator's longest template is 4065 samples (N = 4096)")
    n = 60_000 + L
    t = np.arange(n)
    chans = [rng.standard_normal(n) + 5.0 + 4.0 * np.sin(2 * np.pi * t / 20_000.0 + k) for k in range(2)]
    assign = [0, 1, 1]
    tps = [rng.standard_normal(L) for _ in assign]
    p = _params(mf, tps, n)
    f = mf.MultiChannel.MatchedFilter(dtype=dtype)
    f.initialize(p, template_channels=assign, n_channels=2, correlator_variant=variant)
    for c, s in enumerate(chans):
        f.set_channel_signal(c, s.astype(dtype))
    f.apply()
    sig = [chans[c].astype(dtype) for c in assign]
    ref = oracle.matched_filter(tps, sig, multi=True, fp64_from_f32=dtype == np.float32)
    tol = FP32_TOL if dtype == np.float32 else 1e-11
    for i in range(len(assign)):
        a = f.get_valid_matched_filtered_signal(i)
        assert np.max(np.abs(a - ref[i])) < tol, (i, np.max(np.abs(a - ref[i])))


def test_staged_upload_pipeline(gpu, rng):
    """stage_channel_signals: results of a pipelined loop (stage step i+1,
    then read step i's results) equal those of synchronous uploads; staged
    signals become current on apply, get_signal or a synchronous setter,
    and a second stage before apply replaces the first."""
    mf = gpu
    n, nch = 20_000, 3
    steps = [rng.standard_normal((nch, n)).astype(np.float32) for _ in range(4)]
    assign = [0, 1, 2, 2]
    tps = [rng.standard_normal(120) for _ in assign]
    p = _params(mf, tps, n)
    ref = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    ref.initialize(p, template_channels=assign, n_channels=nch)
    want = []
    for x in steps:
        ref.set_channel_signals(x)
        ref.apply()
        want.append([ref.get_matched_filtered_signal(i) for i in range(len(assign))])
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, template_channels=assign, n_channels=nch)
    f.stage_channel_signals(steps[0])
    for k in range(len(steps)):
        f.apply()
        if k + 1 < len(steps):
            f.stage_channel_signals(steps[k + 1])
        for i in range(len(assign)):
            np.testing.assert_array_equal(f.get_matched_filtered_signal(i), want[k][i])
    # get_signal makes staged signals current
    f.stage_channel_signals(steps[1])
    np.testing.assert_array_equal(f.get_signal(0), steps[1][0])
    # a synchronous setter after a stage: the stage lands first, then the setter
    f.stage_channel_signals(steps[2])
    f.set_channel_signal(1, steps[3][1])
    mixed = steps[2].copy()
    mixed[1] = steps[3][1]
    for c in range(nch):
        np.testing.assert_array_equal(f.get_signal(assign.index(c)), mixed[c])
    # two stages before apply: the second wins
    f.stage_channel_signals(steps[0])
    f.stage_channel_signals(steps[3])
    f.apply()
    for i in range(len(assign)):
        np.testing.assert_array_equal(f.get_matched_filtered_signal(i), want[3][i])
    # a dead channel staged is flagged like a synchronous one
    z = steps[0].copy()
    z[2] = 0.0
    f.stage_channel_signals(z)
    f.apply()
    assert not np.any(f.get_matched_filtered_signal(3))
    f.synchronize()


@pytest.mark.parametrize("L", [16, 100, 500, 1000])
@pytest.mark.parametrize("ntpl", [1, 3, 8])
def test_tensor_core_correlator(gpu, oracle, rng, L, ntpl, capsys):
    """Split-precision tensor-core correlation (correlator_variant 4): the
    FP16 hi+lo Hankel GEMM gives the oracle's FP64 coefficients within the
    1e-4 bound stated for the split-precision form; odd template counts pad
    a group, the last tile is partial, one channel is dead."""
    mf = gpu
    n = 47_111 + L
    t = np.arange(n)
    chans = [rng.standard_normal(n) + 40.0 + 3.0 * np.sin(2 * np.pi * t / 9_000.0 + k) for k in range(3)]
    chans[2][:] = 7.0  # dead
    assign = [c for c in range(3) for _ in range(ntpl)]
    tps = [rng.standard_normal(L) for _ in assign]
    p = _params(mf, tps, n)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, template_channels=assign, n_channels=3, correlator_variant=4)
    f.set_channel_signals(np.stack([c.astype(np.float32) for c in chans]))
    f.apply()
    sig = [chans[c].astype(np.float32) for c in assign]
    ref = oracle.matched_filter(tps, sig, multi=True, fp64_from_f32=True)
    worst = 0.0
    for i, c in enumerate(assign):
        a = f.get_valid_matched_filtered_signal(i).astype(np.float64)
        assert a.size == ref[i].size
        if c == 2:
            assert not np.any(a)
            continue
        worst = max(worst, float(np.max(np.abs(a - ref[i]))))
    with capsys.disabled():
        print("\ntensor-core correlator L=%d templates/channel=%d: max|drho| %.3g" % (L, ntpl, worst))
    assert worst < 1e-4


def test_tensor_core_errors(gpu, rng):
    mf = gpu
    p = _params(mf, [rng.standard_normal(100), rng.standard_normal(120)], 5000)
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    with pytest.raises(ValueError):
        f.initialize(p, correlator_variant=4)  # needs one template length
    g = mf.MultiChannel.MatchedFilter(dtype=np.float64)
    with pytest.raises(ValueError):
        g.initialize(_params(mf, [rng.standard_normal(100)], 5000), correlator_variant=4)  # FP32 only


@pytest.mark.parametrize("variant", [0, 4, 1])
def test_apply_graph_replay(gpu, rng, variant):
    """apply replayed as a CUDA graph gives the direct launches' results
    bit for bit, through staged uploads that alternate the input buffers and
    with candidate gathering on; FFT organisations and tensor cores."""
    mf = gpu
    n, L = 50_000, 200
    assign = [0, 0, 1, 1, 2, 2]
    tps = [rng.standard_normal(L) for _ in assign]
    p = _params(mf, tps, n)
    objs = []
    for graph in (False, True):
        f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
        f.initialize(p, template_channels=assign, n_channels=3, correlator_variant=variant)
        f.set_peak_threshold(0.3)
        f.set_graph(graph)
        objs.append(f)
    plain, graphed = objs
    for step in range(6):
        x = rng.standard_normal((3, n)).astype(np.float32)
        for f in objs:
            f.stage_channel_signals(x)
            f.apply()
            f.find_peaks(0.3, 50)
        for t in range(len(assign)):
            np.testing.assert_array_equal(graphed.get_matched_filtered_signal(t), plain.get_matched_filtered_signal(t))
        for a, b in zip(graphed.get_all_peaks(), plain.get_all_peaks()):
            np.testing.assert_array_equal(a, b)
    assert graphed.graph_launches() >= 2 and plain.graph_launches() == 0
    # same input again: replayed too
    k = graphed.graph_launches()
    graphed.apply()
    assert graphed.graph_launches() == k + 1
