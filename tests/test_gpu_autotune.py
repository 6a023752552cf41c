"""Per-bucket plan overrides (mfgpu_mf_params.bucket_fft_lengths /
bucket_variants) and the measured autotune on top of them: the chosen plans
are the ones asked for, bad overrides fail with the reference's
invalid-argument error, and a tuned object's coefficients match the oracle
and the untuned object's."""
import numpy as np
import pytest

from test_gpu_configs import _bp, _params, _template

pytestmark = pytest.mark.gpu


def _uneven(nt=24, nch=4, n=60_000, seed=200):
    rng = np.random.default_rng(seed)
    lens = rng.integers(200, 2001, nt)
    tps = []
    for t, L in enumerate(lens):
        lo = rng.uniform(1, 7)
        tps.append(_template(1000 + t, int(L), lo, rng.uniform(lo + 2, 15)))
    chan = rng.integers(0, nch, nt)
    sigs = np.stack([_bp(np.random.default_rng(300 + c).standard_normal(n), 1.0, 15.0) for c in range(nch)])
    return tps, chan, sigs.astype(np.float32), n


def _filter(mf, tps, chan, n, nch, **kw):
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(_params(mf, tps, n), template_channels=chan, n_channels=nch, **kw)
    return f


def test_bucket_plan_overrides(gpu, oracle):
    mf = gpu
    tps, chan, sigs, n = _uneven()
    f = _filter(mf, tps, chan, n, sigs.shape[0], length_buckets=2)
    auto = f.get_plan()["bucket_plans"]
    assert len(auto) == 2
    f0 = auto[0]["fft_length"]
    alt = f0 // 2 if f0 >= 8192 else 2 * f0  # FP32 transforms go up to N = 8192
    want = [(alt, 1), (0, 2)]
    f = _filter(mf, tps, chan, n, sigs.shape[0], length_buckets=2, bucket_plans=want)
    got = f.get_plan()["bucket_plans"]
    assert got[0]["fft_length"] == alt and got[0]["correlator"] == 1
    # a forced organisation keeps the automatic choice of FFT length among
    # the lengths where it fits
    assert got[1]["correlator"] == 2
    assert sum(b["templates"] for b in got) == len(tps)
    f.set_channel_signals(sigs)
    f.apply()
    ref = oracle.matched_filter(tps, [sigs[c] for c in chan], multi=True, fp64_from_f32=True)
    worst = max(float(np.max(np.abs(f.get_valid_matched_filtered_signal(t).astype(np.float64) - ref[t])))
                for t in range(len(tps)))
    assert worst < 1e-5, worst


@pytest.mark.parametrize("plans", [[(1000, 0)], [(0, 3)], [(0, 4)], [(0, 5)], [(256, 1), (256, 1), (256, 1)]])
def test_bad_bucket_plans(gpu, plans):
    """Not a power of two; teams or tensor cores for several template
    lengths; an FFT length shorter than the longest template."""
    mf = gpu
    tps, chan, sigs, n = _uneven()
    with pytest.raises(ValueError):
        _filter(mf, tps, chan, n, sigs.shape[0], length_buckets=3, bucket_plans=plans)


def test_autotune_uneven(gpu, oracle):
    mf = gpu
    tps, chan, sigs, n = _uneven()
    f = _filter(mf, tps, chan, n, sigs.shape[0])
    f.set_peak_threshold(0.5)
    res = f.autotune(sigs, repeats=1, max_buckets=2)
    ok = [t for t in res["trials"] if t["apply_ms"] is not None]
    assert len(ok) >= 4
    assert {t["config"]["length_buckets"] for t in ok} == {1, 2}
    assert res["apply_ms"] == min(t["apply_ms"] for t in ok)
    assert all("error" in t for t in res["trials"] if t["apply_ms"] is None)
    # the object is left with the winner, signals loaded
    assert f.get_plan()["bucket_plans"] == res["plan"]["bucket_plans"]
    f.apply()
    ref = oracle.matched_filter(tps, [sigs[c] for c in chan], multi=True, fp64_from_f32=True)
    worst = max(float(np.max(np.abs(f.get_valid_matched_filtered_signal(t).astype(np.float64) - ref[t])))
                for t in range(len(tps)))
    assert worst < 1e-5, worst
    # the peak threshold set before tuning still gathers candidates
    f.find_peaks(0.5, 100)
    g = _filter(mf, tps, chan, n, sigs.shape[0])
    g.set_channel_signals(sigs)
    g.apply()
    g.find_peaks(0.5, 100)
    for t in range(len(tps)):
        np.testing.assert_array_equal(f.get_peaks(t), g.get_peaks(t))


def test_autotune_one_length(gpu, oracle):
    """One template length in FP32: the organisations, FFT lengths and the
    tensor-core correlator are all timed."""
    mf = gpu
    rng = np.random.default_rng(5)
    tps = [_template(50 + t, 300) for t in range(8)]
    nch, n = 2, 50_000
    chan = np.arange(8) % nch
    sigs = np.stack([_bp(rng.standard_normal(n), 1.0, 10.0) for _ in range(nch)]).astype(np.float32)
    f = _filter(mf, tps, chan, n, nch)
    res = f.autotune(sigs, repeats=1)
    ok = [t for t in res["trials"] if t["apply_ms"] is not None]
    assert any(t["config"]["correlator_variant"] == 4 for t in ok)
    assert {t["plan"]["bucket_plans"][0]["correlator"] for t in ok} >= {1, 2, 3, 4}
    f.apply()
    ref = oracle.matched_filter(tps, [sigs[c] for c in chan], multi=True, fp64_from_f32=True)
    worst = max(float(np.max(np.abs(f.get_valid_matched_filtered_signal(t).astype(np.float64) - ref[t])))
                for t in range(len(tps)))
    assert worst < 2e-5, worst
    # the tensor-core tile shapes were timed, each trial at the shape asked for
    tc = [t for t in ok if t["config"]["correlator_variant"] == 4 and t["config"]["tc_group"]]
    assert len({t["plan"]["tc_group"] for t in tc}) >= 3
    assert all(t["plan"]["tc_group"] == t["config"]["tc_group"] for t in tc)


@pytest.mark.parametrize("g", [2, 4, 8, 16])
def test_tensor_core_tile_shape(gpu, oracle, g):
    """tc_group sets the tensor-core correlator's templates per group (MMA
    N = 16 per template); every shape gives oracle-equal coefficients."""
    mf = gpu
    rng = np.random.default_rng(6)
    tps = [_template(70 + t, 240) for t in range(10)]
    nch, n = 2, 40_000
    chan = np.arange(10) % nch
    sigs = np.stack([_bp(rng.standard_normal(n), 1.0, 10.0) for _ in range(nch)]).astype(np.float32)
    f = _filter(mf, tps, chan, n, nch, correlator_variant=4, tc_group=g)
    assert f.get_plan()["correlator"] == 4 and f.get_plan()["tc_group"] == g
    f.set_channel_signals(sigs)
    f.apply()
    ref = oracle.matched_filter(tps, [sigs[c] for c in chan], multi=True, fp64_from_f32=True)
    worst = max(float(np.max(np.abs(f.get_valid_matched_filtered_signal(t).astype(np.float64) - ref[t])))
                for t in range(len(tps)))
    assert worst < 2e-5, worst


@pytest.mark.parametrize("g", [1, 3, 18, -2])
def test_bad_tensor_core_tile_shape(gpu, g):
    mf = gpu
    tps = [_template(90 + t, 240) for t in range(4)]
    with pytest.raises(ValueError):
        _filter(mf, tps, np.arange(4) % 2, 20_000, 2, correlator_variant=4, tc_group=g)
