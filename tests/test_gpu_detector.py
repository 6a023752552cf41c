"""Single-channel detector on the GPU (mfgpu_mf_detect through
SingleChannel.Detector): against the reference's own detector output
(tests/golden/detector_golden.npz) and against the oracle restatement run on
the GPU's own Pearson traces, for every option combination."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "detector_golden.npz")


def _filter(mf, tps, x, dtype, fs):
    p = mf.SingleChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(fs)
        wt.set_polarity(mf.Polarity.compression)
        p.add_template(wt)
    p.set_signal_size(x.size)
    f = mf.SingleChannel.MatchedFilter(dtype=dtype)
    f.initialize(p)
    f.set_signal(x.astype(dtype))
    f.apply()
    return f


def _detect(mf, f, single, interp, absm, thr, mind, alpha=51, npts=100, amplitudes=True):
    from mflib_gb300 import detector as D
    prm = mf.SingleChannel.DetectorParameters()
    prm.set_detection_threshold(thr)
    prm.set_minimum_detection_spacing(mind)
    prm.set_matched_filtered_signal_detector_policy(single)
    prm.set_maxima_policy(absm)
    ip = mf.SingleChannel.DetectionTimeInterpolationParameters()
    {0: ip.enable_lanczos, 1: ip.enable_quadratic, 2: ip.disable_interpolation}[interp]()
    ip.set_lanczos_alpha(alpha)
    ip.set_lanczos_number_of_interpolation_points(npts)
    prm.set_detection_time_interpolation_parameters(ip)
    if not amplitudes:
        prm.disable_save_amplitude_scaling_factor()
    det = mf.SingleChannel.Detector()
    det.initialize(prm)
    det.detect(f)
    ds = det.get_detections()
    gr = D.RelativeMagnitudeType.gibbons_ringdal_2006
    sr = D.RelativeMagnitudeType.schaff_richards_2014
    return {
        "template": np.array([d.get_template_identifier()[1] for d in ds], dtype=np.int64),
        "time": np.array([d.get_detection_time() for d in ds]),
        "interpolated_time": np.array([d.get_interpolated_detection_time() for d in ds]),
        "correlation": np.array([d.get_correlation_coefficient() for d in ds]),
        "polarity": np.array([int(d.get_polarity()) for d in ds]),
        "have_amplitude": np.array([int(d.have_amplitude_scaling_factor(gr)) for d in ds]),
        "gibbons_ringdal": np.array([d.get_amplitude_scaling_factor(gr) if d.have_amplitude_scaling_factor(gr)
                                     else 0.0 for d in ds]),
        "schaff_richards": np.array([d.get_amplitude_scaling_factor(sr) if d.have_amplitude_scaling_factor(sr)
                                     else 0.0 for d in ds]),
    }


@pytest.mark.parametrize("single", [0, 1])
@pytest.mark.parametrize("interp", [0, 1, 2])
@pytest.mark.parametrize("absm", [0, 1])
def test_detector_vs_reference_golden(gpu, single, interp, absm):
    """FP64 end to end (matched filter + detector on the GPU) against the
    reference's SingleChannel::Detector<double> on the same inputs."""
    mf = gpu
    g = dict(np.load(GOLDEN))
    tps = list(g["templates"])
    f = _filter(mf, tps, g["signal"], np.float64, float(g["fs"]))
    got = _detect(mf, f, single, interp, absm, float(g["threshold"]), int(g["min_distance"]))
    key = "s%d_i%d_a%d_" % (single, interp, absm)
    np.testing.assert_array_equal(got["template"], g[key + "template"])
    np.testing.assert_allclose(got["time"], g[key + "time"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["interpolated_time"], g[key + "interpolated_time"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got["correlation"], g[key + "correlation"], rtol=0, atol=1e-10)
    np.testing.assert_array_equal(got["polarity"], g[key + "polarity"])
    np.testing.assert_array_equal(got["have_amplitude"], g[key + "have_amplitude"])
    np.testing.assert_allclose(got["gibbons_ringdal"], g[key + "gibbons_ringdal"], rtol=1e-10)
    np.testing.assert_allclose(got["schaff_richards"], g[key + "schaff_richards"], rtol=1e-10)


def _case(rng, nt, lens, n):
    from scipy.signal.windows import hann
    tps = [rng.standard_normal(L) * hann(L) for L in lens]
    x = rng.standard_normal(n)
    for t in range(nt):
        for o in rng.integers(0, n - lens[t], 5):
            x[o:o + lens[t]] += rng.choice([-2.0, 2.0]) * tps[t]
    return tps, x


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("single", [0, 1])
@pytest.mark.parametrize("interp", [0, 1, 2])
@pytest.mark.parametrize("absm", [0, 1])
def test_detector_vs_oracle(gpu, oracle, rng, dtype, single, interp, absm):
    """The GPU detector against the restatement on the GPU's own traces:
    the same detections, coefficients and polarities exactly; quadratic
    refinements to rounding; Lanczos refinements on the same grid point for
    nearly all detections and never more than one point apart; amplitudes
    to 1e-9 relative."""
    mf = gpu
    nt = 4
    tps, x = _case(rng, nt, [180, 250, 250, 97], 40_000)
    fs = 40.0
    f = _filter(mf, tps, x, dtype, fs)
    alpha, npts = 17, 64
    got = _detect(mf, f, single, interp, absm, 0.35, 60, alpha=alpha, npts=npts)
    rho = np.stack([f.get_matched_filtered_signal(t) for t in range(nt)]).astype(dtype)
    xs = [x.astype(dtype)] * nt
    o = oracle.detect(rho, tps, xs, fs, threshold=0.35, min_distance=60, single=single, interpolation=interp,
                      absolute_maximum=absm, alpha=alpha, npts=npts)
    assert o["template"].size > 10
    np.testing.assert_array_equal(got["template"], o["template"])
    np.testing.assert_array_equal(got["time"], o["time"])
    np.testing.assert_array_equal(got["correlation"], o["correlation"])
    np.testing.assert_array_equal(got["polarity"], o["sign"])
    d = np.abs(got["interpolated_time"] - o["interpolated_time"])
    if interp == 0:
        step = 1.0 / fs / npts
        assert np.all(d <= step * 1.01), d.max()
        assert np.mean(d <= 1e-9) >= 0.9
    else:
        tol = 1e-12 if dtype == np.float64 else 2e-7 / fs
        assert np.all(d <= tol), d.max()
    np.testing.assert_array_equal(got["have_amplitude"], o["have_amplitude"])
    np.testing.assert_allclose(got["gibbons_ringdal"], o["gibbons_ringdal"], rtol=1e-9)
    np.testing.assert_allclose(got["schaff_richards"], o["schaff_richards"], rtol=1e-9)


def test_detector_errors_and_waveforms(gpu, rng):
    mf = gpu
    tps, x = _case(rng, 2, [120, 120], 8_000)
    det = mf.SingleChannel.Detector()
    with pytest.raises(ValueError):
        det.detect(_filter(mf, tps, x, np.float32, 100.0))  # not initialized
    prm = mf.SingleChannel.DetectorParameters()
    with pytest.raises(ValueError):
        prm.set_detection_threshold(0.0)
    prm.set_detection_threshold(0.4)
    prm.enable_save_detected_waveform()
    det.initialize(prm)
    f = _filter(mf, tps, x, np.float64, 100.0)
    det.detect(f)
    assert det.get_number_of_detections() > 0
    d = det.get_detection(0)
    t = int(round(d.get_detection_time() * 100.0))
    np.testing.assert_array_equal(d.get_detected_signal(), x[t:t + 120])
    with pytest.raises(ValueError):
        det.get_detection(det.get_number_of_detections())


def test_pymflib_relative_magnitude(gpu, rng):
    # python/unit_tests.py:301-326 (and testing/relativeMagnitude.cpp:21-62 at
    # 1e-12): both magnitude perturbations of random windows equal their
    # closed forms over the demeaned signals to 1e-14
    mf = gpu
    xt, yt = rng.uniform(5, 7, 355), rng.uniform(-2, 1, 355)
    wt = mf.WaveformTemplate()
    wt.set_sampling_rate(100.0)
    wt.set_signal(xt)
    rm = mf.SingleChannel.RelativeMagnitude()
    rm.initialize(wt)
    assert rm.is_initialized() and rm.get_detected_signal_length() == 355
    rm.set_detected_signal(yt)
    assert rm.have_detected_signal()
    xd, yd = xt - xt.mean(), yt - yt.mean()
    gr = np.log10(abs(xd @ yd) / (xd @ xd))
    sr = 0.5 * np.log10((yd @ yd) / (xd @ xd))
    assert abs(rm.compute_magnitude_perturbation(mf.RelativeMagnitudeType.gibbons_ringdal_2006) - gr) < 1e-14
    assert abs(rm.compute_magnitude_perturbation(mf.RelativeMagnitudeType.schaff_richards_2014) - sr) < 1e-14


def test_detections_survive_wire_records(gpu, rng):
    """The GPU detector's detections (detected waveforms, amplitudes,
    interpolated times, polarities) through the MPI wire records
    (mflib_gb300.mpi) come back field for field; float32 signals round to
    float32."""
    from mflib_gb300 import mpi
    mf = gpu
    tps, x = _case(rng, 3, [120, 200, 160], 20_000)
    prm = mf.SingleChannel.DetectorParameters()
    prm.set_detection_threshold(0.3)
    prm.enable_save_detected_waveform()
    det = mf.SingleChannel.Detector()
    det.initialize(prm)
    det.detect(_filter(mf, tps, x, np.float64, 100.0))
    ds = det.get_detections()
    assert len(ds) > 2 and all(d.have_detected_signal() for d in ds)
    for dtype in (np.float64, np.float32):
        recs, sig = mpi.pack_detections(ds, dtype)
        got = mpi.unpack_detections(recs, sig)
        for a, b in zip(ds, got):
            sa, sb = a.__getstate__(), b.__getstate__()
            sa["sig"] = np.asarray(sa["sig"], dtype).tolist()
            assert sa == sb


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_relative_magnitude(gpu, oracle, rng, dtype):
    """RelativeMagnitude on the GPU against the restatement (pinned to the
    reference's RelativeMagnitude<double>), one window and a batch."""
    mf = gpu
    L = 333
    b = rng.standard_normal(L)
    wt = mf.WaveformTemplate()
    wt.set_signal(b)
    wt.set_sampling_rate(100.0)
    rm = mf.SingleChannel.RelativeMagnitude(dtype=dtype)
    with pytest.raises(RuntimeError):
        rm.compute_amplitude_scaling_factor(0)
    rm.initialize(wt)
    ys = (rng.uniform(0.1, 5, (50, 1)) * (b + 0.2 * rng.standard_normal((50, L))) + 7.0).astype(dtype)
    gr, sr, ok = rm.amplitude_scaling_factors(ys)
    g0, s0, ok0 = oracle.relative_amplitudes(b, ys.astype(np.float64))
    assert ok.all() and ok0.all()
    np.testing.assert_allclose(gr, g0, rtol=1e-10)
    np.testing.assert_allclose(sr, s0, rtol=1e-10)
    rm.set_detected_signal(ys[3])
    assert abs(rm.compute_amplitude_scaling_factor(mf.RelativeMagnitudeType.gibbons_ringdal_2006) - g0[3]) <= 1e-10 * g0[3]
    assert abs(rm.compute_magnitude_perturbation(mf.RelativeMagnitudeType.schaff_richards_2014)
               - np.log10(s0[3])) < 1e-9
    with pytest.raises(ValueError):
        rm.set_detected_signal(np.full(L, 3.0, dtype=dtype))  # constant window
    with pytest.raises(ValueError):
        rm.set_detected_signal(ys[0, :10])
