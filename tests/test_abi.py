"""The C ABI library loads and exports every entry point include/mfgpu.h
declares; host-side API logic that needs no GPU.  No compute calls."""
import ctypes
import os
import pickle
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "mfgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mfgpu_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(mflib):
    from mflib_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = header_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert sorted(_lib.exported_symbols()) == syms


def test_fft_sizes_through_abi(mflib, oracle, rng):
    for nb, nx, expect in ((4500, 75000, (32768, 28269)), (4500, 8640000, (65536, 61037)),
                           (101, 1024, (512, 412))):
        assert mflib.compute_optimal_fft_and_block_length(nb, nx) == expect
    for _ in range(300):
        nb = int(rng.integers(1, 5000))
        nx = int(rng.integers(nb + 1, 20_000_000))
        assert mflib.compute_optimal_fft_and_block_length(nb, nx) == oracle.fft_sizes(nb, nx)
    with pytest.raises(ValueError):
        mflib.compute_optimal_fft_and_block_length(10, 10)
    with pytest.raises(ValueError):
        mflib.compute_optimal_fft_and_block_length(0, 10)


def test_waveform_template_time_errors(mflib):
    # python/waveformTemplate.cpp:135-160: negative onset and travel times are
    # invalid arguments
    wt = mflib.WaveformTemplate()
    wt.set_signal(np.arange(10.0))
    wt.set_sampling_rate(10.0)
    with pytest.raises(ValueError):
        wt.set_phase_travel_time(-1.0)
    with pytest.raises(ValueError):
        wt.set_phase_onset_time_in_signal(-0.1)
    wt.set_phase_travel_time(0.0)
    assert wt.have_travel_time() and wt.get_phase_travel_time() == 0.0


def test_parameters_without_templates(mflib):
    # pymflib's parameters return 0 for the sizes while no template is set
    # (python/multiChannelMatchedFilterParameters.cpp:79-107,
    # python/singleChannel/matchedFilterParameters.cpp:75-103)
    for p in (mflib.MultiChannel.MatchedFilterParameters(), mflib.SingleChannel.MatchedFilterParameters()):
        p.set_signal_size(1000)
        assert p.get_fft_length() == 0 and p.block_length() == 0 and p.get_signal_size() == 0
        wt = mflib.WaveformTemplate()
        wt.set_signal(np.arange(50.0))
        wt.set_sampling_rate(10.0)
        p.add_template(wt)
        assert p.get_signal_size() == 1000 and p.get_fft_length() > 0
        p.clear()
        p.add_template(wt)
        with pytest.raises(RuntimeError):
            p.get_signal_size()  # templates but no size: the reference's getSignalSize throws
        with pytest.raises(RuntimeError):
            p.get_fft_length()


def test_parameters_window_length_vs_reference(mflib, reference, rng):
    """MatchedFilterParameters.get_fft_length / get_block_length follow the
    reference's getFFTLength (computeWindowLength,
    src/matchedFilterParameters.cpp:47-104, :268-300): a signal as long as the
    longest template is accepted; only a shorter one is an error.  Checked
    against the compiled reference's own parameters object."""
    cases = [(100, 100), (1, 1), (2, 2), (4097, 4097), (512, 513), (3000, 2999), (7, 3)]
    cases += [(int(a), int(a + rng.integers(0, 3))) for a in rng.integers(1, 300_000, 150)]
    cases += [(int(a), int(b)) for a, b in zip(rng.integers(1, 5000, 100), rng.integers(1, 200_000, 100))]
    for nb, nx in cases:
        try:
            want = reference.window_length(nb, nx)
        except ValueError:
            want = None
        p = mflib.MultiChannel.MatchedFilterParameters()
        wt = mflib.WaveformTemplate()
        wt.set_signal(np.arange(nb) % 7 - 3.0)
        wt.set_sampling_rate(1.0)
        p.add_template(wt)
        p.set_signal_size(nx)
        if want is None:
            with pytest.raises(ValueError):
                p.get_fft_length()
        else:
            assert (p.get_fft_length(), p.get_block_length()) == want, (nb, nx)


def test_network_station_phase(mflib):
    # python/unit_tests.py:8-35
    nsp = mflib.NetworkStationPhase()
    nsp.set_network("UU")
    nsp.set_station("ALT")
    nsp.set_channel("EHN")
    nsp.set_location_code("01")
    nsp.set_phase("P")
    assert (nsp.get_network(), nsp.get_station(), nsp.get_channel(), nsp.get_location_code(),
            nsp.get_phase()) == ("UU", "ALT", "EHN", "01", "P")
    p = pickle.loads(pickle.dumps(nsp, 2))
    assert p == nsp and p.get_station() == "ALT"
    q = mflib.NetworkStationPhase()
    q.set_network(" uu")
    assert q.get_network() == "UU"


def test_waveform_template(mflib):
    # python/unit_tests.py:37-117
    wt = mflib.WaveformTemplate()
    sig = np.arange(1, 400, 1)
    wt.set_signal(sig)
    assert np.max(np.abs(wt.get_signal() - sig)) == 0
    wt.set_sampling_rate(100)
    assert wt.get_sampling_rate() == 100
    wt.set_shift_and_stack_weight(0.8)
    assert wt.get_shift_and_stack_weight() == 0.8
    wt.set_phase_travel_time(9)
    assert wt.get_phase_travel_time() == 9
    wt.set_phase_onset_time_in_signal(0.5)
    assert wt.get_phase_onset_time_in_signal() == 0.5
    wt.set_magnitude(6)
    assert wt.get_magnitude() == 6
    wt.set_polarity(mflib.Polarity.compression)
    assert wt.get_polarity() == mflib.Polarity.compression
    nsp = mflib.NetworkStationPhase()
    nsp.set_station("FORU")
    wt.set_identifier([nsp, 4])
    idb = wt.get_identifier()
    assert idb[0].get_station() == "FORU" and idb[1] == 4
    cp = pickle.loads(pickle.dumps(wt))
    assert np.max(np.abs(cp.get_signal() - sig)) == 0
    assert cp.get_phase_onset_time_in_signal() == 0.5 and cp.get_identifier()[1] == 4
    wt.clear()
    assert wt.get_shift_and_stack_weight() == 1
    with pytest.raises(ValueError):
        wt.set_sampling_rate(0)
    with pytest.raises(ValueError):
        wt.set_shift_and_stack_weight(1.5)
    with pytest.raises(RuntimeError):
        wt.get_signal()


def test_matched_filter_parameters(mflib):
    # python/unit_tests.py:121-180
    wf1, wf2 = mflib.WaveformTemplate(), mflib.WaveformTemplate()
    p = mflib.MultiChannel.MatchedFilterParameters()
    t1, t2 = np.arange(1, 100, 1), np.arange(1, 95, 1)
    wf1.set_signal(t1)
    wf2.set_signal(t2)
    for w in (wf1, wf2):
        w.set_sampling_rate(100)
        w.set_shift_and_stack_weight(0.8)
        w.set_phase_onset_time_in_signal(0.05)
        w.set_phase_travel_time(4)
    p.add_template(wf1)
    p.add_template(wf2)
    p.set_signal_size(1024)
    assert p.get_number_of_templates() == 2
    assert p.get_fft_length() == 512
    p.set_fft_length(550)
    assert p.get_fft_length() == 550
    for i, t in enumerate((t1, t2)):
        wb = p.get_template(i)
        assert wb.get_sampling_rate() == 100 and wb.get_shift_and_stack_weight() == 0.8
        assert wb.get_phase_onset_time_in_signal() == 0.05 and wb.get_phase_travel_time() == 4
        assert np.max(np.abs(wb.get_signal() - t)) == 0
    p.clear_templates()
    assert p.get_number_of_templates() == 0
    bad = mflib.WaveformTemplate()
    bad.set_signal(t1)
    bad.set_sampling_rate(50)
    p.add_template(wf1)
    with pytest.raises(ValueError):
        p.add_template(bad)


def test_single_channel_parameters(mflib, rng):
    # testing/singleChannel.cpp:28-102
    p = mflib.SingleChannel.MatchedFilterParameters()
    p.set_signal_size(3823)
    assert p.get_detection_mode() == mflib.MatchedFilterDetectionMode.single_channel
    assert not p.is_valid()
    for L in (410, 411):
        wt = mflib.WaveformTemplate()
        wt.set_signal(rng.uniform(-1, 1, L))
        wt.set_sampling_rate(1)
        p.add_template(wt)
    assert p.get_max_template_length() == 411 and p.is_valid()
    p.clear_templates()
    assert p.get_number_of_templates() == 0
    p.clear()
    assert not p.is_valid()


def test_single_channel_detection(mflib, rng):
    # python/unit_tests.py:328-457: every field's have / set / get, the same
    # object through an alias, and a pickle round trip (which here also
    # carries the detected signal)
    sc, rmt = mflib.SingleChannel, mflib.RelativeMagnitudeType
    nsp = mflib.NetworkStationPhase()
    nsp.set_network("UU")
    nsp.set_station("CMU")
    nsp.set_channel("EHZ")
    nsp.set_location_code("01")
    nsp.set_phase("P")
    xt = rng.uniform(5, 7, 400)
    d = sc.Detection()
    fields = [("phase_onset_time", 4.0), ("interpolated_phase_onset_time", 9.0), ("detection_time", 2.0),
              ("interpolated_detection_time", 3.0), ("travel_time", 13.0), ("correlation_coefficient", 0.3)]
    assert not d.have_template_identifier()
    d.set_template_identifier([nsp, 204])
    for name, v in fields:
        assert not getattr(d, "have_" + name)()
        getattr(d, "set_" + name)(v)
        assert getattr(d, "have_" + name)() and getattr(d, "get_" + name)() == v
    assert not d.have_amplitude_scaling_factor()
    d.set_amplitude_scaling_factor(9, rmt.gibbons_ringdal_2006)
    assert not d.have_amplitude_scaling_factor()  # pymflib: true once both are set
    d.set_amplitude_scaling_factor(10, rmt.schaff_richards_2014)
    assert d.have_amplitude_scaling_factor() and d.have_amplitude_scaling_factor(rmt.schaff_richards_2014)
    with pytest.raises(ValueError):
        d.set_amplitude_scaling_factor(0.0, rmt.gibbons_ringdal_2006)
    with pytest.raises(ValueError):
        d.set_correlation_coefficient(1.5)
    # pymflib refuses negative times (python/singleChannel/detection.cpp:191-290)
    for name in ("detection_time", "interpolated_detection_time", "phase_onset_time",
                 "interpolated_phase_onset_time", "travel_time"):
        with pytest.raises(ValueError):
            getattr(d, "set_" + name)(-1.0)
    assert not d.have_detected_signal()
    d.set_detected_signal(xt)
    assert d.have_detected_signal() and np.max(np.abs(d.get_detected_signal() - xt)) < 1e-14
    for e in (d, pickle.loads(pickle.dumps(d, 2))):
        ident = e.get_template_identifier()
        assert ident[1] == 204
        assert [ident[0].get_network(), ident[0].get_station(), ident[0].get_channel(),
                ident[0].get_location_code(), ident[0].get_phase()] == ["UU", "CMU", "EHZ", "01", "P"]
        for name, v in fields:
            assert getattr(e, "get_" + name)() == v
        assert e.get_amplitude_scaling_factor(rmt.gibbons_ringdal_2006) == 9
        assert e.get_amplitude_scaling_factor(rmt.schaff_richards_2014) == 10
        assert np.max(np.abs(e.get_detected_signal() - xt)) < 1e-14


def test_single_channel_detector_parameters(mflib):
    # python/unit_tests.py:459-489, with pymflib's spelling of the maxima
    # policy enumeration (python/pymflib.cpp:29)
    p = mflib.SingleChannel.DetectorParameters()
    p.set_maxima_policy(mflib.MaxmimumMatchedFilterPolicy.absolute_maximum)
    p.set_matched_filtered_signal_detector_policy(mflib.MatchedFilteredSignalDetectorPolicy.single)
    p.set_minimum_detection_spacing(5)
    p.set_detection_threshold(0.5)
    p.enable_save_detected_waveform()
    p.disable_save_amplitude_scaling_factor()
    for q in (p, p):
        assert q.get_maxima_policy() == mflib.MaxmimumMatchedFilterPolicy.absolute_maximum
        assert q.get_maxima_policy() == mflib.MaximumMatchedFilterPolicy.absolute_maximum
        assert q.get_minimum_detection_spacing() == 5 and q.get_detection_threshold() == 0.5
        assert q.want_detected_waveform() and not q.want_amplitude_scaling_factor()
        assert q.get_matched_filtered_signal_detector_policy() == mflib.MatchedFilteredSignalDetectorPolicy.single


def test_single_channel_associator_parameters(mflib):
    # python/unit_tests.py:491-507
    p = mflib.SingleChannel.AssociatorParameters()
    p.set_origin_time_tolerance(0.5)
    p.set_minimum_number_of_picks_in_event(8)
    p.enable_correlation_coefficient_weighting()
    for q in (p, p):
        assert q.get_origin_time_tolerance() == 0.5
        assert q.get_minimum_number_of_picks_in_event() == 8
        assert q.use_correlation_coefficient_weighting()


def test_weighted_statistics_known_answers(mflib):
    # testing/associator.cpp:36-78 (values from R's spatstat weighted.median)
    from mflib_gb300.associator import mean, median, weighted_mean, weighted_median
    x = [1.1, 5.3, 3.7, 2.1, 7.0, 9.9]
    w = [1.1, 0.4, 2.1, 3.5, 1.2, 0.8]
    xp = [0.1, 0.35, 0.05, 0.1, 0.15, 0.05, 0.2]
    assert abs(weighted_median(x, w) - 2.085714) < 1e-6
    assert abs(weighted_median(xp, xp) - 0.1625) < 1e-6
    assert abs(weighted_median(xp[:-1], xp[:-1]) - 0.1333333) < 1e-6
    assert abs(weighted_median([1, 2], [1, 4]) - 1.375) < 1e-6
    assert weighted_median(x[:1], w[:1]) == x[0]
    assert abs(median(x) - 4.5) < 1e-6 and abs(median(x[:-1]) - 3.7) < 1e-6 and median(x[:1]) == x[0]
    assert abs(weighted_mean(xp, xp) - 0.21) < 1e-6 and weighted_mean(x[:1], x[:1]) == x[0]
    assert abs(mean(xp) - 0.1428571) < 1e-6 and mean(x[:1]) == x[0]
    # empty input and no weights, as the reference's helpers
    assert median([]) == mean([]) == weighted_median([], None) == weighted_mean([], None) == 0.0
    assert weighted_median(x) == median(x) and weighted_mean(x) == mean(x)
