"""The CPU oracle pinned against the reference's own golden vectors and
known-answer tests (and, where it was compiled here, against the reference
itself).  No GPU."""
import numpy as np
import pytest


# FFT sizing: testing/matchedFilterParameters.cpp:14-33, :82-89; python/unit_tests.py:159
@pytest.mark.parametrize("nb,nx,expect", [
    (4500, 75000, (32768, 28269)),
    (4500, 8640000, (65536, 61037)),
    (101, 1024, (512, 412)),
    (99, 1024, (512, 414)),
])
def test_fft_sizes_golden(oracle, nb, nx, expect):
    assert oracle.fft_sizes(nb, nx) == expect


def test_fft_sizes_errors(oracle):
    with pytest.raises(ValueError):
        oracle.fft_sizes(0, 10)
    with pytest.raises(ValueError):
        oracle.fft_sizes(10, 10)


def test_fft_sizes_vs_reference(oracle, reference, rng):
    for _ in range(200):
        nb = int(rng.integers(1, 5000))
        nx = int(rng.integers(nb + 1, 10_000_000))
        assert oracle.fft_sizes(nb, nx) == reference.fft_sizes(nb, nx)


def damped_case(signal_size=1000):
    """testing/matchedFilter.cpp:63-90 (damped sine/cosine, 2 s template)."""
    tmax = 8.0
    dt = tmax / (signal_size - 1)
    f0 = 4.0 / tmax
    t = np.arange(signal_size) * dt
    x = 2 * np.exp(-0.1 * t) * np.sin(2 * np.pi * f0 * t)
    x2 = 2 * np.exp(-0.15 * t) * np.cos(2 * np.pi * f0 * t)
    nb = int(2.0 / dt + 0.5) + 1
    tb = np.arange(nb) * dt
    return x, x2, np.sin(2 * np.pi * f0 * tb), np.cos(2 * np.pi * f0 * tb)


def test_mf_double_known_answer(oracle):
    # testing/matchedFilter.cpp:58-168: < 1e-13 vs the naive Pearson correlation
    x, x2, b, b2 = damped_case()
    out = oracle.matched_filter([b, b2, b, b2], [x, x2, x, x2], multi=True)
    for r, tp, sg in zip(out, [b, b2, b, b2], [x, x2, x, x2]):
        ref = oracle.pearson_naive(tp, sg)
        assert np.max(np.abs(r - ref)) < 1e-13


def test_mf_float_known_answer(oracle):
    # testing/matchedFilter.cpp:172-271: < 2e-6 in float
    x, x2, b, b2 = damped_case()
    out = oracle.matched_filter([b, b2], [x, x2], multi=True, dtype=np.float32)
    for r, tp, sg in zip(out, [b, b2], [x, x2]):
        ref = oracle.pearson_naive(tp.astype(np.float32), sg.astype(np.float32))
        assert np.max(np.abs(r.astype(np.float64) - ref)) < 2e-6


def test_mf_single_channel_uneven(oracle, rng):
    # testing/singleChannel.cpp:104-160 (U(2,3) signal, templates cut from it)
    wave = rng.uniform(2, 3, 4000)
    tps = [wave[25:155], wave[1124:1264], wave[3601:3726]]
    out = oracle.matched_filter(tps, [wave], multi=False)
    for r, tp in zip(out, tps):
        assert np.max(np.abs(r - oracle.pearson_naive(tp, wave))) < 1e-12


def test_mf_vs_reference(oracle, reference, rng):
    for multi in (True, False):
        sig = [rng.standard_normal(3000) + 5.0 for _ in range(3 if multi else 1)]
        tps = [rng.standard_normal(L) for L in (90, 150, 200)]
        a = oracle.matched_filter(tps, sig, multi=multi)
        b = reference.matched_filter(tps, sig, multi=multi)
        for x, y in zip(a, b):
            assert np.max(np.abs(x - y)) < 1e-12
        af = oracle.matched_filter(tps[:1] * 2, [s.astype(np.float32) for s in sig[:2]] if multi else
                                   [sig[0].astype(np.float32)], multi=multi, dtype=np.float32)
        bf = reference.matched_filter(tps[:1] * 2, [s.astype(np.float32) for s in sig[:2]] if multi else
                                      [sig[0].astype(np.float32)], multi=multi, dtype=np.float32)
        for x, y in zip(af, bf):
            assert np.max(np.abs(x - y)) < 1e-5


def gaussian_sine(tdur=4.0, dt=0.01, sigma=1.2, freq=12.0):
    """testing/peakFinder.cpp:145-170."""
    t0, t1 = -tdur / 2, tdur / 2
    npts = int((t1 - t0) / dt + 0.5) + 1
    t = t0 + np.arange(npts) * dt
    y = np.exp(-((t / sigma) ** 2) ** 2) * np.cos(2 * np.pi * (t - t0) / tdur * freq)
    y = y / np.max(np.abs(y))
    y[0] = 0
    y[-1] = 0
    return y


def peak_signal(n=4000):
    """Signal layout of testing/peakFinder.cpp:38-54."""
    tp = gaussian_sine()
    sig = np.zeros(n)
    ih = tp.size // 2
    sig[: tp.size - ih] = tp[ih:]
    for frac in (0.25, 0.5, 0.75):
        i1 = int(n * frac) - ih
        sig[i1:i1 + tp.size] = tp
    i1 = n - ih
    sig[i1:i1 + ih] = tp[1:ih + 1]
    return sig


PEAKS_13 = [0, 67, 1000 - 67, 1000, 1000 + 67, 2000 - 67, 2000, 2000 + 67, 3000 - 67, 3000, 3000 + 67,
            4000 - 1 - 67, 4000 - 1]
PEAKS_21 = [0, 33, 67, 1000 - 67, 1000 - 33, 1000, 1000 + 33, 1000 + 67, 2000 - 67, 2000 - 33, 2000, 2000 + 33,
            2000 + 67, 3000 - 67, 3000 - 33, 3000, 3000 + 33, 3000 + 67, 4000 - 1 - 67, 4000 - 1 - 33, 4000 - 1]


def test_peaks_golden(oracle):
    # testing/peakFinder.cpp:16-143
    assert oracle.peaks(np.full(4000, 0.4), 0.8, 52).size == 0
    sig = peak_signal()
    np.testing.assert_array_equal(oracle.peaks(sig, 0.8, int(0.5 / 0.01 + 1) + 1), PEAKS_13)
    np.testing.assert_array_equal(oracle.peaks(sig, 0.8, 0), PEAKS_21)


def test_peaks_vs_reference(oracle, reference, rng):
    for _ in range(20):
        n = int(rng.integers(2, 20000))
        x = rng.standard_normal(n)
        thr = float(rng.uniform(0, 1))
        md = int(rng.integers(0, 300))
        np.testing.assert_array_equal(oracle.peaks(x, thr, md), reference.peaks(x, thr, md))


DBSCAN_X = np.array([[1, 2], [2, 2], [2, 2], [8, 7], [8, 8], [25, 80]], dtype=float)


def test_dbscan_golden(oracle):
    # testing/dbscan.cpp:8-60
    ncl, lab = oracle.dbscan(DBSCAN_X, 3, 2)
    assert ncl == 2
    np.testing.assert_array_equal(lab, [0, 0, 0, 1, 1, -1])
    ncl, lab = oracle.dbscan(DBSCAN_X[:5], 3, 2)
    assert ncl == 2
    np.testing.assert_array_equal(lab, [0, 0, 0, 1, 1])


def test_dbscan_vs_sklearn(oracle, rng):
    sk = pytest.importorskip("sklearn.cluster")
    for nf in (1, 2, 3):
        for _ in range(5):
            X = rng.uniform(0, 20, (int(rng.integers(5, 300)), nf))
            eps = float(rng.uniform(0.5, 3))
            mo = int(rng.integers(1, 6))
            w = rng.uniform(0.2, 2.0, X.shape[0])
            for weights in (None, w):
                ncl, lab = oracle.dbscan(X, eps, mo, weights)
                ref = sk.DBSCAN(eps=eps, min_samples=mo).fit(X, sample_weight=weights).labels_
                assert ncl == (ref.max() + 1 if ref.size else 0)
                np.testing.assert_array_equal(lab, ref)


def dbscan_1d(x, eps, min_obs, weights=None):
    """DBSCAN over one feature by sorting, for sizes where the oracle's
    all-pairs scans take too long.  Exact where |x_i - x_j| and the weight
    sums are exact (values on a binary grid): the eps-neighbourhood of a
    point is a contiguous range of the sorted values; the clusters are the
    runs of sorted core points with gaps <= eps, numbered by their smallest
    index; a border point takes the smallest cluster number among the core
    points in its range (the oracle's index-order expansion gives the same).
    Pinned against the oracle in test_dbscan_1d_checker."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    if n == 0:
        return 0, np.zeros(0, np.int32)
    order = np.argsort(x, kind="stable")
    xs = x[order]
    lo = np.searchsorted(xs, xs - eps, side="left")
    hi = np.searchsorted(xs, xs + eps, side="right")
    w = np.ones(n) if weights is None else np.asarray(weights, np.float64)[order]
    cw = np.concatenate([[0.0], np.cumsum(w)])
    core = (cw[hi] - cw[lo]) >= min_obs
    cpos = np.flatnonzero(core)
    labels_s = np.full(n, -1, np.int64)
    if cpos.size:
        new = np.concatenate([[True], np.diff(xs[cpos]) > eps])
        comp = np.cumsum(new) - 1
        first = np.full(comp[-1] + 1, n, np.int64)
        np.minimum.at(first, comp, order[cpos])
        ids = np.argsort(np.argsort(first, kind="stable"), kind="stable")
        cid = np.full(n + 1, np.iinfo(np.int64).max, np.int64)
        cid[cpos] = ids[comp]
        idx = np.empty(2 * n, np.int64)
        idx[0::2], idx[1::2] = lo, hi
        best = np.minimum.reduceat(cid, idx)[0::2]
        labels_s = np.where(best == np.iinfo(np.int64).max, -1, best)
        ncl = int(comp[-1] + 1)
    else:
        ncl = 0
    labels = np.empty(n, np.int32)
    labels[order] = labels_s
    return ncl, labels


def test_dbscan_1d_checker(oracle, rng):
    for _ in range(12):
        n = int(rng.integers(1, 1500))
        x = np.round(rng.uniform(0, 200, n) * 4) / 4
        eps = float(rng.integers(1, 12)) / 4
        mo = int(rng.integers(1, 9))
        w = rng.integers(1, 7, n) / 2.0
        for weights in (None, w):
            assert dbscan_1d(x, eps, mo, weights)[0] == oracle.dbscan(x, eps, mo, weights)[0]
            np.testing.assert_array_equal(dbscan_1d(x, eps, mo, weights)[1], oracle.dbscan(x, eps, mo, weights)[1])


def _golden_detector():
    import os
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "detector_golden.npz")))


@pytest.mark.parametrize("single", [0, 1])
@pytest.mark.parametrize("interp", [0, 1, 2])
@pytest.mark.parametrize("absm", [0, 1])
def test_detector_oracle_vs_golden(oracle, single, interp, absm):
    """The detector restatement (orc_detect_d) on the oracle's FP64 traces
    reproduces the reference's own SingleChannel::Detector<double> output
    stored in tests/golden/detector_golden.npz (generated by
    make_detector_golden.py from the reference compiled unchanged): the
    same detections in the same order, times and coefficients to 1e-12,
    polarity, amplitude scaling factors to 1e-12 relative."""
    g = _golden_detector()
    tps = list(g["templates"])
    x = g["signal"]
    fs = float(g["fs"])
    rho = np.stack(oracle.matched_filter(tps, [x] * len(tps), multi=False, dtype=np.float64))
    o = oracle.detect(rho, tps, [x] * len(tps), fs, threshold=float(g["threshold"]),
                      min_distance=int(g["min_distance"]), single=single, interpolation=interp,
                      absolute_maximum=absm)
    key = "s%d_i%d_a%d_" % (single, interp, absm)
    assert g[key + "template"].size > 5
    np.testing.assert_array_equal(o["template"], g[key + "template"])
    np.testing.assert_allclose(o["time"], g[key + "time"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(o["interpolated_time"], g[key + "interpolated_time"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(o["correlation"], g[key + "correlation"], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(o["sign"], g[key + "polarity"])  # templates carry COMPRESSION (+1)
    np.testing.assert_array_equal(o["have_amplitude"], g[key + "have_amplitude"])
    np.testing.assert_allclose(o["gibbons_ringdal"], g[key + "gibbons_ringdal"], rtol=1e-12)
    np.testing.assert_allclose(o["schaff_richards"], g[key + "schaff_richards"], rtol=1e-12)


def test_detector_oracle_vs_reference(oracle, reference, rng):
    """Random cases against the compiled reference detector (FP64), every
    option combination; where the checkout exists."""
    from scipy.signal.windows import hann
    for trial in range(3):
        nt = int(rng.integers(1, 5))
        L = int(rng.integers(50, 400))
        tps = [rng.standard_normal(L) * hann(L) for _ in range(nt)]
        n = int(rng.integers(3_000, 12_000))
        x = rng.standard_normal(n)
        for t in range(nt):
            for o in rng.integers(0, n - L, 3):
                x[o:o + L] += rng.choice([-1.5, 1.5]) * tps[t]
        rho = np.stack(oracle.matched_filter(tps, [x] * nt, multi=False, dtype=np.float64))
        for single in (0, 1):
            for interp in (0, 1, 2):
                for absm in (0, 1):
                    kw = dict(threshold=0.4, min_distance=int(rng.integers(0, 200)), single=single,
                              interpolation=interp, absolute_maximum=absm, alpha=int(rng.integers(3, 60)),
                              npts=int(rng.integers(5, 120)))
                    r = reference.detect(tps, x, 50.0, dtype=np.float64, **kw)
                    o = oracle.detect(rho, tps, [x] * nt, 50.0, **kw)
                    np.testing.assert_array_equal(o["template"], r["template"])
                    np.testing.assert_allclose(o["interpolated_time"], r["interpolated_time"], rtol=0, atol=1e-12)
                    np.testing.assert_allclose(o["gibbons_ringdal"], r["gibbons_ringdal"], rtol=1e-11)


def test_associate_known_answer(oracle):
    """Associator<T>::associate restatement on a hand-made case: event 7 has
    picks whose origin times form two groups of 3 (0.0..0.2 s and 10.0..10.4
    s) and one straggler at 30 s; event 3 has 2 picks (below min_picks 3)."""
    evid = [7, 7, 3, 7, 7, 7, 3, 7, 7]
    travel = [1.0, 2.0, 5.0, 3.0, 1.0, 2.0, 5.0, 4.0, 1.0]
    origin = [0.0, 0.1, 50.0, 0.2, 10.0, 10.2, 50.5, 10.4, 30.0]
    onset = [o + t for o, t in zip(origin, travel)]
    order, events = oracle.associate(evid, onset, travel, [1.0] * 9, tol=0.5, min_picks=3)
    # sorted by event id, then onset: event 3 first
    assert [evid[i] for i in order] == [3, 3, 7, 7, 7, 7, 7, 7, 7]
    assert len(events) == 2
    got = [(e, sorted(origin[order[k]] for k in m)) for e, m in events]
    assert got == [(7, [0.0, 0.1, 0.2]), (7, [10.0, 10.2, 10.4])]


def test_relative_amplitudes_vs_reference(oracle, reference, rng):
    """The amplitude restatement against RelativeMagnitude<double> compiled
    unchanged (where the checkout exists)."""
    for _ in range(20):
        L = int(rng.integers(2, 600))
        b = rng.standard_normal(L) + rng.uniform(-3, 3)
        y = rng.uniform(0.1, 10) * (b + 0.3 * rng.standard_normal(L)) + rng.uniform(-50, 50)
        g0, s0 = reference.relative_amplitudes(b, y)
        gr, sr, ok = oracle.relative_amplitudes(b, y[None, :])
        assert ok[0]
        np.testing.assert_allclose([gr[0], sr[0]], [g0, s0], rtol=1e-12)


def test_detection_pickling():
    import pickle
    import mflib_gb300 as mf
    from mflib_gb300.detector import Detection, RelativeMagnitudeType
    d = Detection()
    nsp = mf.NetworkStationPhase()
    nsp.set_network("UU")
    d.set_template_identifier((nsp, 12))
    d.set_correlation_coefficient(-0.75)
    d.set_detection_time(10.5)
    d.set_interpolated_detection_time(10.52)
    d.set_travel_time(3.0)
    d.set_polarity(mf.Polarity.dilatation)
    d.set_amplitude_scaling_factor(2.5, RelativeMagnitudeType.gibbons_ringdal_2006)
    d.set_detected_signal(np.arange(5.0))
    e = pickle.loads(pickle.dumps(d))
    assert e.get_template_identifier()[0].get_network() == "UU" and e.get_template_identifier()[1] == 12
    assert e.get_correlation_coefficient() == -0.75 and e.get_interpolated_detection_time() == 10.52
    assert e.get_polarity() == mf.Polarity.dilatation and e.get_travel_time() == 3.0
    assert e.get_amplitude_scaling_factor(RelativeMagnitudeType.gibbons_ringdal_2006) == 2.5
    assert not e.have_amplitude_scaling_factor(RelativeMagnitudeType.schaff_richards_2014)
    np.testing.assert_array_equal(e.get_detected_signal(), np.arange(5.0))
    assert not e.have_phase_onset_time()
