"""Peak finder and DBSCAN on the GPU against the oracle and the reference's
golden vectors.  Indices and labels are compared exactly."""
import numpy as np
import pytest

from test_oracle import DBSCAN_X, PEAKS_13, PEAKS_21, dbscan_1d, peak_signal

pytestmark = pytest.mark.gpu


def _peaks(mf, x, thr, md, dtype=np.float64):
    pf = mf.PeakFinder(dtype=dtype)
    pf.set_threshold(thr)
    pf.set_minimum_peak_distance(md)
    pf.set_signal(x)
    pf.apply()
    return pf.get_peak_indices()


def test_peak_finder_golden(gpu):
    # testing/peakFinder.cpp:16-143
    mf = gpu
    pf = mf.PeakFinder()
    assert abs(pf.get_threshold() - 0.7) < 1e-14
    pf.set_threshold(0.8)
    pf.set_minimum_peak_distance(52)
    assert pf.get_minimum_peak_distance() == 52
    pf.set_signal(np.full(4000, 0.4))
    pf.apply()
    assert pf.get_number_of_peaks() == 0
    sig = peak_signal()
    np.testing.assert_array_equal(_peaks(mf, sig, 0.8, 52), PEAKS_13)
    np.testing.assert_array_equal(_peaks(mf, sig, 0.8, 0), PEAKS_21)
    np.testing.assert_array_equal(_peaks(mf, sig.astype(np.float32), 0.8, 52, np.float32), PEAKS_13)


def test_peak_finder_errors(gpu):
    mf = gpu
    pf = mf.PeakFinder()
    with pytest.raises(ValueError):
        pf.set_threshold(1.5)
    with pytest.raises(ValueError):
        pf.set_threshold(-0.1)
    with pytest.raises(ValueError):
        pf.set_signal(np.zeros(0))
    pf.apply()  # no signal: no peaks
    assert pf.get_number_of_peaks() == 0


@pytest.mark.parametrize("thr,md", [(0.5, 50), (0.0, 0), (0.0, 3), (0.9, 1000), (0.3, 250), (0.2, 1)])
def test_peaks_random_vs_oracle(gpu, oracle, rng, thr, md):
    mf = gpu
    for n in (1, 2, 3, 17, 4096, 4097, 100_000):
        x = np.clip(rng.standard_normal(n) * 0.6, -1, 1)
        np.testing.assert_array_equal(_peaks(mf, x, thr, md), oracle.peaks(x, thr, md))


def test_peaks_plateaus_and_ties(gpu, oracle, rng):
    mf = gpu
    # quantised values give plateaus and equal-valued candidates
    x = np.round(rng.uniform(0, 1, 50_000) * 8) / 8
    for thr, md in ((0.1, 0), (0.1, 5), (0.5, 40)):
        np.testing.assert_array_equal(_peaks(mf, x, thr, md), oracle.peaks(x, thr, md))
    x = np.zeros(10)
    x[3:6] = 0.9
    np.testing.assert_array_equal(_peaks(mf, x, 0.5, 0), oracle.peaks(x, 0.5, 0))


def test_peaks_dense_long_chain(gpu, oracle):
    """A damped oscillation gives a long run of candidates whose values fall
    with index: the pruning rounds must still match the greedy pass."""
    mf = gpu
    t = np.arange(200_000)
    x = np.exp(-t / 60_000.0) * np.abs(np.sin(t * 0.31)) * 0.99
    for md in (3, 10, 100):
        np.testing.assert_array_equal(_peaks(mf, x, 0.01, md), oracle.peaks(x, 0.01, md))


def test_batched_peaks_on_rho(gpu, oracle, rng):
    mf = gpu
    n = 200_000
    sig = rng.standard_normal(n).astype(np.float32)
    tps = [sig[i:i + 300].astype(np.float64) for i in (1000, 50_000, 123_456)]
    p = mf.SingleChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(100.0)
        p.add_template(wt)
    p.set_signal_size(n)
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p)
    f.set_signal(sig)
    f.apply()
    for thr, md in ((0.3, 100), (0.1, 0)):
        f.find_peaks(thr, md)
        counts, allidx = f.get_all_peaks()
        off = 0
        for i in range(len(tps)):
            rho = f.get_matched_filtered_signal(i).astype(np.float64)
            ref = oracle.peaks(rho, thr, md)
            got = f.get_peaks(i)
            np.testing.assert_array_equal(got, ref)
            np.testing.assert_array_equal(allidx[off:off + counts[i]], ref)
            off += counts[i]
    f.find_peaks(0.5, 200)
    for i, start in enumerate((1000, 50_000, 123_456)):
        assert start in set(f.get_peaks(i).tolist())


def test_dbscan_golden(gpu):
    # testing/dbscan.cpp:8-60
    mf = gpu
    db = mf.DBSCAN()
    db.initialize(3, 2)
    db.set_data(DBSCAN_X)
    db.cluster()
    assert db.get_number_of_clusters() == 2
    np.testing.assert_array_equal(db.get_labels(), [0, 0, 0, 1, 1, -1])
    db.set_data(DBSCAN_X[:5])
    db.cluster()
    assert db.get_number_of_clusters() == 2
    np.testing.assert_array_equal(db.get_labels(), [0, 0, 0, 1, 1])


def test_dbscan_errors(gpu):
    mf = gpu
    db = mf.DBSCAN()
    with pytest.raises(RuntimeError):
        db.set_data(DBSCAN_X)
    with pytest.raises(ValueError):
        db.initialize(-1, 2)
    with pytest.raises(ValueError):
        db.initialize(1, 0)
    db.initialize(1, 2)
    with pytest.raises(RuntimeError):
        db.cluster()
    with pytest.raises(ValueError):
        db.set_weighted_data(DBSCAN_X, np.zeros(6))


@pytest.mark.parametrize("nf", [1, 2, 3])
def test_dbscan_random_vs_oracle(gpu, oracle, rng, nf):
    mf = gpu
    db = mf.DBSCAN()
    for _ in range(6):
        X = rng.uniform(0, 30, (int(rng.integers(1, 2000)), nf))
        if nf == 1:
            X = np.round(X * 4) / 4  # exact ties at the eps boundary
        eps = float(rng.uniform(0.25, 2.5))
        mo = int(rng.integers(1, 8))
        w = rng.uniform(0.1, 3.0, X.shape[0])
        for weights in (None, w):
            db.initialize(eps, mo)
            if weights is None:
                db.set_data(X)
            else:
                db.set_weighted_data(X, weights)
            db.cluster()
            ncl, lab = oracle.dbscan(X, eps, mo, weights)
            assert db.get_number_of_clusters() == ncl
            np.testing.assert_array_equal(db.get_labels(), lab)


@pytest.mark.parametrize("nf", [1, 2])
def test_dbscan_edge_cases_vs_oracle(gpu, oracle, rng, nf):
    # eps = 0 (only exact duplicates are neighbours), every point the same,
    # minPts = 1 (every point a core point) and a single observation, on the
    # one-feature sorted path and the all-pairs path
    db = gpu.DBSCAN()
    dup = np.repeat(rng.integers(0, 40, (60, nf)).astype(np.float64), rng.integers(1, 5, 60), axis=0)
    rng.shuffle(dup)
    cases = [(dup, 0.0, 2), (dup, 0.0, 1), (dup, 0.0, 4), (np.full((500, nf), 7.5), 0.0, 3),
             (np.full((500, nf), 7.5), 1.0, 501), (rng.uniform(0, 100, (300, nf)), 1.5, 1),
             (np.array([[3.0] * nf]), 0.0, 1), (np.array([[3.0] * nf]), 2.0, 2)]
    for X, eps, mo in cases:
        for weights in (None, rng.integers(1, 4, X.shape[0]) / 2.0):
            db.initialize(eps, mo)
            db.set_weighted_data(X[:, 0] if nf == 1 else X, weights)
            db.cluster()
            ncl, lab = oracle.dbscan(X[:, 0] if nf == 1 else X, eps, mo, weights)
            assert db.get_number_of_clusters() == ncl, (eps, mo, X.shape)
            np.testing.assert_array_equal(db.get_labels(), lab)


def test_dbscan_segmented(gpu, oracle, rng):
    mf = gpu
    db = mf.DBSCAN()
    db.initialize(50.0, 3)
    sizes = [0, 5, 300, 1, 1200]
    segs = [rng.uniform(0, 20_000, s) for s in sizes]
    X = np.concatenate(segs) if sum(sizes) else np.zeros(0)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    labels, ncl = db.cluster_segments(X, off)
    for s, seg in enumerate(segs):
        if seg.size == 0:
            assert ncl[s] == 0
            continue
        n_ref, lab_ref = oracle.dbscan(seg, 50.0, 3)
        assert ncl[s] == n_ref
        np.testing.assert_array_equal(labels[off[s]:off[s + 1]], lab_ref)


def test_dbscan_1d_sorted_vs_oracle(gpu, oracle, rng):
    # one feature runs on the per-segment sort; values on a quarter grid put
    # exact ties at eps, and +-inf have no neighbour
    db = gpu.DBSCAN()
    x = np.round(rng.uniform(0, 3000, 20_000) * 4) / 4
    x[rng.integers(0, x.size, 40)] = np.inf
    x[rng.integers(0, x.size, 40)] = -np.inf
    w = rng.integers(1, 7, x.size) / 2.0
    for eps, mo in ((0.25, 2), (0.75, 5), (2.0, 12)):
        for weights in (None, w):
            db.initialize(eps, mo)
            db.set_weighted_data(x, weights)
            db.cluster()
            ncl, lab = oracle.dbscan(x, eps, mo, weights)
            assert db.get_number_of_clusters() == ncl
            np.testing.assert_array_equal(db.get_labels(), lab)


def test_dbscan_1d_nan_keeps_full_scans(gpu, oracle, rng):
    # a NaN has no order: such data keeps the all-pairs scans
    db = gpu.DBSCAN()
    x = np.round(rng.uniform(0, 100, 3000) * 4) / 4
    x[::97] = np.nan
    db.initialize(0.5, 3)
    db.set_data(x)
    db.cluster()
    ncl, lab = oracle.dbscan(x, 0.5, 3)
    assert db.get_number_of_clusters() == ncl
    np.testing.assert_array_equal(db.get_labels(), lab)


def test_dbscan_1d_segmented_large(gpu, rng):
    # 400,000 observations in 700 segments of ragged sizes against the
    # sort-based restatement (pinned against the oracle on the CPU)
    db = gpu.DBSCAN()
    sizes = rng.integers(0, 1150, 700)
    sizes[:3] = (0, 1, 60_000)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    x = np.round(rng.uniform(0, 1000, off[-1]) * 8) / 8
    w = rng.integers(1, 5, x.size) / 2.0
    for eps, mo, weights in ((0.125, 3, None), (0.5, 4, w)):
        db.initialize(eps, mo)
        labels, ncl = db.cluster_segments(x, off, weights)
        for s in range(sizes.size):
            a, b = off[s], off[s + 1]
            n_ref, lab_ref = dbscan_1d(x[a:b], eps, mo, None if weights is None else weights[a:b])
            assert ncl[s] == n_ref
            np.testing.assert_array_equal(labels[a:b], lab_ref)


def _fused_case(mf, rng, dtype, lens, n=60_000, nch=2):
    """Channels of noise with copies of the templates injected, templates
    assigned round-robin to the channels."""
    chans = [rng.standard_normal(n) for _ in range(nch)]
    tps = []
    for i, L in enumerate(lens):
        c = i % nch
        start = int(rng.integers(0, n - L))
        tp = chans[c][start:start + L].copy()
        tps.append(tp)
        for s in rng.integers(0, n - L, 6):
            chans[c][s:s + L] += rng.uniform(0.5, 2.0) * tp
    p = mf.MultiChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(100.0)
        p.add_template(wt)
    p.set_signal_size(n)
    assign = [i % nch for i in range(len(lens))]
    return p, [c.astype(dtype) for c in chans], assign


def _filter(mf, p, chans, assign, dtype, **kw):
    f = mf.MultiChannel.MatchedFilter(dtype=dtype)
    f.initialize(p, template_channels=assign, n_channels=len(chans), **kw)
    for c, s in enumerate(chans):
        f.set_channel_signal(c, s)
    return f


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("fft_length", [256, 1024, 4096])
def test_fused_peak_candidates(gpu, oracle, rng, dtype, variant, fft_length):
    """Candidates gathered inside the correlator give exactly the peaks of
    the stand-alone scan and of the oracle, including chunks with more
    candidates than slots (threshold 0), block seams and the last lag.
    Variant 4 (tensor cores, FP32) flags the 64-lag chunks above the
    threshold instead, and the scan reads only those."""
    mf = gpu
    if dtype == np.float64 and variant == 2 and fft_length == 4096:
        pytest.skip("FP64 spectrum prefetch at N = 4096 exceeds the shared memory of a CTA")
    if variant == 4 and (dtype == np.float64 or fft_length != 4096):
        pytest.skip("the tensor-core correlator takes FP32 data and plans no FFT")
    lens = [150] * 6
    p, chans, assign = _fused_case(mf, rng, dtype, lens)
    fl = 0 if variant == 4 else fft_length
    plain = _filter(mf, p, chans, assign, dtype, fft_length=fl, correlator_variant=variant)
    plain.apply()
    for thr, md in ((0.0, 0), (0.0, 40), (0.35, 0), (0.35, 150), (0.8, 300)):
        f = _filter(mf, p, chans, assign, dtype, fft_length=fl, correlator_variant=variant)
        f.set_peak_threshold(thr)
        f.apply()
        assert f.get_peak_threshold() == (thr, True)
        f.find_peaks(thr, md)
        counts, idx = f.get_all_peaks()
        plain.find_peaks(thr, md)
        counts0, idx0 = plain.get_all_peaks()
        np.testing.assert_array_equal(counts, counts0)
        np.testing.assert_array_equal(idx, idx0)
        off = 0
        for i in range(len(lens)):
            rho = f.get_matched_filtered_signal(i).astype(np.float64)
            np.testing.assert_array_equal(rho, plain.get_matched_filtered_signal(i).astype(np.float64))
            ref = oracle.peaks(rho, thr, md)
            np.testing.assert_array_equal(idx[off:off + counts[i]], ref)
            off += counts[i]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("plan", ["fft2048", "buckets", "wide"])
def test_fused_peak_candidates_mixed_lengths(gpu, oracle, rng, dtype, plan):
    """Templates of several lengths: the peak trace stops at n - Lmax + 1
    lags, inside the shorter templates' valid range; with length buckets the
    templates' blocks differ in length and number."""
    mf = gpu
    lens = [90, 200, 333, 120, 201] + ([1500, 1700] if plan == "buckets" else [])
    p, chans, assign = _fused_case(mf, rng, dtype, lens, n=45_001)
    if plan == "wide" and dtype == np.float64:
        pytest.skip("two 256-thread teams (variant 6) take FP32 data")
    kw = (dict(fft_length=2048) if plan == "fft2048" else
          dict(length_buckets=3) if plan == "buckets" else dict(fft_length=4096, correlator_variant=6))
    f = _filter(mf, p, chans, assign, dtype, **kw)
    if plan == "buckets":
        assert len(f.get_plan()["buckets"]) > 1
    f.set_peak_threshold(0.0)
    f.apply()
    plain = _filter(mf, p, chans, assign, dtype, **kw)
    plain.apply()
    for md in (0, 25):
        f.find_peaks(0.0, md)
        plain.find_peaks(0.0, md)
        c1, i1 = f.get_all_peaks()
        c0, i0 = plain.get_all_peaks()
        np.testing.assert_array_equal(c1, c0)
        np.testing.assert_array_equal(i1, i0)
        off = 0
        for i in range(len(lens)):
            rho = f.get_matched_filtered_signal(i).astype(np.float64)
            np.testing.assert_array_equal(i1[off:off + c1[i]], oracle.peaks(rho, 0.0, md))
            off += c1[i]


def test_fused_peak_threshold_switching(gpu, rng):
    """Another threshold or trace length, a short FFT, or gathering turned
    off all fall back to the scan and give the same peaks."""
    mf = gpu
    p, chans, assign = _fused_case(mf, rng, np.float32, [150] * 4, n=30_000)
    f = _filter(mf, p, chans, assign, np.float32, fft_length=1024)
    g = _filter(mf, p, chans, assign, np.float32, fft_length=1024)
    g.apply()
    f.set_peak_threshold(0.4)
    f.apply()
    for thr, md, tl in ((0.4, 50, 0), (0.5, 50, 0), (0.4, 50, 20_000)):
        f.find_peaks(thr, md, tl)
        g.find_peaks(thr, md, tl)
        for a, b in zip(f.get_all_peaks(), g.get_all_peaks()):
            np.testing.assert_array_equal(a, b)
    f.set_peak_threshold(None)
    f.apply()
    assert f.get_peak_threshold() == (None, False)
    with pytest.raises(ValueError):
        f.set_peak_threshold(1.5)
    s = _filter(mf, p, chans, assign, np.float32, fft_length=256)
    s.set_peak_threshold(0.4)
    s.apply()
    assert s.get_peak_threshold() == (0.4, True)
    t = _filter(mf, p, chans, assign, np.float32, fft_length=256)
    t.apply()
    s.find_peaks(0.4, 50)
    t.find_peaks(0.4, 50)
    for a, b in zip(s.get_all_peaks(), t.get_all_peaks()):
        np.testing.assert_array_equal(a, b)
