"""DBSCAN entry point that allocates no device memory.

mfgpu_dbscan_segmented_noalloc serves callers that cannot call cudaMalloc
(a host framework that has reserved all device memory for its own pools,
or a real-time pipeline that must not allocate after start-up).  The
caller passes device buffers and a stream; the library's working memory is
a fixed static device array.  This test drives it through the C ABI and
checks it against the allocating entry point, mfgpu_dbscan_segmented, on
two calls in a row (the second call reuses the array the first one left
behind).  Labels are integers and must match exactly.  Once the module is
loaded, further calls leave the device's free memory unchanged; an empty
problem and malformed (clamped) segment offsets stay inside the caller's
buffers.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, X, seg_off, eps, min_obs, weights=None):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    Xd = torch.tensor(np.ascontiguousarray(X, dtype=np.float64), device=dev)
    so = torch.tensor(np.ascontiguousarray(seg_off, dtype=np.int32), device=dev)
    wd = None if weights is None else torch.tensor(np.ascontiguousarray(weights, dtype=np.float64), device=dev)
    n = X.shape[0]
    nseg = len(seg_off) - 1
    labels = torch.full((max(n, 1),), -7, dtype=torch.int32, device=dev)
    ncl = torch.full((nseg,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = lib.mfgpu_dbscan_segmented_noalloc(
        nseg, ctypes.c_void_p(so.data_ptr()), n, X.shape[1], ctypes.c_void_p(Xd.data_ptr()),
        ctypes.c_void_p(wd.data_ptr()) if wd is not None else None, float(eps), int(min_obs),
        ctypes.c_void_p(labels.data_ptr()), ctypes.c_void_p(ncl.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    from mflib_gb300 import _lib
    _lib.check(st)
    torch.cuda.synchronize(dev)
    return labels.cpu().numpy()[:n], ncl.cpu().numpy()


def _case(rng, sizes, nf):
    segs = [rng.uniform(0, 400.0, (s, nf)) for s in sizes]
    X = np.concatenate(segs) if sum(sizes) else np.zeros((0, nf))
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    return X, off


def test_noalloc_matches_allocating_entry_point(gpu):
    mf = gpu
    from mflib_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.default_rng(7)
    db = mf.DBSCAN()
    cases = [(_case(rng, [300, 0, 1200, 7], 1), 2.0, 3, None),
             (_case(rng, [50, 2500, 640], 2), 6.0, 4, "w")]
    for (X, off), eps, mo, wflag in cases:   # two calls in a row
        w = rng.uniform(0.5, 2.0, X.shape[0]) if wflag else None
        db.initialize(eps, mo)
        ref_labels, ref_ncl = db.cluster_segments(X, off, weights=w)
        labels, ncl = _noalloc(lib, X, off, eps, mo, weights=w)
        np.testing.assert_array_equal(ncl, ref_ncl)
        np.testing.assert_array_equal(labels, ref_labels)


def test_noalloc_rejects_oversize(gpu):
    from mflib_gb300 import _lib
    lib = _lib.lib()
    st = lib.mfgpu_dbscan_segmented_noalloc(1, None, 65536 + 1, 1, None, None, 1.0, 2, None, None, None)
    assert st == _lib.MFGPU_EINVAL
    assert "65536" in lib.mfgpu_last_error().decode()
    st = lib.mfgpu_dbscan_segmented_noalloc(4097, None, 10, 1, None, None, 1.0, 2, None, None, None)
    assert st == _lib.MFGPU_EINVAL


def test_noalloc_allocates_nothing(gpu):
    """After a first call (which loads the module holding the scratch array),
    repeated calls change neither the device's free memory nor anything the
    caller did not pass."""
    torch = pytest.importorskip("torch")
    from mflib_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.default_rng(11)
    X, off = _case(rng, [400, 900], 1)
    dev = torch.device("cuda", 0)
    Xd = torch.tensor(X, device=dev)
    so = torch.tensor(off, device=dev)
    labels = torch.empty(X.shape[0], dtype=torch.int32, device=dev)
    ncl = torch.empty(2, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def call():
        st = lib.mfgpu_dbscan_segmented_noalloc(
            2, ctypes.c_void_p(so.data_ptr()), X.shape[0], 1, ctypes.c_void_p(Xd.data_ptr()), None, 3.0, 3,
            ctypes.c_void_p(labels.data_ptr()), ctypes.c_void_p(ncl.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        _lib.check(st)
        torch.cuda.synchronize(dev)

    call()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(5):
        call()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0


def test_noalloc_empty_and_malformed_offsets(gpu):
    from mflib_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.default_rng(13)
    # no observations: every segment gets zero clusters
    labels, ncl = _noalloc(lib, np.zeros((0, 1)), np.array([0, 0, 0], np.int32), 1.0, 2)
    np.testing.assert_array_equal(ncl, [0, 0])
    # decreasing / out-of-range offsets are clamped: labels stay in range and
    # the clusters of the clamped partition are counted
    X, _ = _case(rng, [500], 1)
    bad = np.array([5, 300, 100, 10_000], np.int32)   # first not 0, decreasing, last past n
    labels, ncl = _noalloc(lib, X, bad, 2.0, 3)
    assert labels.shape == (500,)
    assert labels.min() >= -1
    assert np.all(ncl >= 0) and int(ncl.sum()) <= 500
    assert labels.max() < max(1, int(ncl.max()))
    # NaN epsilon is rejected before any work is enqueued
    st = lib.mfgpu_dbscan_segmented_noalloc(1, None, 10, 1, None, None, float("nan"), 2, None, None, None)
    assert st == _lib.MFGPU_EINVAL


def test_noalloc_one_feature_sorted_on_device(gpu, oracle):
    """One feature: the entry point sorts every segment on the device
    (bitonic network) and visits neighbourhoods only.  Checked against the
    oracle with ties at eps, +-inf and NaN values (a NaN is no neighbour of
    anything), weights, and at the scratch's full capacity in one segment
    against the sort-based restatement."""
    from mflib_gb300 import _lib
    from test_oracle import dbscan_1d
    lib = _lib.lib()
    rng = np.random.default_rng(11)
    sizes = [700, 0, 1, 2500, 33]
    x = np.round(rng.uniform(0, 300, sum(sizes)) * 4) / 4
    x[rng.integers(0, x.size, 25)] = np.inf
    x[rng.integers(0, x.size, 25)] = -np.inf
    x[rng.integers(0, x.size, 25)] = np.nan
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    w = rng.integers(1, 6, x.size) / 2.0
    for eps, mo, weights in ((0.25, 2, None), (0.75, 4, w)):
        labels, ncl = _noalloc(lib, x[:, None], off, eps, mo, weights)
        for s in range(len(sizes)):
            a, b = off[s], off[s + 1]
            n_ref, lab_ref = oracle.dbscan(x[a:b], eps, mo, None if weights is None else weights[a:b])
            assert ncl[s] == n_ref
            np.testing.assert_array_equal(labels[a:b], lab_ref)
    # the full capacity in one segment, and ragged segments up to it
    n = 65_536
    x = np.round(rng.uniform(0, 6000, n) * 8) / 8
    for off in (np.array([0, n], np.int32), np.array([0, 17, 40_000, 40_001, n], np.int32)):
        labels, ncl = _noalloc(lib, x[:, None], off, 0.125, 3)
        for s in range(len(off) - 1):
            a, b = off[s], off[s + 1]
            n_ref, lab_ref = dbscan_1d(x[a:b], 0.125, 3)
            assert ncl[s] == n_ref
            np.testing.assert_array_equal(labels[a:b], lab_ref)
