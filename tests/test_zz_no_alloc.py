"""DBSCAN entry point that allocates no device memory.

mfgpu_dbscan_segmented_noalloc serves callers that cannot call cudaMalloc
(a host framework that has reserved all device memory for its own pools,
or a real-time pipeline that must not allocate after start-up).  The
caller passes device buffers and a stream; the library's working memory is
a fixed static device array.  This test drives it through the C ABI and
checks it against the allocating entry point, mfgpu_dbscan_segmented, on
two calls in a row (the second call reuses the array the first one left
behind).  Labels are integers and must match exactly.
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
