"""PeakFinder and DBSCAN with the reference's interface, on the GPU.

``PeakFinder`` mirrors MFLib::PeakFinder<T> (include/private/peakFinder.hpp,
src/peakFinder.cpp); ``DBSCAN`` mirrors MFLib::DBSCAN
(include/private/dbscan.hpp, src/dbscan.cpp).  Both call libmfgpu.
"""
import ctypes as C

import numpy as np

from . import _lib

_ip = C.POINTER(C.c_int)


class PeakFinder:
    def __init__(self, dtype=np.float64):
        self._dtype = np.dtype(dtype)
        prec = _lib.MFGPU_FLOAT32 if self._dtype == np.float32 else _lib.MFGPU_FLOAT64
        h = C.c_void_p()
        _lib.call("mfgpu_peaks_create", prec, C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().mfgpu_peaks_destroy(h)
            except Exception:
                pass
            self._h = None

    def clear(self):
        _lib.call("mfgpu_peaks_clear", self._h)

    def set_threshold(self, thr):
        _lib.call("mfgpu_peaks_set_threshold", self._h, float(thr))

    def get_threshold(self):
        v = C.c_double()
        _lib.call("mfgpu_peaks_get_threshold", self._h, C.byref(v))
        return v.value

    def set_minimum_peak_distance(self, d):
        _lib.call("mfgpu_peaks_set_minimum_peak_distance", self._h, int(d))

    def get_minimum_peak_distance(self):
        v = C.c_int()
        _lib.call("mfgpu_peaks_get_minimum_peak_distance", self._h, C.byref(v))
        return v.value

    def set_signal(self, x):
        x = np.ascontiguousarray(x, dtype=self._dtype).ravel()
        _lib.call("mfgpu_peaks_set_signal", self._h, int(x.size), x.ctypes.data_as(C.c_void_p))

    def apply(self):
        _lib.call("mfgpu_peaks_apply", self._h)

    def get_number_of_peaks(self):
        v = C.c_int()
        _lib.call("mfgpu_peaks_get_number_of_peaks", self._h, C.byref(v))
        return v.value

    def get_peak_indices(self):
        n = self.get_number_of_peaks()
        out = np.zeros(max(n, 1), dtype=np.int32)
        _lib.call("mfgpu_peaks_get_peak_indices", self._h, int(out.size), out.ctypes.data_as(_ip))
        return out[:n].copy()


class DBSCAN:
    def __init__(self):
        h = C.c_void_p()
        _lib.call("mfgpu_dbscan_create", C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().mfgpu_dbscan_destroy(h)
            except Exception:
                pass
            self._h = None

    def clear(self):
        _lib.call("mfgpu_dbscan_clear", self._h)

    def initialize(self, epsilon, min_observations):
        _lib.call("mfgpu_dbscan_initialize", self._h, float(epsilon), int(min_observations))

    @staticmethod
    def _matrix(X):
        X = np.ascontiguousarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        return X

    def set_data(self, X):
        X = self._matrix(X)
        _lib.call("mfgpu_dbscan_set_data", self._h, int(X.shape[0]), int(X.shape[1]),
                  X.ctypes.data_as(C.c_void_p))
        self._nobs = int(X.shape[0])

    def set_weighted_data(self, X, weights=None):
        X = self._matrix(X)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=np.float64)
        _lib.call("mfgpu_dbscan_set_weighted_data", self._h, int(X.shape[0]), int(X.shape[1]),
                  X.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p) if w is not None else None)
        self._nobs = int(X.shape[0])

    def cluster(self):
        _lib.call("mfgpu_dbscan_cluster", self._h)

    def _flag(self, name):
        v = C.c_int()
        _lib.call(name, self._h, C.byref(v))
        return bool(v.value)

    def is_initialized(self):
        return self._flag("mfgpu_dbscan_is_initialized")

    def have_data(self):
        return self._flag("mfgpu_dbscan_have_data")

    def have_labels(self):
        return self._flag("mfgpu_dbscan_have_labels")

    def launch_count(self):
        v = C.c_longlong()
        _lib.call("mfgpu_dbscan_get_launch_count", self._h, C.byref(v))
        return v.value

    def get_number_of_clusters(self):
        v = C.c_int()
        _lib.call("mfgpu_dbscan_get_number_of_clusters", self._h, C.byref(v))
        return v.value

    def get_labels(self):
        buf = np.zeros(max(1, getattr(self, "_nobs", 0)), dtype=np.int32)
        _lib.call("mfgpu_dbscan_get_labels", self._h, int(buf.size), buf.ctypes.data_as(_ip))
        return buf[: getattr(self, "_nobs", 0)].copy()

    def cluster_segments(self, X, seg_offsets, weights=None):
        """Extension: independent DBSCAN runs over row ranges
        seg_offsets[s]..seg_offsets[s+1]; returns (labels, n_clusters)."""
        X = self._matrix(X)
        so = np.ascontiguousarray(seg_offsets, dtype=np.int32)
        nseg = so.size - 1
        labels = np.zeros(max(1, X.shape[0]), dtype=np.int32)
        ncl = np.zeros(max(1, nseg), dtype=np.int32)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        _lib.call("mfgpu_dbscan_segmented", self._h, int(nseg), so.ctypes.data_as(_ip), int(X.shape[1]),
                  X.ctypes.data_as(C.c_void_p), w.ctypes.data_as(C.c_void_p) if w is not None else None,
                  labels.ctypes.data_as(_ip), ncl.ctypes.data_as(_ip))
        return labels[: X.shape[0]].copy(), ncl[:nseg].copy()
