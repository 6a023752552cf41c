"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``oracle/liborc.so`` (the project's C restatement of the
reference algorithms, see ``mf_oracle.c`` for the file:line each function
follows).  ``Reference`` wraps ``oracle/_ref/libmflib_ref.so`` -- the
reference's own sources compiled against the FFTW/MKL shim -- and is only
available where the reference checkout was present at build time.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def _ptr_array(arrays, ctype):
    arr = (C.POINTER(ctype) * len(arrays))()
    for i, a in enumerate(arrays):
        arr[i] = a.ctypes.data_as(C.POINTER(ctype))
    return arr


class Oracle:
    """Restated reference algorithms, FP64 and FP32, on the host cores."""

    def __init__(self, path=None):
        path = path or _build.build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_fft_sizes.argtypes = [C.c_int, C.c_int, _ip, _ip]
        L.orc_mf_d.argtypes = [C.c_int, C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p,
                               _dp, C.c_long, C.c_int]
        L.orc_mf_f.argtypes = [C.c_int, C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p,
                               _fp, C.c_long, C.c_int, C.c_int]
        L.orc_mf_d_from_f.argtypes = [C.c_int, C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p,
                                      _dp, C.c_long, C.c_int]
        L.orc_shift_and_stack.argtypes = [C.c_int, _dp, C.c_long, C.c_int, _ip, _dp, C.c_int,
                                          _dp, _ip]
        L.orc_pearson_naive.argtypes = [C.c_int, _dp, C.c_int, _dp, _ip, C.c_int, _dp]
        L.orc_peaks.argtypes = [C.c_int, _dp, C.c_double, C.c_int, _ip]
        L.orc_peaks.restype = C.c_int
        L.orc_dbscan.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_int, _ip]
        L.orc_dbscan.restype = C.c_int
        for nm in ("orc_detect_f", "orc_detect_d"):
            getattr(L, nm).argtypes = [C.c_int, C.c_long, C.c_void_p, C.c_long, C.c_int, C.c_int, C.c_double,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _ip, C.c_void_p,
                                       C.c_void_p, C.c_long, C.c_int, _ip, _ip, _dp, _dp, _ip, _ip, _dp, _dp]
            getattr(L, nm).restype = C.c_int

    def fft_sizes(self, nb, nx):
        a, b = C.c_int(), C.c_int()
        if self.lib.orc_fft_sizes(nb, nx, C.byref(a), C.byref(b)) != 0:
            raise ValueError("invalid sizes nb=%d nx=%d" % (nb, nx))
        return a.value, b.value

    def matched_filter(self, templates, signals, multi=True, dtype=np.float64,
                       float_quirk=False, fp64_from_f32=False, threads=None):
        """Reference MatchedFilter<T> restated.  Returns a list of arrays, one per
        template, holding lags 0..n-L_t (the full valid range)."""
        threads = threads or os.cpu_count() or 1
        tp = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        lens = np.array([len(t) for t in tp], dtype=np.int32)
        nt = len(tp)
        if dtype == np.float32 or fp64_from_f32:
            sg = [np.ascontiguousarray(s, dtype=np.float32) for s in signals]
        else:
            sg = [np.ascontiguousarray(s, dtype=np.float64) for s in signals]
        n = len(sg[0])
        if any(len(x) != n for x in sg) or int(lens.max()) > n:
            # MatchedFilter::initialize rejects signals shorter than a template
            raise ValueError("signals must share one length of at least the longest template")
        tarr = _ptr_array(tp, C.c_double)
        if dtype == np.float32 and not fp64_from_f32:
            out = np.zeros((nt, n), dtype=np.float32)
            sarr = _ptr_array(sg, C.c_float)
            rc = self.lib.orc_mf_f(int(multi), nt, lens.ctypes.data_as(_ip), tarr, n, sarr,
                                   out.ctypes.data_as(_fp), n, int(float_quirk), threads)
        elif fp64_from_f32:
            out = np.zeros((nt, n), dtype=np.float64)
            sarr = _ptr_array(sg, C.c_float)
            rc = self.lib.orc_mf_d_from_f(int(multi), nt, lens.ctypes.data_as(_ip), tarr, n,
                                          sarr, out.ctypes.data_as(_dp), n, threads)
        else:
            out = np.zeros((nt, n), dtype=np.float64)
            sarr = _ptr_array(sg, C.c_double)
            rc = self.lib.orc_mf_d(int(multi), nt, lens.ctypes.data_as(_ip), tarr, n, sarr,
                                   out.ctypes.data_as(_dp), n, threads)
        if rc != 0:
            raise ValueError("oracle matched filter failed")
        return [out[t, : n - lens[t] + 1].copy() for t in range(nt)]

    def shift_and_stack(self, rho_rows, nfilt, shifts, weights, stack_abs=True):
        nt = len(rho_rows)
        ld = max(len(r) for r in rho_rows)
        rho = np.zeros((nt, ld), dtype=np.float64)
        for t, r in enumerate(rho_rows):
            rho[t, : len(r)] = r
        sh = np.ascontiguousarray(shifts, dtype=np.int32)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        out = np.zeros(nfilt, dtype=np.float64)
        nout = C.c_int()
        rc = self.lib.orc_shift_and_stack(nt, rho.ctypes.data_as(_dp), ld, nfilt,
                                          sh.ctypes.data_as(_ip), w.ctypes.data_as(_dp),
                                          int(stack_abs), out.ctypes.data_as(_dp), C.byref(nout))
        if rc != 0:
            raise ValueError("shift and stack failed")
        return out[: nout.value].copy()

    def pearson_naive(self, b, x, lags=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        if lags is None:
            out = np.zeros(len(x) - len(b) + 1, dtype=np.float64)
            self.lib.orc_pearson_naive(len(b), b.ctypes.data_as(_dp), len(x),
                                       x.ctypes.data_as(_dp), None, 0, out.ctypes.data_as(_dp))
        else:
            lg = np.ascontiguousarray(lags, dtype=np.int32)
            out = np.zeros(len(lg), dtype=np.float64)
            self.lib.orc_pearson_naive(len(b), b.ctypes.data_as(_dp), len(x),
                                       x.ctypes.data_as(_dp), lg.ctypes.data_as(_ip), len(lg),
                                       out.ctypes.data_as(_dp))
        return out

    def peaks(self, x, threshold, min_distance):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(max(len(x), 1), dtype=np.int32)
        n = self.lib.orc_peaks(len(x), x.ctypes.data_as(_dp), float(threshold),
                               int(min_distance), out.ctypes.data_as(_ip))
        return out[:n].copy()

    def dbscan(self, X, eps, min_obs, weights=None):
        X = np.ascontiguousarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        nobs, nf = X.shape
        labels = np.zeros(nobs, dtype=np.int32)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=np.float64)
        ncl = self.lib.orc_dbscan(nobs, nf, X.ctypes.data_as(_dp),
                                  w.ctypes.data_as(_dp) if w is not None else None,
                                  float(eps), int(min_obs), labels.ctypes.data_as(_ip))
        return ncl, labels


    def detect(self, rho, templates, signals, fs, threshold=0.7, min_distance=0, absolute_maximum=False,
               single=False, interpolation=1, alpha=51, npts=100, amplitudes=True):
        """Detector<T>::detect restated (orc_detect_f/_d) on given traces:
        rho [nt, len] (float32 or float64), templates (FP64), one signal per
        template (same dtype as rho).  interpolation: 0 Lanczos, 1 quadratic,
        2 none.  Returns a dict of per-detection arrays."""
        rho = np.ascontiguousarray(rho)
        dt = rho.dtype
        ct = C.c_float if dt == np.float32 else C.c_double
        nt, ln = rho.shape
        tps = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        sig = [np.ascontiguousarray(x, dtype=dt) for x in signals]
        lens = np.array([t.size for t in tps], dtype=np.int32)
        maxdet = nt * ln + 1
        o = {k: np.zeros(maxdet, np.int32) for k in ("template", "sample", "sign", "have_amplitude")}
        o.update({k: np.zeros(maxdet, np.float64) for k in ("correlation", "shift", "gibbons_ringdal",
                                                             "schaff_richards")})
        fn = self.lib.orc_detect_f if dt == np.float32 else self.lib.orc_detect_d
        nd = fn(nt, ln, rho.ctypes.data_as(C.c_void_p), ln, int(absolute_maximum), int(single), float(threshold),
                int(min_distance), int(interpolation), int(alpha), int(npts), float(fs), int(amplitudes),
                lens.ctypes.data_as(_ip), _ptr_array(tps, C.c_double), _ptr_array(sig, ct), sig[0].size, maxdet,
                o["template"].ctypes.data_as(_ip), o["sample"].ctypes.data_as(_ip),
                o["correlation"].ctypes.data_as(_dp), o["shift"].ctypes.data_as(_dp),
                o["sign"].ctypes.data_as(_ip), o["have_amplitude"].ctypes.data_as(_ip),
                o["gibbons_ringdal"].ctypes.data_as(_dp), o["schaff_richards"].ctypes.data_as(_dp))
        out = {k: v[:nd].copy() for k, v in o.items()}
        out["time"] = out["sample"] * (1.0 / fs)
        out["interpolated_time"] = out["time"] + out["shift"]
        return out


    def associate(self, evid, onset, travel, xc, tol, min_picks, weighted=False):
        """Associator<T>::associate (src/singleChannel/associator.cpp:
        156-267) restated: detections sorted by event id then onset time
        (stable), DBSCAN (orc_dbscan) of each event's origin times (onset -
        travel), eps = tol, minPts = min_picks, optionally weighted by xc.
        Returns the sort order and the events as (event id, [positions in
        the sorted order]), ordered by event id then cluster."""
        evid = np.asarray(evid, dtype=np.uint64)
        onset = np.asarray(onset, dtype=np.float64)
        travel = np.asarray(travel, dtype=np.float64)
        xc = np.asarray(xc, dtype=np.float64)
        order = np.lexsort((onset, evid))
        events = []
        ev, on, tr, w = evid[order], onset[order], travel[order], xc[order]
        i = 0
        while i < ev.size:
            j = i
            while j < ev.size and ev[j] == ev[i]:
                j += 1
            ot = (on[i:j] - tr[i:j]).reshape(-1, 1)
            ncl, lab = self.dbscan(ot, tol, min_picks, w[i:j] if weighted else None)
            for c in range(ncl):
                events.append((int(ev[i]), [i + k for k in range(j - i) if lab[k] == c]))
            i = j
        return order, events


    @staticmethod
    def relative_amplitudes(b, windows):
        """RelativeMagnitude<double> (src/singleChannel/relativeMagnitude.cpp:
        35-130): per window y, |<b, y>| / <b, b> and sqrt(<y, y> / <b, b>) of
        the demeaned template and window, sequential double sums."""
        b = np.asarray(b, dtype=np.float64)
        bd = b - np.sum(b) / b.size
        bb = float(np.dot(bd, bd))
        out = []
        for y in np.atleast_2d(np.asarray(windows, dtype=np.float64)):
            yd = y - np.sum(y) / y.size
            yy = float(np.dot(yd, yd))
            out.append((abs(float(np.dot(bd, yd))) / bb, np.sqrt(yy / bb), yy > 0))
        gr, sr, ok = (np.array(v) for v in zip(*out))
        return gr, sr, ok


class Reference:
    """The reference's own classes (compiled against the FFTW/MKL shim)."""

    def __init__(self, path=None):
        path = path or _build.ref_lib_path()
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_fft_sizes.argtypes = [C.c_int, C.c_int, _ip, _ip]
        L.ref_window_length.argtypes = [C.c_int, C.c_int, _ip, _ip]
        L.ref_mf_d.argtypes = [C.c_int, C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p,
                               _dp, C.c_long]
        L.ref_mf_f.argtypes = [C.c_int, C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p,
                               _fp, C.c_long]
        L.ref_mf_stack_d.argtypes = [C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p, _dp,
                                     C.c_long, C.c_double, _dp, _dp, _dp, C.c_int, _dp, _ip]
        L.ref_peaks_d.argtypes = [C.c_int, _dp, C.c_double, C.c_int, _ip]
        L.ref_peaks_f.argtypes = [C.c_int, _fp, C.c_float, C.c_int, _ip]
        L.ref_relmag_d.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        for nm in ("ref_detect_d", "ref_detect_f"):
            getattr(L, nm).argtypes = [C.c_int, _ip, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_double,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       _ip, _dp, _dp, _dp, _ip, _ip, _dp, _dp]
            getattr(L, nm).restype = C.c_int

    def relative_amplitudes(self, b, y):
        b = np.ascontiguousarray(b, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        gr, sr = C.c_double(), C.c_double()
        if self.lib.ref_relmag_d(b.size, b.ctypes.data_as(_dp), y.ctypes.data_as(_dp), C.byref(gr), C.byref(sr)):
            raise ValueError("reference RelativeMagnitude rejected the input")
        return gr.value, sr.value

    def detect(self, templates, signal, fs, threshold=0.7, min_distance=0, absolute_maximum=False, single=False,
               interpolation=1, alpha=51, npts=100, amplitudes=True, dtype=np.float64, maxdet=100000):
        """SingleChannel::MatchedFilter<T> + SingleChannel::Detector<T> of the
        reference on one signal; templates carry COMPRESSION polarity."""
        tps = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        x = np.ascontiguousarray(signal, dtype=dtype)
        lens = np.array([t.size for t in tps], dtype=np.int32)
        o = {k: np.zeros(maxdet, np.int32) for k in ("template", "polarity", "have_amplitude")}
        o.update({k: np.zeros(maxdet, np.float64) for k in ("correlation", "time", "interpolated_time",
                                                             "gibbons_ringdal", "schaff_richards")})
        fn = self.lib.ref_detect_f if x.dtype == np.float32 else self.lib.ref_detect_d
        nd = fn(len(tps), lens.ctypes.data_as(_ip), _ptr_array(tps, C.c_double), x.size,
                x.ctypes.data_as(C.c_void_p), float(fs), float(threshold), int(min_distance), int(absolute_maximum),
                int(single), int(interpolation), int(alpha), int(npts), int(amplitudes), maxdet,
                o["template"].ctypes.data_as(_ip), o["correlation"].ctypes.data_as(_dp),
                o["time"].ctypes.data_as(_dp), o["interpolated_time"].ctypes.data_as(_dp),
                o["polarity"].ctypes.data_as(_ip), o["have_amplitude"].ctypes.data_as(_ip),
                o["gibbons_ringdal"].ctypes.data_as(_dp), o["schaff_richards"].ctypes.data_as(_dp))
        if nd < 0:
            raise RuntimeError("reference detector failed")
        return {k: v[:min(nd, maxdet)].copy() for k, v in o.items()}

    @staticmethod
    def available():
        return os.path.exists(_build.ref_lib_path())

    def fft_sizes(self, nb, nx):
        a, b = C.c_int(), C.c_int()
        if self.lib.ref_fft_sizes(nb, nx, C.byref(a), C.byref(b)) != 0:
            raise ValueError("invalid sizes")
        return a.value, b.value

    def window_length(self, nb, nx):
        """MatchedFilterParameters::getFFTLength / getBlockLength for a
        template of nb samples and a signal of nx."""
        a, b = C.c_int(), C.c_int()
        if self.lib.ref_window_length(nb, nx, C.byref(a), C.byref(b)) != 0:
            raise ValueError("invalid sizes")
        return a.value, b.value

    def matched_filter(self, templates, signals, multi=True, dtype=np.float64):
        tp = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        lens = np.array([len(t) for t in tp], dtype=np.int32)
        nt = len(tp)
        sg = [np.ascontiguousarray(s, dtype=dtype) for s in signals]
        n = len(sg[0])
        tarr = _ptr_array(tp, C.c_double)
        out = np.zeros((nt, n), dtype=dtype)
        if dtype == np.float32:
            rc = self.lib.ref_mf_f(int(multi), nt, lens.ctypes.data_as(_ip), tarr, n,
                                   _ptr_array(sg, C.c_float), out.ctypes.data_as(_fp), n)
        else:
            rc = self.lib.ref_mf_d(int(multi), nt, lens.ctypes.data_as(_ip), tarr, n,
                                   _ptr_array(sg, C.c_double), out.ctypes.data_as(_dp), n)
        if rc != 0:
            raise ValueError("reference matched filter failed")
        return [out[t, : n - lens[t] + 1].copy() for t in range(nt)]

    def matched_filter_stack(self, templates, signals, fs, onsets, travel, weights,
                             stack_abs=True):
        tp = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        lens = np.array([len(t) for t in tp], dtype=np.int32)
        nt = len(tp)
        sg = [np.ascontiguousarray(s, dtype=np.float64) for s in signals]
        n = len(sg[0])
        out = np.zeros((nt, n), dtype=np.float64)
        stack = np.zeros(n, dtype=np.float64)
        ns = C.c_int()
        on = np.ascontiguousarray(onsets, dtype=np.float64)
        tt = np.ascontiguousarray(travel, dtype=np.float64)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        rc = self.lib.ref_mf_stack_d(nt, lens.ctypes.data_as(_ip), _ptr_array(tp, C.c_double),
                                     n, _ptr_array(sg, C.c_double), out.ctypes.data_as(_dp), n,
                                     float(fs), on.ctypes.data_as(_dp), tt.ctypes.data_as(_dp),
                                     w.ctypes.data_as(_dp), int(stack_abs),
                                     stack.ctypes.data_as(_dp), C.byref(ns))
        if rc != 0:
            raise ValueError("reference matched filter failed")
        return [out[t, : n - lens[t] + 1].copy() for t in range(nt)], stack[: ns.value].copy()

    def peaks(self, x, threshold, min_distance, dtype=np.float64):
        x = np.ascontiguousarray(x, dtype=dtype)
        out = np.zeros(max(len(x), 1), dtype=np.int32)
        if dtype == np.float32:
            n = self.lib.ref_peaks_f(len(x), x.ctypes.data_as(_fp), float(threshold),
                                     int(min_distance), out.ctypes.data_as(_ip))
        else:
            n = self.lib.ref_peaks_d(len(x), x.ctypes.data_as(_dp), float(threshold),
                                     int(min_distance), out.ctypes.data_as(_ip))
        if n < 0:
            raise ValueError("reference peak finder failed")
        return out[:n].copy()
