"""Single-channel detector: MFLib::SingleChannel::{Detector, DetectorParameters,
DetectionTimeInterpolationParameters, Detection} with the pymflib names
(python/singleChannel/detector*.cpp, detection.cpp).

The data-parallel work -- the reduction of the Pearson traces across
templates, the PeakFinder, the detection-time refinement and the relative
amplitudes -- runs in libmfgpu (mfgpu_mf_detect); this module holds the
parameters and assembles Detection objects from the templates' metadata, as
Detector<T>::detect does (src/singleChannel/detector.cpp:419-691).

Differences from the reference, kept on purpose: the relative amplitudes of
FP32 signals use the window's mean (the reference's float overload subtracts
the window's sum, src/singleChannel/relativeMagnitude.cpp:105-121); SINGLE
detections with equal times keep template order (the reference sorts with an
unstable sort).
"""
import ctypes as C
import enum
import math

import numpy as np

from . import _lib
from .matched_filter import MatchedFilter
from .waveform import MatchedFilterDetectionMode, NetworkStationPhase, Polarity


class MaximumMatchedFilterPolicy(enum.IntEnum):
    """include/mflib/enums.hpp:53-60."""
    maximum = 0
    absolute_maximum = 1


class MatchedFilteredSignalDetectorPolicy(enum.IntEnum):
    """include/mflib/enums.hpp:66-75 (pymflib name ``reduce`` for REDUCED)."""
    reduce = 0
    single = 1


class DetectionTimeInterpolationType(enum.IntEnum):
    """include/mflib/enums.hpp:81-92."""
    lanczos = 0
    quadratic = 1
    none = 2


class RelativeMagnitudeType(enum.IntEnum):
    """include/mflib/enums.hpp:37-47."""
    gibbons_ringdal_2006 = 0
    schaff_richards_2014 = 1


class DetectionTimeInterpolationParameters:
    """src/singleChannel/detectionTimeInterpolationParameters.cpp."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._alpha, self._npts, self._type = 51, 100, DetectionTimeInterpolationType.quadratic

    def enable_lanczos(self):
        self._type = DetectionTimeInterpolationType.lanczos

    def enable_quadratic(self):
        self._type = DetectionTimeInterpolationType.quadratic

    def disable_interpolation(self):
        self._type = DetectionTimeInterpolationType.none

    def get_type(self):
        return self._type

    def set_lanczos_alpha(self, alpha):
        if alpha < 1:
            raise ValueError("alpha must be positive")
        self._alpha = int(alpha)

    def get_lanczos_alpha(self):
        return self._alpha

    def set_lanczos_number_of_interpolation_points(self, npts):
        if npts < 1:
            raise ValueError("Number of interpolation points must be positive")
        self._npts = int(npts)

    def get_lanczos_number_of_interpolation_points(self):
        return self._npts


class DetectorParameters:
    """src/singleChannel/detectorParameters.cpp (defaults :9-12, :20-26)."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._thr = 0.7
        self._maxp = MaximumMatchedFilterPolicy.maximum
        self._mfp = MatchedFilteredSignalDetectorPolicy.single
        self._mind = 0
        self._wave = False
        self._amp = True
        self._interp = DetectionTimeInterpolationParameters()

    def set_detection_threshold(self, tol):
        if tol <= 0 or tol > 1:
            raise ValueError("Threshold = %g must be in range (0,1]" % tol)
        self._thr = float(tol)

    def get_detection_threshold(self):
        return self._thr

    def set_minimum_detection_spacing(self, n):
        self._mind = int(n)

    def get_minimum_detection_spacing(self):
        return self._mind

    def set_matched_filtered_signal_detector_policy(self, policy):
        self._mfp = MatchedFilteredSignalDetectorPolicy(int(policy))

    def get_matched_filtered_signal_detector_policy(self):
        return self._mfp

    def set_maxima_policy(self, policy):
        self._maxp = MaximumMatchedFilterPolicy(int(policy))

    def get_maxima_policy(self):
        return self._maxp

    def enable_save_detected_waveform(self):
        self._wave = True

    def disable_save_detected_waveform(self):
        self._wave = False

    def want_detected_waveform(self):
        return self._wave

    def enable_save_amplitude_scaling_factor(self):
        self._amp = True

    def disable_save_amplitude_scaling_factor(self):
        self._amp = False

    def want_amplitude_scaling_factor(self):
        return self._amp

    def set_detection_time_interpolation_parameters(self, p):
        q = DetectionTimeInterpolationParameters()
        q._alpha, q._npts, q._type = p._alpha, p._npts, p._type
        self._interp = q

    def get_detection_time_interpolation_parameters(self):
        return self._interp


def _non_negative(t, what):
    # the pymflib setters refuse negative times (python/singleChannel/detection.cpp:191-290)
    if t < 0:
        raise ValueError("%s = %g must not be negative" % (what, t))


class Detection:
    """src/singleChannel/detection.cpp: a detection's value fields, each with
    get / set / have."""

    __slots__ = ("_id", "_xc", "_sig", "_t", "_ti", "_tt", "_po", "_poi", "_amp", "_pol")

    def __init__(self):
        self.clear()

    def clear(self):
        self._id = None
        self._xc = None
        self._sig = None
        self._t = self._ti = self._tt = self._po = self._poi = None
        self._amp = {}
        self._pol = Polarity.unknown

    def _get(self, v, what):
        if v is None:
            raise RuntimeError("%s not set" % what)
        return v

    def set_template_identifier(self, ident):
        self._id = (ident[0], int(ident[1]))

    def get_template_identifier(self):
        return self._get(self._id, "Template identifier")

    def have_template_identifier(self):
        return self._id is not None

    def set_correlation_coefficient(self, v):
        if v < -1 or v > 1:
            raise ValueError("Correlation coefficient = %g must be in range [-1,1]" % v)
        self._xc = float(v)

    def get_correlation_coefficient(self):
        return self._get(self._xc, "Correlation coefficient")

    def have_correlation_coefficient(self):
        return self._xc is not None

    def set_detected_signal(self, x):
        self._sig = np.array(x, dtype=np.float64)

    def get_detected_signal(self):
        return self._get(self._sig, "Detected signal").copy()

    def have_detected_signal(self):
        return self._sig is not None

    def set_detection_time(self, t):
        _non_negative(t, 'Detection time')
        self._t = float(t)

    def get_detection_time(self):
        return self._get(self._t, "Detection time")

    def have_detection_time(self):
        return self._t is not None

    def set_interpolated_detection_time(self, t):
        _non_negative(t, 'Detection time')
        self._ti = float(t)

    def get_interpolated_detection_time(self):
        return self._get(self._ti, "Interpolated detection time")

    def have_interpolated_detection_time(self):
        return self._ti is not None

    def set_travel_time(self, t):
        _non_negative(t, 'Travel time')
        self._tt = float(t)

    def get_travel_time(self):
        return self._get(self._tt, "Travel time")

    def have_travel_time(self):
        return self._tt is not None

    def set_phase_onset_time(self, t):
        _non_negative(t, 'Onset time')
        self._po = float(t)

    def get_phase_onset_time(self):
        return self._get(self._po, "Phase onset time")

    def have_phase_onset_time(self):
        return self._po is not None

    def set_interpolated_phase_onset_time(self, t):
        _non_negative(t, 'Onset time')
        self._poi = float(t)

    def get_interpolated_phase_onset_time(self):
        return self._get(self._poi, "Interpolated phase onset time")

    def have_interpolated_phase_onset_time(self):
        return self._poi is not None

    def set_amplitude_scaling_factor(self, value, mag_type):
        """python/singleChannel/detection.cpp:333-343: the factor must be
        positive."""
        if not value > 0:
            raise ValueError("Scaling factor = %g must be positive" % value)
        self._amp[RelativeMagnitudeType(int(mag_type))] = float(value)

    def get_amplitude_scaling_factor(self, mag_type):
        return self._get(self._amp.get(RelativeMagnitudeType(int(mag_type))), "Amplitude scaling factor")

    def have_amplitude_scaling_factor(self, mag_type=None):
        """With a type: that factor is set.  Without one, as pymflib
        (python/singleChannel/detection.cpp:353-362): both factors are set."""
        if mag_type is None:
            return len(self._amp) == len(RelativeMagnitudeType)
        return RelativeMagnitudeType(int(mag_type)) in self._amp

    def get_magnitude_perturbation(self, mag_type):
        """log10 of the amplitude scaling factor (relativeMagnitude.cpp)."""
        a = self.get_amplitude_scaling_factor(mag_type)
        if a <= 0:
            raise ValueError("Scaling factor = %g must be positive" % a)
        return math.log10(a)

    def have_magnitude_perturbation(self, mag_type):
        return self.have_amplitude_scaling_factor(mag_type)

    def set_polarity(self, p):
        self._pol = Polarity(int(p))

    def get_polarity(self):
        return self._pol

    # pickling (python/singleChannel/detection.cpp:498-585 keeps the same fields)
    def __getstate__(self):
        ident = None if self._id is None else (self._id[0].__getstate__(), self._id[1])
        return {"id": ident, "xc": self._xc, "sig": None if self._sig is None else self._sig.tolist(),
                "t": self._t, "ti": self._ti, "tt": self._tt, "po": self._po, "poi": self._poi,
                "amp": {int(k): v for k, v in self._amp.items()}, "pol": int(self._pol)}

    def __setstate__(self, st):
        self.clear()
        if st["id"] is not None:
            nsp = NetworkStationPhase()
            nsp.__setstate__(st["id"][0])
            self._id = (nsp, int(st["id"][1]))
        self._xc = st["xc"]
        self._sig = None if st["sig"] is None else np.array(st["sig"], dtype=np.float64)
        self._t, self._ti, self._tt, self._po, self._poi = st["t"], st["ti"], st["tt"], st["po"], st["poi"]
        self._amp = {RelativeMagnitudeType(k): v for k, v in st["amp"].items()}
        self._pol = Polarity(st["pol"])


class Detector:
    """Detector<T> (src/singleChannel/detector.cpp): initialize(parameters),
    detect(matched_filter), get_number_of_detections(), get_detection(i)."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._params = None
        self._dets = []

    def is_initialized(self):
        return self._params is not None

    def initialize(self, parameters):
        if not isinstance(parameters, DetectorParameters):
            raise ValueError("parameters must be DetectorParameters")
        self.clear()
        p = DetectorParameters()
        p.__dict__.update(parameters.__dict__)
        p.set_detection_time_interpolation_parameters(parameters.get_detection_time_interpolation_parameters())
        self._params = p

    def detect(self, mf):
        """Detections of the matched filter's last apply (any MatchedFilter of
        this package: every template's trace takes part)."""
        self._dets = []
        if not self.is_initialized():
            raise ValueError("Detector class not initialized")
        if not mf.have_matched_filtered_signals():
            raise ValueError("Matched filtered signals not computed")
        nt = mf.get_number_of_templates()
        if nt < 1:
            raise ValueError("No templates on matched filter class")
        prm = self._params
        ip = prm.get_detection_time_interpolation_parameters()
        templates = mf._templates  # read only: metadata of the detected templates
        fs = templates[0].get_sampling_rate()
        dp = _lib.MfgpuDetectParams()
        dp.threshold = min(1.0, max(0.0, prm.get_detection_threshold()))
        dp.min_distance = prm.get_minimum_detection_spacing()
        dp.absolute_maximum = int(prm.get_maxima_policy() == MaximumMatchedFilterPolicy.absolute_maximum)
        dp.single = int(prm.get_matched_filtered_signal_detector_policy() == MatchedFilteredSignalDetectorPolicy.single)
        dp.interpolation = int(ip.get_type())
        dp.lanczos_alpha = ip.get_lanczos_alpha()
        dp.lanczos_points = ip.get_lanczos_number_of_interpolation_points()
        dp.sampling_rate = fs
        dp.amplitudes = int(prm.want_amplitude_scaling_factor())
        n = C.c_int()
        _lib.call("mfgpu_mf_detect", mf._h, C.byref(dp), C.byref(n))
        raw = (_lib.MfgpuDetection * max(1, n.value))()
        _lib.call("mfgpu_mf_get_detections", mf._h, n.value, raw, C.byref(n))
        want_wave = prm.want_detected_waveform()
        signals = {}
        meta = {}
        pols = {v: Polarity(v) for v in (-1, 0, 1)}
        for r in raw[: n.value]:
            it = r.template_index
            if it not in meta:
                wt = templates[it]
                meta[it] = (wt.get_identifier() if wt.have_identifier() else (NetworkStationPhase(), it),
                            wt.get_phase_onset_time_in_signal() if wt.have_phase_onset_time() else None,
                            int(wt.get_polarity()),
                            wt.get_phase_travel_time() if wt.have_travel_time() else None,
                            wt.get_signal_length())
            ident, onset, pol, travel, L = meta[it]
            d = Detection()
            d._id = (ident[0], int(ident[1]))
            d._xc = r.correlation  # clamped to [-1, 1] on the device
            d._t = r.detection_time
            d._ti = r.interpolated_time
            if onset is not None:
                d._po = r.detection_time + onset
                d._poi = r.interpolated_time + onset
            d._pol = pols[r.sign * pol]
            if travel is not None:
                d._tt = travel
            if r.have_amplitude:
                d._amp = {RelativeMagnitudeType.gibbons_ringdal_2006: r.gibbons_ringdal,
                          RelativeMagnitudeType.schaff_richards_2014: r.schaff_richards}
            if want_wave:
                # single-channel objects hold one signal (slot 0)
                slot = 0 if mf._params.get_detection_mode() == MatchedFilterDetectionMode.single_channel else it
                if slot not in signals:
                    signals[slot] = MatchedFilter.get_signal(mf, slot)
                d.set_detected_signal(signals[slot][r.sample:r.sample + L])
            self._dets.append(d)
        return self

    def get_number_of_detections(self):
        return len(self._dets)

    def get_detection(self, i):
        if i < 0 or i >= len(self._dets):
            if not self._dets:
                raise ValueError("No detections")
            raise ValueError("i = %d cannot exceed %d" % (i, len(self._dets)))
        return self._dets[i]

    def get_detections(self):
        return list(self._dets)


class RelativeMagnitude:
    """RelativeMagnitude<T> (src/singleChannel/relativeMagnitude.cpp):
    initialize(template), set_detected_signal(y),
    compute_amplitude_scaling_factor(type), compute_magnitude_perturbation
    (type).  The sums run on the GPU (mfgpu_relative_amplitudes, which also
    takes many windows at once: amplitude_scaling_factors)."""

    def __init__(self, dtype=np.float64):
        self._dtype = np.dtype(dtype)
        if self._dtype not in (np.float32, np.float64):
            raise ValueError("dtype must be float32 or float64")
        self.clear()

    def clear(self):
        self._b = None
        self._alpha = None

    def initialize(self, wt):
        self.clear()
        b = np.ascontiguousarray(wt.get_signal(), dtype=np.float64)
        if b.size < 1:
            raise ValueError("Template signal length = %d must be positive" % b.size)
        if np.all(b == b[0]):
            raise ValueError("Template signal cannot be constant")
        self._b = b

    def is_initialized(self):
        return self._b is not None

    def get_detected_signal_length(self):
        if self._b is None:
            raise RuntimeError("Class not initialized")
        return self._b.size

    def amplitude_scaling_factors(self, windows):
        """Extension: (gibbons_ringdal, schaff_richards, valid) for every row
        of the 2-D array windows (n x template length)."""
        if self._b is None:
            raise RuntimeError("Class not initialized")
        y = np.ascontiguousarray(np.atleast_2d(windows), dtype=self._dtype)
        if y.shape[1] != self._b.size:
            raise ValueError("Signal length = %d must = %d" % (y.shape[1], self._b.size))
        nw = y.shape[0]
        gr, sr = np.zeros(max(1, nw)), np.zeros(max(1, nw))
        ok = np.zeros(max(1, nw), dtype=np.int32)
        _lib.call("mfgpu_relative_amplitudes", int(self._dtype.itemsize), int(self._b.size),
                  self._b.ctypes.data_as(C.c_void_p), nw, y.ctypes.data_as(C.c_void_p), int(y.shape[1]),
                  gr.ctypes.data_as(C.c_void_p), sr.ctypes.data_as(C.c_void_p), ok.ctypes.data_as(C.POINTER(C.c_int)))
        return gr[:nw], sr[:nw], ok[:nw].astype(bool)

    def set_detected_signal(self, y):
        self._alpha = None
        gr, sr, ok = self.amplitude_scaling_factors(np.asarray(y).reshape(1, -1))
        if not ok[0]:
            raise ValueError("Detected signal cannot be constant")
        self._alpha = {RelativeMagnitudeType.gibbons_ringdal_2006: float(gr[0]),
                       RelativeMagnitudeType.schaff_richards_2014: float(sr[0])}

    def have_detected_signal(self):
        return self._alpha is not None

    def compute_amplitude_scaling_factor(self, mag_type):
        if self._b is None:
            raise RuntimeError("Class is not initialized")
        if self._alpha is None:
            raise RuntimeError("Detected waveform not set")
        return self._alpha[RelativeMagnitudeType(int(mag_type))]

    def compute_magnitude_perturbation(self, mag_type):
        a = self.compute_amplitude_scaling_factor(mag_type)
        if a <= 0:
            raise ValueError("Scaling factor = %g must be positive" % a)
        return math.log10(a)
