"""Matched-filter parameters and engines with the pymflib interface.

``MultiChannel.MatchedFilterParameters`` / ``MultiChannel.MatchedFilter``
mirror python/multiChannelMatchedFilterParameters.cpp and
python/multiChannelMatchedFilter.cpp (MFLib::MatchedFilterParameters and
MFLib::MatchedFilter<T> in MULTI_CHANNEL mode); the ``SingleChannel``
versions mirror python/singleChannel/matchedFilter*.cpp
(MFLib::SingleChannel::*).  The compute runs in libmfgpu on the GPU; this
module only marshals arguments through the C ABI.
"""
import ctypes as C

import numpy as np

from . import _lib
from .waveform import MatchedFilterDetectionMode, MatchedFilterImplementation, WaveformTemplate


def compute_optimal_fft_and_block_length(nb, nx):
    """MFLib::computeOptimalFFTAndBlockLength (src/matchedFilterParameters.cpp:371-385)."""
    a, b = C.c_int(), C.c_int()
    _lib.call("mfgpu_fft_sizes", int(nb), int(nx), C.byref(a), C.byref(b))
    return a.value, b.value


class MatchedFilterParameters:
    """MFLib::MatchedFilterParameters (src/matchedFilterParameters.cpp:108-369)."""

    def __init__(self, detection_mode=MatchedFilterDetectionMode.multi_channel):
        self._mode = MatchedFilterDetectionMode(detection_mode)
        self.clear()

    def clear(self):
        mode = self._mode
        self._templates = []
        self._fs = -1.0
        self._signal_size = 0
        self._fft = 0
        self._block = 0
        self._impl = MatchedFilterImplementation.direct
        self._stack_abs = True
        self._mode = mode

    def add_template(self, wt):
        """:199-219 -- the template must have a signal; sampling rates must agree to 1e-4."""
        self._fft = self._block = 0
        if not isinstance(wt, WaveformTemplate) or not wt.have_signal():
            raise ValueError("Waveform not yet set on template")
        df = wt.get_sampling_rate()
        if self._fs < 0:
            self._fs = df
        if abs(df - self._fs) > 1.e-4:
            raise ValueError("Template sampling rate = %f must equal %f" % (df, self._fs))
        self._templates.append(wt.copy())

    def get_template(self, it):
        nt = len(self._templates)
        if it < 0 or it >= nt:
            raise ValueError("template index = %d must be in range [0,%d]" % (it, nt - 1))
        return self._templates[it].copy()

    def get_number_of_templates(self):
        return len(self._templates)

    def clear_templates(self):
        self._fs = -1.0
        self._templates = []

    def get_max_template_length(self):
        if not self._templates:
            raise RuntimeError("No templates set")
        return max(t.get_signal_length() for t in self._templates)

    def set_signal_size(self, n):
        self._fft = self._block = 0
        if n < 1:
            raise ValueError("Signal size must be positive")
        self._signal_size = int(n)

    def get_signal_size(self):
        """0 while no template is set, as pymflib's binding returns
        (python/multiChannelMatchedFilterParameters.cpp:103-107,
        python/singleChannel/matchedFilterParameters.cpp:99-103)."""
        if not self._templates:
            return 0
        if self._signal_size < 1:
            raise RuntimeError("Signal size not set")
        return self._signal_size

    def set_fft_length(self, n):
        """:250-265 -- stored only: like the reference, initialize() picks its own sizes."""
        if not self._templates:
            raise RuntimeError("No templates set")
        nb = self.get_max_template_length()
        if n < nb:
            raise ValueError("fftLength = %d must be at least %d" % (n, nb))
        self._fft = int(n)
        self._block = self._fft - nb + 1

    def _sizes(self):
        # getFFTLength / getBlockLength (src/matchedFilterParameters.cpp:268-300):
        # the window-length rule, which accepts a signal as long as the template
        if not self._templates:
            raise RuntimeError("Templates must be set prior to calling this")
        if self._fft < 1:
            a, b = C.c_int(), C.c_int()
            _lib.call("mfgpu_window_length", self.get_max_template_length(), self.get_signal_size(),
                      C.byref(a), C.byref(b))
            self._fft, self._block = a.value, b.value
        return self._fft, self._block

    def get_fft_length(self):
        """0 while no template is set, as pymflib's binding returns
        (python/multiChannelMatchedFilterParameters.cpp:79-84)."""
        return self._sizes()[0] if self._templates else 0

    def get_block_length(self):
        return self._sizes()[1] if self._templates else 0

    def block_length(self):
        """pymflib binds this name to getFFTLength (python/multiChannelMatchedFilterParameters.cpp:160-162);
        here it returns the overlap-add block length its docstring describes."""
        return self.get_block_length()

    def set_matched_filter_implementation(self, impl):
        self._impl = MatchedFilterImplementation(impl)

    def get_matched_filter_implementation(self):
        return self._impl

    def set_detection_mode(self, mode):
        self._mode = MatchedFilterDetectionMode(mode)

    def get_detection_mode(self):
        return self._mode

    def set_stack_absolute_values(self, flag):
        self._stack_abs = bool(flag)

    def get_stack_absolute_values(self):
        return self._stack_abs

    def is_valid(self):
        if not self._templates or self._signal_size < 1:
            return False
        return self.get_max_template_length() >= 1


class SignalRing:
    """Extension (no reference counterpart): the latest ``capacity`` samples
    of ``n_channels`` station channels kept on the device.  ``append`` sends
    only new samples; ``MatchedFilter.set_window_ring`` sets a request
    window from the ring by a device gather.  Samples are counted from the
    first append; ``head`` is the count so far."""

    def __init__(self, n_channels, capacity, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("dtype must be float32 or float64")
        prec = _lib.MFGPU_FLOAT32 if self.dtype == np.float32 else _lib.MFGPU_FLOAT64
        h = C.c_void_p()
        _lib.call("mfgpu_ring_create", prec, int(n_channels), int(capacity), C.byref(h))
        self._h = h
        self.n_channels = int(n_channels)
        self.capacity = int(capacity)

    def __del__(self):
        self.close()

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.lib().mfgpu_ring_destroy(h)
            except Exception:
                pass
            self._h = None

    def append(self, x):
        """Append the columns of x (n_channels x n samples) to every channel."""
        x = np.asarray(x)
        if x.ndim == 1:
            x = x[None, :]
        if x.ndim != 2 or x.shape[0] != self.n_channels or x.shape[1] < 1:
            raise ValueError("x must be %d x n samples" % self.n_channels)
        if x.dtype != self.dtype or x.strides[1] != x.itemsize or x.strides[0] % x.itemsize:
            x = np.ascontiguousarray(x, dtype=self.dtype)
        _lib.call("mfgpu_ring_append", self._h, int(x.shape[1]), x.ctypes.data_as(C.c_void_p),
                  int(x.strides[0] // x.itemsize))

    @property
    def head(self):
        v = C.c_longlong()
        _lib.call("mfgpu_ring_get_head", self._h, C.byref(v))
        return v.value


class MatchedFilter:
    """MFLib::MatchedFilter<T> (include/mflib/matchedFilter.hpp:28-178) on the GPU.

    ``dtype`` selects the instantiation (numpy.float64 is the one pymflib
    exposes; numpy.float32 is the FP32 engine)."""

    def __init__(self, dtype=np.float64):
        self._dtype = np.dtype(dtype)
        if self._dtype not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("dtype must be float32 or float64")
        prec = _lib.MFGPU_FLOAT32 if self._dtype == np.float32 else _lib.MFGPU_FLOAT64
        h = C.c_void_p()
        _lib.call("mfgpu_mf_create", prec, C.byref(h))
        self._h = h
        self._params = None
        self._nt = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().mfgpu_mf_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def dtype(self):
        return self._dtype

    def initialize(self, params, template_channels=None, n_channels=None, fft_length=0, correlator_variant=0,
                   length_buckets=0, bucket_plans=None, persistent=False, tc_bf16=False, tc_group=0):
        """MatchedFilter<T>::initialize (src/matchedFilter.cpp:507-821).

        Extensions: ``template_channels`` (one channel index per template,
        with ``n_channels`` channels) lets several templates share one
        signal; ``fft_length`` forces the overlap-save FFT length;
        ``correlator_variant`` forces the correlator organisation (0 automatic,
        1 whole CTA, 2 whole CTA with spectrum prefetch, 3 two teams per CTA,
        templates of one length only; 4 split-precision tensor-core
        correlation, FP32 and templates of one length; 5 two teams with the
        normalisation computed inside each CTA, templates of one length;
        6 two 256-thread teams per 512-thread CTA, FP32 and templates of
        several lengths);
        ``length_buckets`` caps the length buckets of a mixed-length bank
        (0 automatic, 1 one plan for every template); ``bucket_plans``
        overrides the plan of each length bucket (shortest templates first):
        a list of (fft_length, correlator_variant) pairs, 0 keeping the
        automatic choice (see ``autotune``); ``persistent`` runs the FFT
        correlator as one persistent launch fed by a device work ticket
        (FP32, variants 3 and 6; the static grid is the default);
        ``tc_bf16`` splits the tensor-core correlator's operands into BF16
        hi + lo instead of FP16 (its error bound lists more runs for the
        accuracy fix-up); ``tc_group`` sets the
        tensor-core tile shape as templates per group (even, 2..16, MMA N =
        16 per template; 0 automatic)."""
        if not isinstance(params, MatchedFilterParameters) or not params.is_valid():
            raise ValueError("Parameters are invalid")
        tmpls = [params.get_template(i) for i in range(params.get_number_of_templates())]
        nt = len(tmpls)
        arrs = [np.ascontiguousarray(t.get_signal(), dtype=np.float64) for t in tmpls]
        lens = (C.c_int * nt)(*[a.size for a in arrs])
        ptrs = (C.POINTER(C.c_double) * nt)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])
        p = _lib.MfgpuParams()
        p.detection_mode = int(params.get_detection_mode())
        p.n_templates = nt
        p.template_lengths = lens
        p.templates = ptrs
        p.signal_size = params.get_signal_size()
        # shift-and-stack inputs exist only when every template has an onset
        # and a travel time (src/matchedFilter.cpp:577-592)
        if all(t.have_phase_onset_time() and t.have_travel_time() for t in tmpls):
            sh = (C.c_int * nt)(*[int((t.get_phase_travel_time() - t.get_phase_onset_time_in_signal())
                                      * t.get_sampling_rate() + 0.5) for t in tmpls])
            w = (C.c_double * nt)(*[t.get_shift_and_stack_weight() for t in tmpls])
            p.stack_shifts = sh
            p.stack_weights = w
        p.stack_absolute_values = 1 if params.get_stack_absolute_values() else 0
        chans = None
        if template_channels is not None:
            chans = np.ascontiguousarray(template_channels, dtype=np.int32)
            if chans.size != nt:
                raise ValueError("template_channels needs one entry per template")
            p.n_channels = int(n_channels if n_channels is not None else chans.max() + 1)
            p.template_channel = chans.ctypes.data_as(C.POINTER(C.c_int))
        p.fft_length = int(fft_length)
        p.correlator_variant = int(correlator_variant)
        p.length_buckets = int(length_buckets)
        if bucket_plans:
            nbp = len(bucket_plans)
            bfl = (C.c_int * nbp)(*[int(fv[0]) for fv in bucket_plans])
            bva = (C.c_int * nbp)(*[int(fv[1]) for fv in bucket_plans])
            p.n_bucket_plans = nbp
            p.bucket_fft_lengths = bfl
            p.bucket_variants = bva
        p.persistent = 1 if persistent else 0
        p.tc_bf16 = 1 if tc_bf16 else 0
        p.tc_group = int(tc_group)
        _lib.call("mfgpu_mf_initialize", self._h, C.byref(p))
        self._init_kw = dict(template_channels=template_channels, n_channels=n_channels, fft_length=fft_length,
                             correlator_variant=correlator_variant, length_buckets=length_buckets,
                             bucket_plans=list(bucket_plans) if bucket_plans else None, persistent=persistent,
                             tc_bf16=tc_bf16, tc_group=tc_group)
        self._params = params
        self._nt = nt
        self._templates = tmpls
        self._n = params.get_signal_size()

    def clear(self):
        _lib.call("mfgpu_mf_clear", self._h)
        self._params = None
        self._nt = 0

    def is_initialized(self):
        f = C.c_int()
        _lib.call("mfgpu_mf_is_initialized", self._h, C.byref(f))
        return bool(f.value)

    def _int(self, name):
        v = C.c_int()
        _lib.call(name, self._h, C.byref(v))
        return v.value

    def get_number_of_templates(self):
        """0 before initialize, as pymflib's binding returns
        (python/multiChannelMatchedFilter.cpp and
        python/singleChannel/matchedFilter.cpp:97-101); the C++ class throws."""
        if not self.is_initialized():
            return 0
        return self._int("mfgpu_mf_get_number_of_templates")

    def get_signal_length(self):
        return self._int("mfgpu_mf_get_signal_length")

    def get_filtered_signal_length(self):
        return self._int("mfgpu_mf_get_filtered_signal_length")

    def _samples(self, x):
        if x is None:
            raise ValueError("x is null")
        return np.ascontiguousarray(x, dtype=self._dtype).ravel()

    def set_signal(self, it, x):
        """MatchedFilter<T>::setSignal (src/matchedFilter.cpp:863-921)."""
        x = self._samples(x)
        _lib.call("mfgpu_mf_set_signal", self._h, int(it), int(x.size), x.ctypes.data_as(C.c_void_p))

    def set_channel_signal(self, channel, x):
        """Extension: signal of a shared channel (see initialize)."""
        x = self._samples(x)
        _lib.call("mfgpu_mf_set_channel_signal", self._h, int(channel), int(x.size),
                  x.ctypes.data_as(C.c_void_p))

    def set_channel_signals(self, x, first_channel=0):
        """Extension: signals of channels first_channel.. from the rows of a
        2-D array (one copy and one dead-trace pass for all rows).  Rows may
        be strided; pinned host memory makes the copy asynchronous DMA."""
        x = np.asarray(x)
        if x.ndim != 2:
            raise ValueError("x must be 2-D (channels x samples)")
        if x.dtype != self._dtype or x.strides[1] != x.itemsize or x.strides[0] % x.itemsize:
            x = np.ascontiguousarray(x, dtype=self._dtype)
        _lib.call("mfgpu_mf_set_channel_signals", self._h, int(first_channel), int(x.shape[0]), int(x.shape[1]),
                  x.ctypes.data_as(C.c_void_p), int(x.strides[0] // x.itemsize))

    def stage_channel_signals(self, x):
        """Extension: asynchronous upload of every channel (rows of the 2-D
        array x) for the next apply, overlapping the work already enqueued.
        x must stay unchanged until the next apply's results are read (or
        synchronize()); this object keeps references to the last two staged
        arrays so they stay alive."""
        x = np.asarray(x)
        if x.ndim != 2:
            raise ValueError("x must be 2-D (channels x samples)")
        if x.dtype != self._dtype or x.strides[1] != x.itemsize or x.strides[0] % x.itemsize:
            x = np.ascontiguousarray(x, dtype=self._dtype)
        _lib.call("mfgpu_mf_stage_channel_signals", self._h, int(x.shape[1]), x.ctypes.data_as(C.c_void_p),
                  int(x.strides[0] // x.itemsize))
        self._staged = (x, getattr(self, "_staged", (None, None))[0])

    def set_window(self, x):
        """Extension for a serving loop: upload a request window, the rows of
        the 2-D array x (n_src channels x n <= signal-length samples).
        Channel c of this object receives row c % n_src, zero-filled past n;
        dead traces are decided over the n window samples.  Coefficients at
        lags up to n - L_t depend on window samples only."""
        x = np.asarray(x)
        if x.ndim != 2:
            raise ValueError("x must be 2-D (channels x samples)")
        if x.dtype != self._dtype or x.strides[1] != x.itemsize or x.strides[0] % x.itemsize:
            x = np.ascontiguousarray(x, dtype=self._dtype)
        _lib.call("mfgpu_mf_set_window", self._h, int(x.shape[0]), int(x.shape[1]), x.ctypes.data_as(C.c_void_p),
                  int(x.strides[0] // x.itemsize))

    def set_window_ring(self, ring, end, n, channels):
        """Extension for a serving loop: the request window is samples
        [end - n, end) of the ring's channels ``channels`` (a SignalRing of
        this object's dtype), gathered on the device; otherwise as
        ``set_window`` with one source row per listed channel."""
        ch = np.ascontiguousarray(channels, dtype=np.int32)
        if ch.ndim != 1 or ch.size < 1:
            raise ValueError("channels must list at least one ring channel")
        if np.dtype(ring.dtype) != np.dtype(self._dtype):
            raise ValueError("the ring holds %s samples, the object %s" % (np.dtype(ring.dtype).name,
                                                                         np.dtype(self._dtype).name))
        _lib.call("mfgpu_mf_set_window_ring", self._h, ring._h, int(ch.size), ch.ctypes.data_as(C.POINTER(C.c_int)),
                  int(end), int(n))

    def set_graph(self, enable=True):
        """Extension: replay apply as a CUDA graph (captured on the second
        apply with the same input buffer and peak-gathering setup)."""
        _lib.call("mfgpu_mf_set_graph", self._h, 1 if enable else 0)

    def graph_launches(self):
        v = C.c_longlong()
        _lib.call("mfgpu_mf_get_graph_launches", self._h, C.byref(v))
        return v.value

    def device_bytes(self):
        """Device memory held by this object (buffers and peak scratch)."""
        v = C.c_ulonglong()
        _lib.call("mfgpu_mf_get_device_bytes", self._h, C.byref(v))
        return int(v.value)

    def zero_signal(self, it):
        _lib.call("mfgpu_mf_zero_signal", self._h, int(it))

    def get_signal(self, it):
        """Copy of the stored signal (MatchedFilter<T>::getSignalPointer)."""
        out = np.empty(self.get_signal_length(), dtype=self._dtype)
        _lib.call("mfgpu_mf_get_signal", self._h, int(it), int(out.size), out.ctypes.data_as(C.c_void_p))
        return out

    def apply(self):
        _lib.call("mfgpu_mf_apply", self._h)

    def synchronize(self):
        _lib.call("mfgpu_mf_synchronize", self._h)

    def have_matched_filtered_signals(self):
        f = C.c_int()
        _lib.call("mfgpu_mf_have_matched_filtered_signals", self._h, C.byref(f))
        return bool(f.value)

    def get_matched_filtered_signal(self, it):
        """Coefficients of template it at lags 0..getFilteredSignalLength()-1."""
        n = max(0, self.get_filtered_signal_length())
        out = np.empty(max(n, 1), dtype=self._dtype)
        cnt = C.c_int()
        _lib.call("mfgpu_mf_get_matched_filtered_signal", self._h, int(it), int(out.size),
                  out.ctypes.data_as(C.c_void_p), C.byref(cnt))
        return out[: cnt.value]

    def get_valid_matched_filtered_signal(self, it):
        """Extension: every valid lag of template it (n - L_t + 1 values)."""
        out = np.empty(max(self.get_signal_length(), 1), dtype=self._dtype)
        cnt = C.c_int()
        _lib.call("mfgpu_mf_get_valid_signal", self._h, int(it), int(out.size), out.ctypes.data_as(C.c_void_p),
                  C.byref(cnt))
        return out[: cnt.value]

    def shift_and_stack(self):
        out = np.empty(max(self.get_filtered_signal_length(), 1), dtype=self._dtype)
        cnt = C.c_int()
        _lib.call("mfgpu_mf_shift_and_stack", self._h, int(out.size), out.ctypes.data_as(C.c_void_p),
                  C.byref(cnt))
        return out[: cnt.value]

    def get_spectra_of_template(self, it):
        """Debug view (src/matchedFilter.cpp:1412-1431): rfft of the reversed,
        demeaned, unit-norm template at the reference's FFT length."""
        nfft, _ = compute_optimal_fft_and_block_length(self._templates and max(
            t.get_signal_length() for t in self._templates), self._n + max(
            t.get_signal_length() for t in self._templates) - 1)
        buf = np.empty(2 * (nfft // 2 + 1), dtype=self._dtype)
        cnt = C.c_int()
        _lib.call("mfgpu_mf_get_spectra_of_template", self._h, int(it), int(buf.size),
                  buf.ctypes.data_as(C.c_void_p), C.byref(cnt))
        return buf[0::2] + 1j * buf[1::2]

    def get_waveform_template(self, it):
        if it < 0 or it >= self._nt:
            raise ValueError("it = %d must be in the range [0,%d]" % (it, self._nt - 1))
        return self._templates[it].copy()

    # -- extensions ---------------------------------------------------------
    def get_plan(self):
        """The plan chosen at initialize: FFT length, lags per block, blocks,
        and the correlator (1-3, 5 FFT organisations, 4 tensor cores; for the
        latter also the templates per group and the padded K)."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _lib.call("mfgpu_mf_get_plan", self._h, C.byref(a), C.byref(b), C.byref(c))
        v, g, k = C.c_int(), C.c_int(), C.c_int()
        _lib.call("mfgpu_mf_get_correlator", self._h, C.byref(v), C.byref(g), C.byref(k))
        cnt = C.c_int()
        fl, ntb = (C.c_int * 8)(), (C.c_int * 8)()
        _lib.call("mfgpu_mf_get_buckets", self._h, 8, fl, ntb, C.byref(cnt))
        lpb, bv = (C.c_int * 8)(), (C.c_int * 8)()
        _lib.call("mfgpu_mf_get_bucket_plans", self._h, 8, lpb, bv, C.byref(cnt))
        nb = min(8, cnt.value)
        return {"fft_length": a.value, "lags_per_block": b.value, "n_blocks": c.value, "correlator": v.value,
                "tc_group": g.value, "tc_k": k.value,
                "buckets": [(fl[i], ntb[i]) for i in range(nb)],
                "bucket_plans": [{"fft_length": fl[i], "templates": ntb[i], "lags_per_block": lpb[i],
                                  "correlator": bv[i]} for i in range(nb)]}

    def autotune(self, x, repeats=3, max_buckets=3, fft_lengths=None, variants=None, tc_groups=(2, 4, 6, 8, 12, 16)):
        """Extension: measured plan choice on this object's templates and the
        signals ``x`` (a 2-D array: channel rows when the object was
        initialised with shared channels, else one row per signal slot).

        The planner's choice comes from a cost model calibrated on GB300;
        this times the real thing instead.  For 1 .. ``max_buckets`` length
        buckets (a mixed-length bank; one bucket for one length) it re-plans
        every bucket in turn (coordinate descent, shortest bucket first) over
        the FFT lengths half, equal to and twice the current one and every
        organisation allowed for the bucket, timing ``repeats`` applies of
        each candidate after one untimed apply; for one template length in
        FP32 it also times the tensor-core correlator at its automatic tile
        shape and at each of ``tc_groups`` templates per group (the MMA's N).  The object is left
        initialised with the fastest configuration (its signals loaded) and
        the method returns it with its apply time and every trial.
        ``fft_lengths`` / ``variants`` restrict the candidates.  User-forced
        fft_length and correlator_variant are replaced by the tuned plans.
        Candidates that do not fit (invalid argument, no device memory) are
        recorded with their error and skipped; any other failure puts the
        object back on the configuration it had, then propagates."""
        if self._params is None:
            raise RuntimeError("Class not initialized")
        x = np.asarray(x)
        if x.ndim != 2:
            raise ValueError("x must be 2-D")
        base = dict(self._init_kw)
        params = self._params
        peak_thr = getattr(self, "_peak_thr", None)
        lens = [t.get_signal_length() for t in self._templates]
        one_length = min(lens) == max(lens)

        def load():
            if base["template_channels"] is not None:
                self.set_channel_signals(x)
            else:
                for i in range(x.shape[0]):
                    MatchedFilter.set_signal(self, i, x[i])  # slot i (SingleChannel: slot 0 only)
            if peak_thr is not None:
                self.set_peak_threshold(peak_thr)

        trials = []

        def run(kw):
            try:
                self.initialize(params, **kw)
            except (ValueError, RuntimeError, MemoryError) as e:  # infeasible, or no room for this plan
                trials.append({"config": kw, "apply_ms": None, "error": str(e)})
                return None
            load()
            self.apply()
            self.synchronize()
            ts = []
            for _ in range(max(1, int(repeats))):
                self.apply()
                self.synchronize()
                ts.append(self.last_timings()["apply_ms"])
            ms = float(np.median(ts))
            trials.append({"config": kw, "apply_ms": ms, "plan": self.get_plan()})
            return ms

        def common(**over):
            kw = dict(base, fft_length=0, correlator_variant=0, tc_group=0)
            kw.update(over)
            return kw

        try:
            best_ms, best_kw = None, None
            allowed_v = [1, 2, 3, 5] if one_length else [1, 2]
            if variants is not None:
                allowed_v = [v for v in allowed_v if v in variants]
            for nb in range(1, (1 if one_length else max(1, int(max_buckets))) + 1):
                kw = common(length_buckets=nb, bucket_plans=None)
                ms = run(kw)
                if ms is None:
                    continue
                plans = [(bp["fft_length"], bp["correlator"]) for bp in self.get_plan()["bucket_plans"]]
                if any(v == 4 for _, v in plans):
                    plans = [(0, 0)] * len(plans)  # the automatic choice took the tensor cores: tune the FFT plans
                cur_ms, cur = ms, plans
                for b in range(len(plans)):
                    f0 = plans[b][0] if plans[b][0] > 0 else self.get_plan()["fft_length"]
                    fmax = 8192 if self._dtype == np.float32 else 4096  # longest transforms built
                    cands_f = [f for f in (f0 // 2, f0, 2 * f0) if 64 <= f <= fmax]
                    if fft_lengths is not None:
                        cands_f = [f for f in cands_f if f in fft_lengths]
                    for f in cands_f:
                        for v in allowed_v:
                            if (f, v) == cur[b]:
                                continue
                            trial = list(cur)
                            trial[b] = (f, v)
                            ms = run(common(length_buckets=nb, bucket_plans=trial))
                            if ms is not None and ms < cur_ms:
                                cur_ms, cur = ms, trial
                if best_ms is None or cur_ms < best_ms:
                    best_ms, best_kw = cur_ms, common(length_buckets=nb, bucket_plans=cur)
            if one_length and self._dtype == np.float32 and (variants is None or 4 in variants):
                seen = set()
                for g in (0,) + tuple(tc_groups or ()):
                    kw = common(correlator_variant=4, length_buckets=1, bucket_plans=None, tc_group=int(g))
                    ms = run(kw)
                    if ms is None:
                        continue  # this tile shape does not fit the templates' length
                    shape = self.get_plan()["tc_group"]
                    if shape in seen:
                        continue
                    seen.add(shape)
                    if best_ms is None or ms < best_ms:
                        best_ms, best_kw = ms, kw
            if best_kw is None:
                raise RuntimeError("no candidate plan could be initialised")
            self.initialize(params, **best_kw)
            load()
        except BaseException:
            # leave the object as it was found (best effort), then re-raise
            try:
                self.initialize(params, **base)
                load()
            except Exception:
                pass
            raise
        return {"config": best_kw, "apply_ms": best_ms, "plan": self.get_plan(), "trials": trials}

    def last_timings(self):
        a, b = C.c_float(), C.c_float()
        _lib.call("mfgpu_mf_get_last_timings", self._h, C.byref(a), C.byref(b))
        return {"xcorr_ms": a.value, "apply_ms": b.value}

    def launch_count(self):
        v = C.c_longlong()
        _lib.call("mfgpu_mf_get_launch_count", self._h, C.byref(v))
        return v.value

    def get_fixup_runs(self):
        """FP32: 32-lag runs the last apply recomputed by direct correlation
        (the correlator's rounding-error bound exceeded 2e-5 of the run's
        quietest window); waits for the apply."""
        v = C.c_longlong()
        _lib.call("mfgpu_mf_get_fixup_runs", self._h, C.byref(v))
        return v.value

    def test_skip_fixup(self, skip=True):
        """Test support: later applies flag the runs over the error bound
        (``get_fixup_runs`` counts them) without recomputing them, so the
        coefficients carry the correlator's raw rounding error."""
        _lib.call("mfgpu_mf_test_skip_fixup", self._h, 1 if skip else 0)

    def stream_handle(self):
        """The object's cudaStream_t as an integer (every launch and copy of
        the object is issued on it)."""
        v = C.c_void_p()
        _lib.call("mfgpu_mf_get_stream", self._h, C.byref(v))
        return v.value or 0

    def find_peaks(self, threshold, min_distance, trace_length=0):
        """PeakFinder<T>::apply on every template's coefficients, on the device."""
        _lib.call("mfgpu_mf_find_peaks", self._h, float(threshold), int(min_distance), int(trace_length))

    def set_peak_threshold(self, threshold):
        """From the next apply on, gather the peak candidates above
        ``threshold`` inside the correlator (None or a negative value: off);
        find_peaks with that threshold then skips its scan of the traces."""
        _lib.call("mfgpu_mf_set_peak_threshold", self._h, -1.0 if threshold is None else float(threshold))
        self._peak_thr = None if threshold is None or threshold < 0 else float(threshold)

    def get_peak_threshold(self):
        """(requested gathering threshold or None, whether the last apply gathered)."""
        v, a = C.c_double(), C.c_int()
        _lib.call("mfgpu_mf_get_peak_threshold", self._h, C.byref(v), C.byref(a))
        return (None if v.value < 0 else v.value), bool(a.value)

    def get_peaks(self, it):
        cap = max(1, self.get_signal_length())
        out = np.empty(cap, dtype=np.int32)
        cnt = C.c_int()
        _lib.call("mfgpu_mf_get_peaks", self._h, int(it), cap, out.ctypes.data_as(C.POINTER(C.c_int)),
                  C.byref(cnt))
        return out[: cnt.value].copy()

    def get_all_peaks(self):
        """(counts[nt], concatenated indices) of the last find_peaks."""
        nt = self._nt
        counts = np.zeros(nt, dtype=np.int32)
        tot = C.c_int()
        _lib.call("mfgpu_mf_get_all_peaks", self._h, nt, counts.ctypes.data_as(C.POINTER(C.c_int)), 0, None,
                  C.byref(tot))
        idx = np.empty(max(1, tot.value), dtype=np.int32)
        _lib.call("mfgpu_mf_get_all_peaks", self._h, nt, counts.ctypes.data_as(C.POINTER(C.c_int)), int(idx.size),
                  idx.ctypes.data_as(C.POINTER(C.c_int)), C.byref(tot))
        return counts, idx[: tot.value].copy()


class _MultiChannel:
    """pymflib.MultiChannel (python/pymflib.cpp:68-70)."""

    class MatchedFilterParameters(MatchedFilterParameters):
        def __init__(self):
            super().__init__(MatchedFilterDetectionMode.multi_channel)

        def set_detection_mode(self, mode):
            raise AttributeError("MultiChannel parameters are always MULTI_CHANNEL")

    class MatchedFilter(MatchedFilter):
        """Multi-channel engine: signal it feeds template it."""

        def initialize(self, params, **kw):
            if params.get_detection_mode() != MatchedFilterDetectionMode.multi_channel:
                raise ValueError("Parameters are invalid")
            super().initialize(params, **kw)


class _SingleChannel:
    """pymflib.SingleChannel matched filter (python/singleChannel/matchedFilter*.cpp,
    src/singleChannel/matchedFilter*.cpp): many templates against one signal."""

    class MatchedFilterParameters(MatchedFilterParameters):
        def __init__(self):
            # src/singleChannel/matchedFilterParameters.cpp:20-25 forces SINGLE_CHANNEL
            super().__init__(MatchedFilterDetectionMode.single_channel)

        def set_detection_mode(self, mode):
            raise AttributeError("SingleChannel parameters are always SINGLE_CHANNEL")

    class MatchedFilter(MatchedFilter):
        def initialize(self, params, **kw):
            if params.get_detection_mode() != MatchedFilterDetectionMode.single_channel:
                raise ValueError("Parameters are invalid")
            super().initialize(params, **kw)

        def set_signal(self, x):
            """src/singleChannel/matchedFilter.cpp:62-67: always signal slot 0."""
            super().set_signal(0, x)

        def zero_signal(self):
            super().zero_signal(0)

        def get_signal(self):
            return super().get_signal(0)


MultiChannel = _MultiChannel
SingleChannel = _SingleChannel


def _attach_detector():
    # pymflib.SingleChannel.{Detector, DetectorParameters, Detection, ...}
    from . import associator as a
    from . import detector as d
    for name in ("Detector", "DetectorParameters", "DetectionTimeInterpolationParameters", "Detection",
                 "RelativeMagnitude"):
        setattr(_SingleChannel, name, getattr(d, name))
    for name in ("Associator", "AssociatorParameters"):
        setattr(_SingleChannel, name, getattr(a, name))
