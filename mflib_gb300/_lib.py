"""ctypes binding of libmfgpu.so (the C ABI declared in include/mfgpu.h).

The shared object is built in-tree by ``mflib_gb300/build.py`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is
missing or cannot be loaded, every entry point raises.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmfgpu.so")

MFGPU_OK, MFGPU_EINVAL, MFGPU_ESTATE, MFGPU_ENOMEM, MFGPU_ECUDA, MFGPU_ETIMEOUT = range(6)
MFGPU_FLOAT32, MFGPU_FLOAT64 = 4, 8
MFGPU_SINGLE_CHANNEL, MFGPU_MULTI_CHANNEL = 0, 1

_lock = threading.Lock()
_lib = None


class MfgpuError(RuntimeError):
    """Device, allocation or timeout failure reported by libmfgpu."""


class MfgpuTimeout(MfgpuError):
    """A bounded device-side wait gave up (MFGPU_ETIMEOUT)."""


class MfgpuDetectParams(C.Structure):
    _fields_ = [
        ("threshold", C.c_double),
        ("min_distance", C.c_int),
        ("absolute_maximum", C.c_int),
        ("single", C.c_int),
        ("interpolation", C.c_int),
        ("lanczos_alpha", C.c_int),
        ("lanczos_points", C.c_int),
        ("sampling_rate", C.c_double),
        ("amplitudes", C.c_int),
    ]


class MfgpuDetection(C.Structure):
    _fields_ = [
        ("template_index", C.c_int),
        ("sample", C.c_int),
        ("correlation", C.c_double),
        ("detection_time", C.c_double),
        ("interpolated_time", C.c_double),
        ("sign", C.c_int),
        ("have_amplitude", C.c_int),
        ("gibbons_ringdal", C.c_double),
        ("schaff_richards", C.c_double),
    ]


class MfgpuParams(C.Structure):
    _fields_ = [
        ("detection_mode", C.c_int),
        ("n_templates", C.c_int),
        ("template_lengths", C.POINTER(C.c_int)),
        ("templates", C.POINTER(C.POINTER(C.c_double))),
        ("signal_size", C.c_int),
        ("stack_shifts", C.POINTER(C.c_int)),
        ("stack_weights", C.POINTER(C.c_double)),
        ("stack_absolute_values", C.c_int),
        ("n_channels", C.c_int),
        ("template_channel", C.POINTER(C.c_int)),
        ("fft_length", C.c_int),
        ("correlator_variant", C.c_int),
        ("length_buckets", C.c_int),
        ("n_bucket_plans", C.c_int),
        ("bucket_fft_lengths", C.POINTER(C.c_int)),
        ("bucket_variants", C.POINTER(C.c_int)),
        ("persistent", C.c_int),
        ("tc_bf16", C.c_int),
        ("tc_group", C.c_int),
    ]


_vp = C.c_void_p
_ip = C.POINTER(C.c_int)
_SIGS = {
    "mfgpu_last_error": ([], C.c_char_p),
    "mfgpu_version": ([], C.c_int),
    "mfgpu_device_count": ([_ip], C.c_int),
    "mfgpu_fft_sizes": ([C.c_int, C.c_int, _ip, _ip], C.c_int),
    "mfgpu_window_length": ([C.c_int, C.c_int, _ip, _ip], C.c_int),
    "mfgpu_mf_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
    "mfgpu_mf_destroy": ([_vp], C.c_int),
    "mfgpu_mf_initialize": ([_vp, C.POINTER(MfgpuParams)], C.c_int),
    "mfgpu_mf_clear": ([_vp], C.c_int),
    "mfgpu_mf_is_initialized": ([_vp, _ip], C.c_int),
    "mfgpu_mf_get_number_of_templates": ([_vp, _ip], C.c_int),
    "mfgpu_mf_get_signal_length": ([_vp, _ip], C.c_int),
    "mfgpu_mf_get_filtered_signal_length": ([_vp, _ip], C.c_int),
    "mfgpu_mf_set_signal": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfgpu_mf_zero_signal": ([_vp, C.c_int], C.c_int),
    "mfgpu_mf_get_signal": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfgpu_mf_apply": ([_vp], C.c_int),
    "mfgpu_mf_have_matched_filtered_signals": ([_vp, _ip], C.c_int),
    "mfgpu_mf_get_matched_filtered_signal": ([_vp, C.c_int, C.c_int, _vp, _ip], C.c_int),
    "mfgpu_mf_shift_and_stack": ([_vp, C.c_int, _vp, _ip], C.c_int),
    "mfgpu_mf_get_spectra_of_template": ([_vp, C.c_int, C.c_int, _vp, _ip], C.c_int),
    "mfgpu_mf_set_channel_signal": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfgpu_mf_set_channel_signals": ([_vp, C.c_int, C.c_int, C.c_int, _vp, C.c_long], C.c_int),
    "mfgpu_mf_stage_channel_signals": ([_vp, C.c_int, _vp, C.c_long], C.c_int),
    "mfgpu_mf_set_channel_signal_device": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfgpu_mf_get_valid_signal": ([_vp, C.c_int, C.c_int, _vp, _ip], C.c_int),
    "mfgpu_mf_get_device_signal": ([_vp, C.c_int, C.POINTER(_vp), _ip], C.c_int),
    "mfgpu_mf_get_plan": ([_vp, _ip, _ip, _ip], C.c_int),
    "mfgpu_mf_get_correlator": ([_vp, _ip, _ip, _ip], C.c_int),
    "mfgpu_mf_get_buckets": ([_vp, C.c_int, _ip, _ip, _ip], C.c_int),
    "mfgpu_mf_get_bucket_plans": ([_vp, C.c_int, _ip, _ip, _ip], C.c_int),
    "mfgpu_mf_detect": ([_vp, C.POINTER(MfgpuDetectParams), _ip], C.c_int),
    "mfgpu_mf_set_graph": ([_vp, C.c_int], C.c_int),
    "mfgpu_mf_get_graph_launches": ([_vp, C.POINTER(C.c_longlong)], C.c_int),
    "mfgpu_relative_amplitudes": ([C.c_int, C.c_int, _vp, C.c_int, _vp, C.c_long, _vp, _vp, _ip], C.c_int),
    "mfgpu_mf_get_detections": ([_vp, C.c_int, C.POINTER(MfgpuDetection), _ip], C.c_int),
    "mfgpu_mf_set_window": ([_vp, C.c_int, C.c_int, _vp, C.c_long], C.c_int),
    "mfgpu_ring_create": ([C.c_int, C.c_int, C.c_long, C.POINTER(_vp)], C.c_int),
    "mfgpu_ring_destroy": ([_vp], C.c_int),
    "mfgpu_ring_append": ([_vp, C.c_int, _vp, C.c_long], C.c_int),
    "mfgpu_ring_get_head": ([_vp, C.POINTER(C.c_longlong)], C.c_int),
    "mfgpu_mf_set_window_ring": ([_vp, _vp, C.c_int, _ip, C.c_longlong, C.c_int], C.c_int),
    "mfgpu_mf_get_device_bytes": ([_vp, C.POINTER(C.c_ulonglong)], C.c_int),
    "mfgpu_mf_synchronize": ([_vp], C.c_int),
    "mfgpu_mf_get_last_timings": ([_vp, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "mfgpu_mf_get_launch_count": ([_vp, C.POINTER(C.c_longlong)], C.c_int),
    "mfgpu_mf_get_fixup_runs": ([_vp, C.POINTER(C.c_longlong)], C.c_int),
    "mfgpu_mf_test_wait_timeout": ([_vp], C.c_int),
    "mfgpu_mf_test_skip_fixup": ([_vp, C.c_int], C.c_int),
    "mfgpu_mf_get_stream": ([_vp, C.POINTER(_vp)], C.c_int),
    "mfgpu_mf_find_peaks": ([_vp, C.c_double, C.c_int, C.c_int], C.c_int),
    "mfgpu_mf_set_peak_threshold": ([_vp, C.c_double], C.c_int),
    "mfgpu_mf_get_peak_threshold": ([_vp, C.POINTER(C.c_double), _ip], C.c_int),
    "mfgpu_mf_get_peaks": ([_vp, C.c_int, C.c_int, _ip, _ip], C.c_int),
    "mfgpu_mf_get_all_peaks": ([_vp, C.c_int, _ip, C.c_int, _ip, _ip], C.c_int),
    "mfgpu_peaks_create": ([C.c_int, C.POINTER(_vp)], C.c_int),
    "mfgpu_peaks_destroy": ([_vp], C.c_int),
    "mfgpu_peaks_set_threshold": ([_vp, C.c_double], C.c_int),
    "mfgpu_peaks_get_threshold": ([_vp, C.POINTER(C.c_double)], C.c_int),
    "mfgpu_peaks_set_minimum_peak_distance": ([_vp, C.c_int], C.c_int),
    "mfgpu_peaks_get_minimum_peak_distance": ([_vp, _ip], C.c_int),
    "mfgpu_peaks_set_signal": ([_vp, C.c_int, _vp], C.c_int),
    "mfgpu_peaks_apply": ([_vp], C.c_int),
    "mfgpu_peaks_get_number_of_peaks": ([_vp, _ip], C.c_int),
    "mfgpu_peaks_get_peak_indices": ([_vp, C.c_int, _ip], C.c_int),
    "mfgpu_peaks_clear": ([_vp], C.c_int),
    "mfgpu_dbscan_create": ([C.POINTER(_vp)], C.c_int),
    "mfgpu_dbscan_destroy": ([_vp], C.c_int),
    "mfgpu_dbscan_initialize": ([_vp, C.c_double, C.c_int], C.c_int),
    "mfgpu_dbscan_set_data": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfgpu_dbscan_set_weighted_data": ([_vp, C.c_int, C.c_int, _vp, _vp], C.c_int),
    "mfgpu_dbscan_cluster": ([_vp], C.c_int),
    "mfgpu_dbscan_get_number_of_clusters": ([_vp, _ip], C.c_int),
    "mfgpu_dbscan_get_labels": ([_vp, C.c_int, _ip], C.c_int),
    "mfgpu_dbscan_get_launch_count": ([_vp, C.POINTER(C.c_longlong)], C.c_int),
    "mfgpu_dbscan_is_initialized": ([_vp, _ip], C.c_int),
    "mfgpu_dbscan_have_data": ([_vp, _ip], C.c_int),
    "mfgpu_dbscan_have_labels": ([_vp, _ip], C.c_int),
    "mfgpu_dbscan_clear": ([_vp], C.c_int),
    "mfgpu_dbscan_segmented": ([_vp, C.c_int, _ip, C.c_int, _vp, _vp, _ip, _ip], C.c_int),
    "mfgpu_dbscan_segmented_noalloc": ([C.c_int, _vp, C.c_int, C.c_int, _vp, _vp, C.c_double, C.c_int, _vp, _vp,
                                        _vp], C.c_int),
}


def exported_symbols():
    """Names of every entry point this binding expects libmfgpu.so to export."""
    return sorted(_SIGS)


def lib():
    """Load libmfgpu.so (once).  Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise MfgpuError("libmfgpu.so is missing (%s): build it with "
                                 "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
            L = C.CDLL(LIB_PATH)
            for name, (args, res) in _SIGS.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            _lib = L
        return _lib


def check(status):
    """Map an mfgpu_status to the reference's exception types."""
    if status == MFGPU_OK:
        return
    msg = lib().mfgpu_last_error().decode(errors="replace")
    if status == MFGPU_EINVAL:
        raise ValueError(msg)
    if status == MFGPU_ESTATE:
        raise RuntimeError(msg)
    if status == MFGPU_ENOMEM:
        raise MemoryError(msg)
    if status == MFGPU_ETIMEOUT:
        raise MfgpuTimeout(msg)
    raise MfgpuError(msg)


def call(name, *args):
    check(getattr(lib(), name)(*args))
