"""mflib_gb300 -- GB300-native matched-filtering hot path with mflib's API.

Python surface of the pymflib module (python/pymflib.cpp:16-71) for the hot
path: WaveformTemplate, NetworkStationPhase, the enumerations,
MultiChannel.{MatchedFilterParameters, MatchedFilter},
SingleChannel.{MatchedFilterParameters, MatchedFilter}, plus PeakFinder and
DBSCAN.  Every computation runs in libmfgpu.so (hand-written sm_103a CUDA
behind the C ABI in include/mfgpu.h).
"""
from .waveform import (MatchedFilterDetectionMode, MatchedFilterImplementation, NetworkStationPhase,
                       Polarity, WaveformTemplate)
from .matched_filter import (MatchedFilter, MatchedFilterParameters, MultiChannel, SignalRing, SingleChannel,
                             compute_optimal_fft_and_block_length)
from .detection import DBSCAN, PeakFinder
from ._lib import MfgpuError, MfgpuTimeout
from .detector import (DetectionTimeInterpolationType, MatchedFilteredSignalDetectorPolicy,
                       MaximumMatchedFilterPolicy, RelativeMagnitudeType)
from .matched_filter import _attach_detector

# pymflib binds this enumeration under a misspelt name (python/pymflib.cpp:29);
# code written against pymflib uses it
MaxmimumMatchedFilterPolicy = MaximumMatchedFilterPolicy

_attach_detector()

__version__ = "1.0.0"

__all__ = [
    "DBSCAN", "MatchedFilter", "MatchedFilterDetectionMode", "MatchedFilterImplementation",
    "MatchedFilterParameters", "MfgpuError", "MfgpuTimeout", "MultiChannel", "NetworkStationPhase",
    "PeakFinder", "Polarity", "SignalRing", "SingleChannel", "WaveformTemplate",
    "compute_optimal_fft_and_block_length",
    "DetectionTimeInterpolationType", "MatchedFilteredSignalDetectorPolicy", "MaximumMatchedFilterPolicy",
    "MaxmimumMatchedFilterPolicy",
    "RelativeMagnitudeType",
]
