"""Host-side value types of the matched-filter API: NetworkStationPhase,
WaveformTemplate and the enumerations.

These mirror MFLib::NetworkStationPhase (src/networkStationPhase.cpp),
MFLib::WaveformTemplate (src/waveformTemplate.cpp) and include/mflib/enums.hpp
with the pymflib method names (python/waveformTemplate.cpp,
python/networkStationPhase.cpp).  They hold metadata and an FP64 copy of the
template samples; all signal processing happens in libmfgpu.
"""
import enum

import numpy as np


class Polarity(enum.IntEnum):
    """include/mflib/enums.hpp:121-126 (pymflib.Polarity)."""
    unknown = 0
    compression = 1
    dilatation = -1


class MatchedFilterImplementation(enum.IntEnum):
    """include/mflib/enums.hpp:8-14.  The reference stores but never
    dispatches on it (src/matchedFilterParameters.cpp:305-316)."""
    direct = 0
    overlap_add = 1
    auto = 2


class MatchedFilterDetectionMode(enum.IntEnum):
    """include/mflib/enums.hpp:24-32."""
    single_channel = 0
    multi_channel = 1


def _canon(s):
    # src/networkStationPhase.cpp: blanks removed, upper case
    return str(s).replace(" ", "").upper()


class NetworkStationPhase:
    """MFLib::NetworkStationPhase: network, station, channel, location code
    and phase, compared by value (the reference compares a hash of the
    concatenated fields, src/networkStationPhase.cpp:197-213)."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._net = self._sta = self._cha = self._loc = self._pha = ""

    def set_network(self, s): self._net = _canon(s)
    def get_network(self): return self._net
    def set_station(self, s): self._sta = _canon(s)
    def get_station(self): return self._sta
    def set_channel(self, s): self._cha = _canon(s)
    def get_channel(self): return self._cha
    def set_location_code(self, s): self._loc = _canon(s)
    def get_location_code(self): return self._loc
    def set_phase(self, s): self._pha = _canon(s)
    def get_phase(self): return self._pha

    def _key(self):
        return (self._net, self._sta, self._cha, self._loc, self._pha)

    def __eq__(self, other):
        return isinstance(other, NetworkStationPhase) and self._key() == other._key()

    def __hash__(self):
        return hash(self._key())

    def __getstate__(self):
        return self._key()

    def __setstate__(self, st):
        self._net, self._sta, self._cha, self._loc, self._pha = st

    def __repr__(self):
        return "NetworkStationPhase(%s.%s.%s.%s.%s)" % self._key()


class WaveformTemplate:
    """MFLib::WaveformTemplate (src/waveformTemplate.cpp:106-410): FP64
    samples, sampling rate, shift-and-stack weight, phase onset time within
    the template, travel time, magnitude, polarity and identifier."""

    def __init__(self):
        self.clear()

    def clear(self):
        """src/waveformTemplate.cpp:60-78: every field back to its default."""
        self._x = None
        self._fs = 0.0
        self._weight = 1.0
        self._onset = -1.0
        self._travel = -1.0
        self._mag = None
        self._polarity = Polarity.unknown
        self._id = None

    # -- signal (:197-283)
    def set_signal(self, x):
        x = np.array(x, dtype=np.float64).ravel()
        if x.size < 1:
            raise ValueError("npts must be positive")
        self._onset = -1.0
        self._x = x.copy()

    def get_signal(self):
        if self._x is None:
            raise RuntimeError("Signal not set")
        return self._x.copy()

    def have_signal(self):
        return self._x is not None and self._x.size > 0

    def get_signal_length(self):
        if self._x is None:
            raise RuntimeError("Signal not set")
        return int(self._x.size)

    # -- sampling rate (:150-177); setting it resets the onset time like the reference
    def set_sampling_rate(self, fs):
        if fs <= 0:
            raise ValueError("Sampling rate = %g must be positive" % fs)
        self._onset = -1.0
        self._fs = float(fs)

    def get_sampling_rate(self):
        if self._fs <= 0:
            raise RuntimeError("Sampling rate not set")
        return self._fs

    def have_sampling_rate(self):
        return self._fs > 0

    # -- shift-and-stack weight (:180-194)
    def set_shift_and_stack_weight(self, w):
        if w < 0 or w > 1:
            raise ValueError("weight = %g must be in range [0,1]" % w)
        self._weight = float(w)

    def get_shift_and_stack_weight(self):
        return self._weight

    # -- onset time (:287-323).  The reference bounds the onset by
    # (npts - 1) * fs (:297); that bound is kept for compatibility.
    def set_phase_onset_time_in_signal(self, t):
        if t < 0:
            raise ValueError("onsetTime = %g must be positive" % t)
        fs = self.get_sampling_rate()
        npts = self.get_signal_length()
        tmax = (npts - 1) * fs
        if t > tmax:
            raise ValueError("onsetTime = %g cannot exceed maxOnsetTime = %g" % (t, tmax))
        self._onset = float(t)

    def get_phase_onset_time_in_signal(self):
        if self._onset < 0:
            raise RuntimeError("Onset time not set")
        return self._onset

    def have_phase_onset_time(self):
        return self._onset >= 0

    # -- travel time (:326-350)
    def set_phase_travel_time(self, t):
        # pymflib refuses a negative time as an invalid argument
        # (python/waveformTemplate.cpp:151-160; the C++ class throws runtime_error)
        if t < 0:
            raise ValueError("travel time = %g must not be negative" % t)
        self._travel = float(t)

    def get_phase_travel_time(self):
        if self._travel < 0:
            raise RuntimeError("Travel time not yet set")
        return self._travel

    def have_travel_time(self):
        return self._travel >= 0

    # -- identifier, magnitude, polarity (:353-410)
    def set_identifier(self, ident):
        nsp, wid = ident
        if not isinstance(nsp, NetworkStationPhase):
            raise ValueError("identifier must be (NetworkStationPhase, int)")
        cp = NetworkStationPhase()
        cp.__setstate__(nsp.__getstate__())
        self._id = (cp, int(wid))

    def get_identifier(self):
        if self._id is None:
            raise RuntimeError("Waveform identifier not set")
        return [self._id[0], self._id[1]]

    def have_identifier(self):
        return self._id is not None

    def set_magnitude(self, m):
        self._mag = float(m)

    def get_magnitude(self):
        if self._mag is None:
            raise RuntimeError("Magnitude not set")
        return self._mag

    def have_magnitude(self):
        return self._mag is not None

    def set_polarity(self, p):
        self._polarity = Polarity(int(p))

    def get_polarity(self):
        return self._polarity

    # -- pickling (python/waveformTemplate.cpp:279-338 keeps the same fields;
    # samples are kept at full FP64 precision here)
    def __getstate__(self):
        ident = None
        if self._id is not None:
            ident = (self._id[0].__getstate__(), self._id[1])
        return dict(x=None if self._x is None else self._x.tolist(), fs=self._fs, weight=self._weight,
                    onset=self._onset, travel=self._travel, mag=self._mag, polarity=int(self._polarity),
                    ident=ident)

    def __setstate__(self, st):
        self.clear()
        self._x = None if st["x"] is None else np.array(st["x"], dtype=np.float64)
        self._fs, self._weight = st["fs"], st["weight"]
        self._onset, self._travel, self._mag = st["onset"], st["travel"], st["mag"]
        self._polarity = Polarity(st["polarity"])
        if st["ident"] is not None:
            nsp = NetworkStationPhase()
            nsp.__setstate__(st["ident"][0])
            self._id = (nsp, st["ident"][1])

    def copy(self):
        wt = WaveformTemplate()
        wt.__setstate__(self.__getstate__())
        return wt
