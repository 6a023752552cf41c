"""Single-channel associator: MFLib::SingleChannel::{Associator,
AssociatorParameters} with the pymflib names
(python/singleChannel/associator*.cpp, src/singleChannel/associator.cpp).

Detections are grouped by their template identifier's id (the event id),
each group sorted by phase onset time, and the origin times (onset - travel
time) of every group clustered by DBSCAN with eps = the origin-time
tolerance and minPts = the minimum number of picks, optionally weighted by
the correlation coefficients (Associator<T>::associate,
src/singleChannel/associator.cpp:156-267).  All groups go to the GPU in one
segmented DBSCAN call (mfgpu_dbscan_segmented); each cluster becomes an
event, events ordered by event id, then cluster.

Differences from the reference, kept on purpose: the sorts are stable (the
reference uses std::sort, so detections with equal ids or onset times come
out in unspecified order); get_detections_in_event checks the event index
against the number of events (the reference checks it against the number of
detections, :277-286).
"""
import numpy as np

from .detection import DBSCAN


class AssociatorParameters:
    """src/singleChannel/associatorParameters.cpp (defaults :10-18)."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._tol, self._minp, self._xcw = 2.0, 5, False

    def set_origin_time_tolerance(self, tol):
        if tol < 0:
            raise ValueError("tolerance = %g must be positive" % tol)
        self._tol = float(tol)

    def get_origin_time_tolerance(self):
        return self._tol

    def set_minimum_number_of_picks_in_event(self, n):
        if n < 1:
            raise ValueError("minPicks = %d must be positive" % n)
        self._minp = int(n)

    def get_minimum_number_of_picks_in_event(self):
        return self._minp

    def enable_correlation_coefficient_weighting(self):
        self._xcw = True

    def disable_correlation_coefficient_weighting(self):
        self._xcw = False

    def use_correlation_coefficient_weighting(self):
        return self._xcw


class Associator:
    """Associator<T>: initialize, add_detection, associate,
    get_number_of_events, get_detections_in_event."""

    def __init__(self):
        self._db = None
        self.clear()

    def clear(self):
        self._params = None
        self._dets = []
        self._events = []

    def initialize(self, parameters):
        if not isinstance(parameters, AssociatorParameters):
            raise ValueError("parameters must be AssociatorParameters")
        self.clear()
        p = AssociatorParameters()
        p._tol, p._minp, p._xcw = parameters._tol, parameters._minp, parameters._xcw
        self._params = p

    def is_initialized(self):
        return self._params is not None

    def add_detection(self, det):
        """addDetection (:100-122): travel time and template identifier
        required, and the coefficient when weighting."""
        self._events = []
        if not self.is_initialized():
            raise RuntimeError("Class not initialized")
        if not det.have_travel_time():
            raise ValueError("Travel time must be set")
        if not det.have_template_identifier():
            raise ValueError("Template identifier must be set")
        if self._params.use_correlation_coefficient_weighting() and not det.have_correlation_coefficient():
            raise ValueError("XC coefficient must be set")
        self._dets.append(det)

    def get_number_of_detections(self):
        return len(self._dets)

    def clear_detections(self):
        self._dets = []
        self._events = []

    def associate(self):
        self._events = []
        if not self.is_initialized():
            raise RuntimeError("Class is not intialized")
        if not self._dets:
            return
        evid = np.array([d.get_template_identifier()[1] for d in self._dets], dtype=np.uint64)
        onset = np.array([d.get_phase_onset_time() for d in self._dets], dtype=np.float64)
        travel = np.array([d.get_travel_time() for d in self._dets], dtype=np.float64)
        # by event id, then onset time (stable)
        order = np.lexsort((onset, evid))
        self._dets = [self._dets[i] for i in order]
        evid, onset, travel = evid[order], onset[order], travel[order]
        ids, starts = np.unique(evid, return_index=True)
        offs = np.append(starts, evid.size).astype(np.int32)
        origin = (onset - travel).reshape(-1, 1)
        w = None
        if self._params.use_correlation_coefficient_weighting():
            w = np.array([d.get_correlation_coefficient() for d in self._dets], dtype=np.float64)
            if np.any(w <= 0):
                raise ValueError("All weights must be positive")
        if self._db is None:
            self._db = DBSCAN()
        self._db.initialize(self._params.get_origin_time_tolerance(),
                            self._params.get_minimum_number_of_picks_in_event())
        labels, ncl = self._db.cluster_segments(origin, offs, w)
        for s, e in enumerate(ids):
            lab = labels[offs[s]:offs[s + 1]]
            for ic in range(int(ncl[s])):
                self._events.append((int(e), [int(offs[s] + i) for i in np.nonzero(lab == ic)[0]]))

    def get_number_of_events(self):
        return len(self._events)

    def get_detections_in_event(self, iev):
        """The detections of event iev; an empty list when there are no events
        (pymflib, python/singleChannel/associator.cpp:127-133)."""
        if not self._events:
            return []
        if iev < 0 or iev >= len(self._events):
            raise ValueError("iev = %d must be in range [0,%d]" % (iev, len(self._events) - 1))
        return [self._dets[i] for i in self._events[iev][1]]

    def get_event_id(self, iev):
        """Extension: the event id (template identifier id) of event iev."""
        if iev < 0 or iev >= len(self._events):
            raise ValueError("iev out of range")
        return self._events[iev][0]


# Summary statistics of an event's picks (include/private/weightedStatistics.hpp:
# median, weightedMedian, mean, weightedMean).  Sums run left to right, as
# std::accumulate does.
def median(x):
    """Median of x; 0 for no values (weightedStatistics.hpp:17-32)."""
    x = np.sort(np.asarray(x, dtype=np.float64).ravel())
    n = x.size
    if n == 0:
        return 0.0
    return float(x[n // 2]) if n % 2 else float((x[n // 2 - 1] + x[n // 2]) / 2)


def weighted_median(x, weights=None):
    """Weighted median (weightedStatistics.hpp:42-85): the x at which the
    weights' normalised cumulative sum, over x sorted ascending, reaches 1/2,
    interpolated linearly between the two observations that straddle it; x
    itself where the sum equals 1/2 exactly.  No weights: the median."""
    x = np.asarray(x, dtype=np.float64).ravel()
    n = x.size
    if n == 0:
        return 0.0
    if n == 1:
        return float(x[0])
    if weights is None:
        return median(x)
    w = np.asarray(weights, dtype=np.float64).ravel()
    if w.size != n:
        raise ValueError("weights must have one value per observation")
    order = np.argsort(x, kind="stable")
    xs, cdf = x[order], np.cumsum(w[order] / np.cumsum(w)[-1])
    if cdf[0] > 0.5:
        return float(xs[0])
    i = int(np.argmax(cdf[1:] >= 0.5)) + 1
    if not cdf[i] >= 0.5:
        return float(xs[0])
    if cdf[i] == 0.5:
        return float(xs[i])
    return float(xs[i - 1] + (xs[i] - xs[i - 1]) * (0.5 - cdf[i - 1]) / (cdf[i] - cdf[i - 1]))


def mean(x):
    """Mean of x; 0 for no values (weightedStatistics.hpp:90-96)."""
    x = np.asarray(x, dtype=np.float64).ravel()
    return float(np.cumsum(x)[-1] / x.size) if x.size else 0.0


def weighted_mean(x, weights=None):
    """Sum of x w over the sum of w (weightedStatistics.hpp:106-115); no
    weights: the mean."""
    x = np.asarray(x, dtype=np.float64).ravel()
    n = x.size
    if n == 0:
        return 0.0
    if n == 1:
        return float(x[0])
    if weights is None:
        return mean(x)
    w = np.asarray(weights, dtype=np.float64).ravel()
    if w.size != n:
        raise ValueError("weights must have one value per observation")
    return float(np.cumsum(x * w)[-1] / np.cumsum(w)[-1])
