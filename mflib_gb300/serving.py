"""Request loop for detection requests on one GPU.

The reference library has no serving layer: its MatchedFilter objects are
initialised once for a fixed signal length and driven by one thread
(src/matchedFilter.cpp).  This module keeps template banks resident on the
device and serves detection requests as they arrive.

* A ``TemplateBank`` is a named list of templates, each assigned to one of
  64 channel slots.
* A ``DetectionRequest`` is a window of continuous data on C = 1..64
  channels (C x n samples) against one bank, given as a host array or as
  a window of a ``SignalRing`` (the stations' latest samples kept on the
  device: producers append only new samples, and the request's window is
  gathered from the ring on the device instead of uploaded).  Template t of the bank
  correlates with request channel ``slot_t % C``.  The result is, for every
  template, the PeakFinder indices (threshold and minimum separation of the
  server) over the window's valid lags n - L_max + 1, the reference's
  filtered-signal length (src/matchedFilter.cpp:941-969); requests may also
  ask for the Pearson traces of chosen templates.
* Resident state: for each (bank, window bucket) a pool of MatchedFilter
  objects, each holding the bank's template spectra (or tensor-core
  operands) and its own CUDA streams.  A window is rounded up to its bucket
  with a zero tail; coefficients at the valid lags read window samples only,
  so the result does not depend on the bucket.
* Admission: a worker slot takes the oldest waiting request and needs an
  object of its (bank, bucket): an idle one, or a new one if the device
  bytes held by all objects stay within the memory budget (idle objects of
  other keys are evicted, least recently used first).  Otherwise the slot
  waits for a release while the other slots go on with later requests.
* Continuous batching: the slots run concurrently, each on its object's
  streams, so a request that arrives while others are on the GPU starts as
  soon as a slot and memory are free and its kernels overlap theirs.  Each
  object's work is the same whatever else runs, so a request's result is
  the same alone and in the mix.

The executor (``GpuExecutor``) is the only part that touches the device; the
queue, admission and statistics are plain host logic.
"""
import collections
import threading
import time

import numpy as np

N_SLOTS = 64
DEFAULT_BUCKETS = (7_500, 10_000, 15_000, 20_000, 30_000, 40_000, 60_000)


class TemplateBank:
    """Named template bank: FP64 templates and their channel slots (0..63,
    default t % 64)."""

    def __init__(self, name, templates, channel_slots=None, sampling_rate=100.0):
        if not templates:
            raise ValueError("a bank needs at least one template")
        self.name = str(name)
        self.templates = [np.ascontiguousarray(t, dtype=np.float64) for t in templates]
        nt = len(self.templates)
        slots = np.arange(nt) % N_SLOTS if channel_slots is None else np.asarray(channel_slots, dtype=np.int64)
        if slots.shape != (nt,) or slots.min() < 0 or slots.max() >= N_SLOTS:
            raise ValueError("channel slots must be %d values in [0, %d)" % (nt, N_SLOTS))
        self.slots = slots
        self.sampling_rate = float(sampling_rate)
        self.lengths = np.array([t.size for t in self.templates])
        self.max_length = int(self.lengths.max())

    def __len__(self):
        return len(self.templates)

    def valid_lags(self, n):
        """Lags per template of a window of n samples (n - L_max + 1)."""
        return max(0, n - self.max_length + 1)


class DetectionRequest:
    """A window (C x n samples) against a named bank: host ``signals``, or
    samples [end - n, end) of the ring channels ``channels`` of ``ring``
    (``end`` defaults to the ring's head when the request is made).
    ``keep`` lists templates whose Pearson traces are returned besides the
    peaks."""

    _ids = iter(range(1 << 62))

    def __init__(self, bank, signals=None, keep=(), arrival=None, ring=None, channels=None, n=None, end=None):
        self.ring = ring
        if ring is not None:
            if signals is not None:
                raise ValueError("give signals or a ring window, not both")
            ch = np.asarray(channels if channels is not None else np.arange(ring.n_channels), dtype=np.int64)
            if ch.ndim != 1 or not 1 <= ch.size <= N_SLOTS or ch.min() < 0 or ch.max() >= ring.n_channels:
                raise ValueError("channels must list 1..%d ring channels" % N_SLOTS)
            if n is None or int(n) < 1:
                raise ValueError("a ring window needs its length n")
            self.ring_channels = ch
            self._n = int(n)
            self.end = int(ring.head if end is None else end)
            x = None
        else:
            x = np.asarray(signals)
            if x.ndim == 1:
                x = x[None, :]
            if x.ndim != 2 or not 1 <= x.shape[0] <= N_SLOTS or x.shape[1] < 1:
                raise ValueError("signals must be C x n with 1 <= C <= %d" % N_SLOTS)
        self.id = next(DetectionRequest._ids)
        self.bank = str(bank)
        self.signals = x
        self.keep = tuple(int(t) for t in keep)
        self.t_arrival = arrival
        self.t_start = self.t_done = None
        self.peaks = None  # per template its int32 peak indices (peaks[t])
        self.rho = {}
        self.error = None
        self.lags = 0
        self._done = threading.Event()

    @property
    def channels(self):
        return self.ring_channels.size if self.ring is not None else self.signals.shape[0]

    @property
    def n(self):
        return self._n if self.ring is not None else self.signals.shape[1]

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival

    def wait(self, timeout=None):
        """Block until served; raises the request's error, if any."""
        if not self._done.wait(timeout):
            raise TimeoutError("request %d not served within %s s" % (self.id, timeout))
        if self.error is not None:
            raise self.error
        return self


class _Peaks:
    """Peak indices of every template of a request, kept as one flat array
    with offsets; template t's indices are sliced out when asked for."""

    __slots__ = ("_off", "_idx")

    def __init__(self, counts, idx):
        self._off = np.concatenate([[0], np.cumsum(counts)])
        self._idx = idx

    def __len__(self):
        return self._off.size - 1

    def __getitem__(self, t):
        if t < 0:
            t += len(self)
        if not 0 <= t < len(self):
            raise IndexError(t)
        return self._idx[self._off[t]:self._off[t + 1]]

    def __iter__(self):
        return (self[t] for t in range(len(self)))

    def counts(self):
        return np.diff(self._off)


class GpuExecutor:
    """Runs requests on MatchedFilter objects of the CUDA library."""

    def __init__(self, threshold=0.7, min_distance=250, correlator_variant=0):
        from . import MultiChannel, WaveformTemplate  # the CUDA library, loaded on first use
        self._MC, self._WT = MultiChannel, WaveformTemplate
        self.threshold = float(threshold)
        self.min_distance = int(min_distance)
        self.correlator_variant = int(correlator_variant)
        self._params = {}  # bank name -> (lock, MatchedFilterParameters)
        self._plock = threading.Lock()

    def estimate_bytes(self, bank, n):
        """Device bytes of an object for (bank, n) before it exists: the
        coefficients, two signal buffers, normalisation rows and resident
        spectra at the largest FFT the planner may pick, with the buffers'
        growth margin."""
        nt = len(bank)
        nfft = 1 << int(np.ceil(np.log2(max(64, 4 * bank.max_length))))
        b = 4 * nt * (n + 64) + 3 * 4 * N_SLOTS * (n + nfft) + 8 * nt * (nfft // 2 + 2)
        return int(1.3 * b) + (16 << 20)

    def create(self, bank, n):
        with self._plock:
            if bank.name not in self._params:
                p = self._MC.MatchedFilterParameters()
                for t in bank.templates:
                    wt = self._WT()
                    wt.set_signal(t)
                    wt.set_sampling_rate(bank.sampling_rate)
                    p.add_template(wt)
                self._params[bank.name] = (threading.Lock(), p)
            lock, p = self._params[bank.name]
        f = self._MC.MatchedFilter(dtype=np.float32)
        with lock:  # initialize copies the parameters
            p.set_signal_size(int(n))
            f.initialize(p, template_channels=[int(s) for s in bank.slots], n_channels=N_SLOTS,
                         correlator_variant=self.correlator_variant)
        f.set_graph(True)  # a pooled object's applies replay one CUDA graph
        return f

    def device_bytes(self, f):
        return f.device_bytes()

    def run(self, f, bank, req):
        if req.ring is not None:
            f.set_window_ring(req.ring, req.end, req.n, req.ring_channels)
        else:
            f.set_window(req.signals.astype(np.float32, copy=False))
        f.apply()
        nv = bank.valid_lags(req.n)
        if nv > 0:
            f.find_peaks(self.threshold, self.min_distance, nv)
            req.peaks = _Peaks(*f.get_all_peaks())
        else:
            req.peaks = _Peaks(np.zeros(len(bank), np.int64), np.zeros(0, np.int32))
        for t in req.keep:
            req.rho[t] = f.get_matched_filtered_signal(t)[:nv].copy()
        req.lags = len(bank) * nv

    def destroy(self, f):
        f.clear()


class Server:
    """Serving loop: ``slots`` worker threads over a FIFO of requests,
    objects pooled per (bank, bucket) within ``memory_budget`` bytes."""

    def __init__(self, banks, executor=None, memory_budget=120e9, slots=4, buckets=DEFAULT_BUCKETS):
        self.banks = {b.name: b for b in banks}
        self.executor = executor if executor is not None else GpuExecutor()
        self.memory_budget = float(memory_budget)
        self.slots = int(slots)
        self.buckets = tuple(sorted(int(b) for b in buckets))
        self._cv = threading.Condition()
        self._queue = collections.deque()
        self._idle = collections.defaultdict(list)  # key -> [object]
        self._lru = collections.OrderedDict()        # id(object) -> (key, object), idle only
        self._bytes = {}                              # id(object) -> device bytes
        self._held = 0                                # bytes of all objects
        self._reserved = 0                            # bytes of objects being created
        self.peak_held = 0
        self.created = 0
        self.evicted = 0
        self.discarded = 0  # objects dropped after a failed request
        self._threads = []
        self._stop = False
        self.served = []

    # -- keys and admission -------------------------------------------------
    def bucket(self, n):
        for b in self.buckets:
            if n <= b:
                return b
        raise ValueError("window of %d samples exceeds the largest bucket (%d)" % (n, self.buckets[-1]))

    def held_bytes(self):
        with self._cv:
            return self._held

    def _evict_one_locked(self):
        _, (key, obj) = self._lru.popitem(last=False)
        self._idle[key].remove(obj)
        self._held -= self._bytes.pop(id(obj))
        self.evicted += 1
        return obj

    def _acquire(self, key):
        bank = self.banks[key[0]]
        est = self.executor.estimate_bytes(bank, key[1])
        if est > self.memory_budget:
            raise MemoryError("bank %s at %d samples needs ~%d bytes, over the budget of %d"
                              % (key[0], key[1], est, self.memory_budget))
        victims = []
        with self._cv:
            while True:
                if self._idle[key]:
                    obj = self._idle[key].pop()
                    self._lru.pop(id(obj))
                    return obj
                while self._held + self._reserved + est > self.memory_budget and self._lru:
                    victims.append(self._evict_one_locked())
                if self._held + self._reserved + est <= self.memory_budget:
                    self._reserved += est
                    break
                self._cv.wait()
        try:
            # inside the try: a failing destroy must not keep the reservation
            for v in victims:
                self.executor.destroy(v)
            obj = self.executor.create(bank, key[1])
            b = self.executor.device_bytes(obj)
        except BaseException:
            with self._cv:
                self._reserved -= est
                self._cv.notify_all()
            raise
        with self._cv:
            self._reserved -= est
            self._bytes[id(obj)] = b
            self._held += b
            self.peak_held = max(self.peak_held, self._held)
            self.created += 1
        return obj

    def _discard(self, obj):
        """Drop an object whose request failed: it leaves the pool instead of
        serving the next request in an unknown state."""
        with self._cv:
            self._held -= self._bytes.pop(id(obj), 0)
            self.discarded += 1
            self._cv.notify_all()
        try:
            self.executor.destroy(obj)
        except Exception:  # noqa: BLE001 -- the request already carries the first error
            pass

    def _release(self, key, obj):
        b = self.executor.device_bytes(obj)  # peak scratch may have grown
        with self._cv:
            self._held += b - self._bytes[id(obj)]
            self._bytes[id(obj)] = b
            self.peak_held = max(self.peak_held, self._held)
            self._idle[key].append(obj)
            self._lru[id(obj)] = (key, obj)
            self._cv.notify_all()

    def warm(self, keys, per_key=1):
        """Create ``per_key`` idle objects per (bank, window length) key
        ahead of traffic, so that concurrent requests find them ready."""
        for bank, n in keys:
            key = (bank, self.bucket(n))
            objs = []
            while len(objs) < per_key:
                objs.append(self._acquire(key))
            for o in objs:
                self._release(key, o)

    # -- request flow -------------------------------------------------------
    def submit(self, req):
        if req.bank not in self.banks:
            raise ValueError("unknown bank %r" % req.bank)
        self.bucket(req.n)
        if req.t_arrival is None:
            req.t_arrival = time.perf_counter()
        with self._cv:
            self._queue.append(req)
            self._cv.notify_all()
        return req

    def _serve(self, req):
        key = (req.bank, self.bucket(req.n))
        try:
            obj = self._acquire(key)
        except BaseException as e:  # noqa: BLE001 -- reported on the request
            req.error = e
            return
        req.t_start = time.perf_counter()
        try:
            self.executor.run(obj, self.banks[req.bank], req)
        except BaseException as e:  # noqa: BLE001
            req.error = e
            self._discard(obj)
        else:
            self._release(key, obj)

    def _worker(self):
        while True:
            with self._cv:
                while not self._queue and not self._stop:
                    self._cv.wait()
                if not self._queue:
                    return
                req = self._queue.popleft()
            self._serve(req)
            req.t_done = time.perf_counter()
            with self._cv:
                self.served.append(req)
            req._done.set()

    def start(self):
        if self._threads:
            return self
        self._stop = False
        self._threads = [threading.Thread(target=self._worker, name="mf-slot-%d" % i, daemon=True)
                         for i in range(self.slots)]
        for t in self._threads:
            t.start()
        return self

    def stop(self):
        """Serve what is queued, then end the worker threads."""
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        self._threads = []

    def close(self):
        """stop() and release every pooled object."""
        self.stop()
        with self._cv:
            objs = [o for _, o in self._lru.values()]
            self._lru.clear()
            self._idle.clear()
            self._bytes.clear()
            self._held = 0
        for o in objs:
            self.executor.destroy(o)

    def run_one(self, req):
        """Serve one request on the calling thread (no queue)."""
        if req.t_arrival is None:
            req.t_arrival = time.perf_counter()
        self._serve(req)
        req.t_done = time.perf_counter()
        req._done.set()
        return req


def latency_stats(reqs):
    """p50 / p99 / mean latency (s) and template-lag correlations/s over the
    span from the first arrival to the last completion."""
    done = [r for r in reqs if r.t_done is not None and r.error is None]
    if not done:
        return {"requests": 0}
    lat = np.array([r.latency for r in done])
    span = max(r.t_done for r in done) - min(r.t_arrival for r in done)
    lags = float(sum(r.lags for r in done))
    return {"requests": len(done), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "span_s": span, "template_lags": lags,
            "throughput": lags / span if span > 0 else None}
