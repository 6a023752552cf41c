"""Benchmark of the matched-filtering hot path on one GB300.

Default workload (the headline line): the uneven bank.  2,000 templates of
200-3,000 samples (uniform) with random 1-15 Hz pass bands, each assigned
to one of 96 channels of 8,640,000 float32 samples (24 h at 100 Hz) of
1-10 Hz band-passed noise.  A step is one apply over the whole day (every
template's Pearson trace, 1.728e10 template-lags; CUDA-graph replay, the
planner's length buckets) plus the batched peak finder (rho > 0.7,
separation 250) with candidates gathered inside the correlator.  Data are
seeded synthetic seismograms (no dataset is used by the reference).

Prints ONE JSON line (rank 0).  `value` is template-lag correlations/s with
inputs resident in HBM; `e2e` is the same metric through the C ABI with
every channel's samples copied from pinned host buffers (staged under the
previous step) and the peaks copied back inside the timed region.  Extra
keys hold the other workloads measured in the same run: the 24-channel
day with peaks and DBSCAN association (`multichannel_day`), the
precision-stress bank on the FFT and split-precision tensor-core paths
(`precision_stress`) and the serving loop at one arrival rate
(`serving`).  `--impl reference` times the reference's algorithm (the CPU
restatement in oracle/) on the host cores instead.  Other modes:
--uneven (the headline alone; with --fp64 in double precision), --day24,
--stress, --serving, --detector.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FS = 100.0
N_STATIONS, N_COMP, N_EVENTS = 8, 3, 8
N_CHANNELS = N_STATIONS * N_COMP
N_SAMPLES = 8_640_000
TEMPLATE_LEN = 500
INJ_PER_EVENT = 50
PEAK_THR, PEAK_SEP = 0.5, 250
DB_EPS, DB_MINPTS = 50.0, 3
METRIC = "template-lag correlations/s"


# ---------------------------------------------------------------------------
# synthetic workload
def bandpass_noise(rng, n, lo, hi, fs=FS, order=4):
    from scipy.signal import butter, sosfilt
    sos = butter(order, [lo, hi], btype="bandpass", fs=fs, output="sos")
    return sosfilt(sos, rng.standard_normal(n)).astype(np.float32)


def gen_channels(seeds, n, lo=1.0, hi=10.0):
    """Band-passed N(0,1) noise, one float32 row per seed (threads: the
    filter runs in compiled code)."""
    from concurrent.futures import ThreadPoolExecutor
    out = np.empty((len(seeds), n), dtype=np.float32)

    def one(i):
        out[i] = bandpass_noise(np.random.default_rng(seeds[i]), n, lo, hi)

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(one, range(len(seeds))))
    return out


def make_template(seed, length=TEMPLATE_LEN, lo=2.0, hi=8.0):
    from scipy.signal import butter, sosfilt
    from scipy.signal.windows import hann
    rng = np.random.default_rng(seed)
    sos = butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos")
    return sosfilt(sos, rng.standard_normal(length)) * hann(length)


def make_workload(n_samples=N_SAMPLES, n_stations=N_STATIONS, n_events=N_EVENTS, inj=INJ_PER_EVENT, seed=10,
                  template_length=TEMPLATE_LEN):
    """Returns dict with channel signals [C, n] float32, templates (list of
    FP64 arrays), template channel/event/shift arrays and the truth."""
    nch = n_stations * N_COMP
    sig = gen_channels([seed + c for c in range(nch)], n_samples)
    rms = float(np.sqrt(np.mean(sig[:, : min(n_samples, 1_000_000)].astype(np.float64) ** 2)))
    rng = np.random.default_rng(1000 + seed)
    shifts = rng.integers(0, 301, (n_events, n_stations))
    templates, tchan, tevent, tshift = [], [], [], []
    for e in range(n_events):
        for c in range(nch):
            templates.append(make_template(100 + e * nch + c, template_length))
            tchan.append(c)
            tevent.append(e)
            tshift.append(int(shifts[e, c // N_COMP]))
    # origin times on a coarse grid: copies never overlap
    slot = 1000
    nslots = (n_samples - 2 * slot) // slot
    picks = rng.choice(nslots, size=min(n_events * inj, (nslots // n_events) * n_events), replace=False)
    origins = (picks.reshape(n_events, -1) + 1) * slot + rng.integers(0, 100, (n_events, picks.size // n_events))
    for t, tp in enumerate(templates):
        c, e, s = tchan[t], tevent[t], tshift[t]
        amp = rng.uniform(0.5, 2.0, origins.shape[1]) * rms / max(1e-12, np.sqrt(np.mean(tp ** 2)))
        for o, a in zip(origins[e], amp):
            sig[c, o + s: o + s + tp.size] += (a * tp).astype(np.float32)
    return dict(signals=sig, templates=templates, tchan=np.array(tchan), tevent=np.array(tevent),
                tshift=np.array(tshift), origins=origins, n=n_samples, nch=nch)


UNEVEN_NT, UNEVEN_NCH, UNEVEN_THR, UNEVEN_SEP = 2000, 96, 0.7, 250


def make_uneven_workload(n_samples=N_SAMPLES, nt=UNEVEN_NT, nch=UNEVEN_NCH, rows=None):
    """The uneven bank: nt templates of 200-3,000 samples (uniform) with
    random 1-15 Hz pass bands (Hann-tapered band-passed noise), each on one
    of nch channels (uniform), against nch channels of band-passed noise
    (only the first `rows` channels' samples are generated when given)."""
    from scipy.signal import butter, sosfilt
    from scipy.signal.windows import hann
    rng = np.random.default_rng(200)
    lens = rng.integers(200, 3001, nt)
    tps = []
    for L in lens:
        lo = rng.uniform(1.0, 7.0)
        hi = rng.uniform(lo + 2.0, 15.0)
        tps.append(sosfilt(butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos"),
                           rng.standard_normal(int(L))) * hann(int(L)))
    chan = rng.integers(0, nch, nt)
    sig = gen_channels([300 + c for c in range(nch if rows is None else rows)], n_samples)
    return dict(signals=sig, templates=tps, tchan=np.array(chan), lens=lens, n=n_samples, nch=nch)


# ---------------------------------------------------------------------------
def build_filter(mf, w, **kw):
    p = mf.MultiChannel.MatchedFilterParameters()
    for tp, s in zip(w["templates"], w["tshift"]):
        wt = mf.WaveformTemplate()
        wt.set_signal(tp)
        wt.set_sampling_rate(FS)
        wt.set_phase_onset_time_in_signal(0.0)
        wt.set_phase_travel_time(s / FS)
        p.add_template(wt)
    p.set_signal_size(w["n"])
    f = mf.MultiChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, template_channels=w["tchan"], n_channels=w["nch"], **kw)
    return f


def associate(db, counts, idx, w):
    """Detections -> origin time (lag - template shift), DBSCAN per event
    (SingleChannel::Associator's use of DBSCAN, src/singleChannel/associator.cpp:192-264)."""
    tev, tsh = w["tevent"], w["tshift"]
    tid = np.repeat(np.arange(counts.size), counts)
    origin = idx.astype(np.float64) - tsh[tid]
    ev = tev[tid]
    order = np.argsort(ev, kind="stable")
    X = origin[order]
    nev = int(tev.max()) + 1
    off = np.searchsorted(ev[order], np.arange(nev + 1)).astype(np.int32)
    labels, ncl = db.cluster_segments(X, off)
    return labels, ncl


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i - 5] for r in self.rows if len(r) >= 9 for i in range(5, 9)
                          if r[i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def max_over_ranks(value, dist, device="cpu"):
    """The largest value over the ranks of the process group (the job's
    time is its slowest rank's); the value itself without a group."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_detections_to_rank0(counts, idx, fs, group):
    """The multi-rank path's one exchange: every rank's detections (template
    index and detection time of each peak of its last step) as the 280-byte
    wire records of mflib_gb300.mpi, gathered on rank 0 over a host (gloo)
    group for association there.  Returns the number of detections rank 0
    received, None on the other ranks."""
    from mflib_gb300 import NetworkStationPhase, mpi
    from mflib_gb300.detector import Detection
    nsp = NetworkStationPhase()
    dets, o = [], 0
    for t, c in enumerate(np.asarray(counts).tolist()):
        for k in np.asarray(idx[o:o + c]).tolist():
            d = Detection()
            d.set_template_identifier((nsp, t))
            d.set_detection_time(k / fs)
            dets.append(d)
        o += c
    got = mpi.gather_detections(dets, dst=0, group=group)
    return None if got is None else len(got)


def measured_peak(key="hbm_gbs"):
    """Measured peak of the GB300s (HBM GB/s or dense BF16 TFLOP/s),
    else the fallback figure of an earlier GB300 measurement."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d[key]), "measured"
    except (OSError, KeyError, ValueError):
        return (6800.0 if key == "hbm_gbs" else 1900.0), "fallback"


def profile_traffic(name="xcorr_fp32_24ch_8.64M_traffic.txt"):
    """DRAM bytes per launch of the correlator from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_full_launch"):
                return float(line.split("=")[1])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
def cpu_baseline(w, minutes=None, threads=None):
    """The reference algorithm (oracle restatement, FP32, MULTI_CHANNEL layout:
    one signal copy per template) on a bounded sample: the first `minutes`
    of every channel for all 192 templates."""
    from oracle.orc import Oracle
    o = Oracle()
    threads = threads or os.cpu_count() or 1
    minutes = minutes if minutes is not None else float(os.environ.get("MFGPU_CPU_MINUTES", "180"))
    n = int(minutes * 60 * FS)
    sigs = [w["signals"][c, :n] for c in w["tchan"]]
    t0 = time.perf_counter()
    o.matched_filter(w["templates"], sigs, multi=True, dtype=np.float32, threads=threads)
    dt = time.perf_counter() - t0
    lags = sum(n - tp.size + 1 for tp in w["templates"])
    return {"value": lags / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "%d templates x first %.1f min of each channel (%d lags), reference overlap-add "
                      "algorithm restated in C, FFT by the oracle's radix-2 transform" % (
                          len(w["templates"]), minutes, lags),
            "seconds": dt}


def cpu_baseline_uneven(w, channels=8, minutes=None, threads=None, dtype=np.float32):
    """The reference algorithm (oracle restatement, FP32 or dtype) on a bounded sample
    of the uneven bank: for each of the first `channels` channels, its
    templates against its first `minutes` of samples in SINGLE_CHANNEL mode
    (a MULTI_CHANNEL instance of the whole bank would hold one signal copy
    per template, 3 x 2,000 x 8.64 M floats, beyond the host's memory)."""
    from oracle.orc import Oracle
    o = Oracle()
    threads = threads or os.cpu_count() or 1
    minutes = minutes if minutes is not None else float(os.environ.get("MFGPU_CPU_MINUTES", "180"))
    # at least four times the longest template (the reference sizes its
    # transforms from the signal length and rejects shorter signals)
    n = min(max(int(minutes * 60 * FS), 4 * int(max(w["lens"]))), w["n"])
    minutes = n / (60 * FS)
    lags, dt, nt = 0, 0.0, 0
    for c in range(channels):
        tps = [w["templates"][t] for t in np.nonzero(w["tchan"] == c)[0]]
        if not tps:
            continue
        x = w["signals"][c, :n]
        t0 = time.perf_counter()
        o.matched_filter(tps, [x], multi=False, dtype=dtype, threads=threads)
        dt += time.perf_counter() - t0
        lags += sum(n - tp.size + 1 for tp in tps)
        nt += len(tps)
    return {"value": lags / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "channels 0-%d (%d templates of the bank) x first %.0f min, SINGLE_CHANNEL mode per channel "
                      "(%d template-lags, %s); reference overlap-add algorithm restated in C, FFT by the "
                      "oracle's radix-2 transform" % (channels - 1, nt, minutes, lags, np.dtype(dtype).name),
            "seconds": dt}


def run_reference(args, rank):
    """The reference arm: the reference's algorithm (the oracle's C
    restatement) on the host cores, each step a bounded sample of the same
    workload as the default line (or of the 24-channel day with --day24)."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    if args.day24:
        w = make_workload(n_samples=min(args.samples, int(180 * 60 * FS)))
        base = lambda quick: cpu_baseline(w, minutes=1.0 if quick else None, threads=cores)
        workload = "24ch x 8.64M f32, 192 templates x 500, peaks 0.5/250, dbscan 50/3"
    else:
        w = make_uneven_workload(n_samples=min(args.samples, int(180 * 60 * FS)), rows=8)
        base = lambda quick: cpu_baseline_uneven(w, channels=1 if quick else 8, minutes=10.0 if quick else None,
                                                 threads=cores)
        workload = ("uneven bank: 2,000 templates of 200-3,000 samples on 96 channels x %d samples, peaks %.1f/%d"
                    % (args.samples, UNEVEN_THR, UNEVEN_SEP))
    for _ in range(args.warmup):
        base(True)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(base(False))
    el = time.perf_counter() - t0
    v = float(np.mean([x["value"] for x in vals]))
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic seeded seismograms (band-passed noise + injected templates)",
            "config": {"workload": workload, "sample_per_step": vals[0]["sample"]},
            "cpu_baseline": {k: vals[0][k] for k in ("kind", "cores", "sample")} | {"value": v, "unit": METRIC},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serving(args, rates=None, requests=None):
    """Serving loop: Poisson arrivals of detection requests (windows of
    60-600 s on 1-64 channels with 0-5 injected events) against 4 resident
    banks of 100 / 500 / 2,000 / 5,000 templates of 200-3,000 samples, under a
    120 GB device-memory budget; p50/p99 latency and template-lag
    correlations/s per arrival rate, next to the same requests served one at
    a time; then, at the first rate, windows of the stations' data read from
    a device ring (SignalRing) against the same windows uploaded."""
    from scipy.signal import butter, sosfilt
    from scipy.signal.windows import hann
    from mflib_gb300 import SignalRing
    from mflib_gb300.serving import DetectionRequest, GpuExecutor, Server, TemplateBank, latency_stats

    rng = np.random.default_rng(400)
    banks = []
    for name, nt in (("bank100", 100), ("bank500", 500), ("bank2000", 2000), ("bank5000", 5000)):
        tps = []
        for L in rng.integers(200, 3001, nt):
            lo = rng.uniform(1.0, 7.0)
            hi = rng.uniform(lo + 2.0, 15.0)
            sos = butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos")
            tps.append(sosfilt(sos, rng.standard_normal(int(L))) * hann(int(L)))
        banks.append(TemplateBank(name, tps))
    pool_n = 240_000
    pool = np.stack([bandpass_noise(np.random.default_rng(4000 + c), pool_n, 1.0, 10.0) for c in range(64)])
    rms = float(np.sqrt(np.mean(pool[:, :100_000].astype(np.float64) ** 2)))

    def make_requests(count, seed):
        r = np.random.default_rng(seed)
        out = []
        for _ in range(count):
            bank = banks[int(r.integers(len(banks)))]
            n = int(r.integers(6_000, 60_001))
            c = int(r.integers(1, 65))
            o = int(r.integers(0, pool_n - n))
            ch = r.choice(64, c, replace=False)
            x = pool[ch, o:o + n].copy()
            for _ in range(int(r.integers(0, 6))):
                t = int(r.integers(len(bank)))
                tp = bank.templates[t]
                if tp.size >= n:
                    continue
                at = int(r.integers(0, n - tp.size))
                amp = r.uniform(0.5, 2.0) * rms / np.sqrt(np.mean(tp ** 2))
                x[bank.slots[t] % c, at:at + tp.size] += (amp * tp).astype(np.float32)
            out.append((bank.name, x))
        return out

    ex = GpuExecutor(threshold=args.serving_threshold, min_distance=250)
    srv = Server(banks, ex, memory_budget=120e9, slots=args.serving_slots)
    t0 = time.perf_counter()
    srv.warm([(b.name, n) for b in banks for n in srv.buckets], per_key=args.serving_slots)
    warm_s = time.perf_counter() - t0
    srv.start()
    for b, x in make_requests(4 * args.serving_slots, 1):  # untimed warm-up traffic
        srv.submit(DetectionRequest(b, x))
    while len(srv.served) < 4 * args.serving_slots:
        time.sleep(0.01)

    out_rates = []
    for k, lam in enumerate(rates if rates is not None else args.rates):
        reqs = make_requests(requests if requests is not None else args.requests, 10 + k)
        # rate 0: every request queued at once (saturation)
        arr = (np.cumsum(np.random.default_rng(500 + k).exponential(1.0 / lam, len(reqs))) if lam > 0
               else np.zeros(len(reqs)))
        objs = [DetectionRequest(b, x) for b, x in reqs]
        base = time.perf_counter() + 0.05
        for r, a in zip(objs, arr):
            d = base + a - time.perf_counter()
            if d > 0:
                time.sleep(d)
            r.t_arrival = base + a
            srv.submit(r)
        for r in objs:
            r.wait(600)
        st = latency_stats(objs)
        # the same requests one at a time (no overlap), back to back
        solo = [DetectionRequest(b, x) for b, x in reqs]
        t1 = time.perf_counter()
        for r in solo:
            r.t_arrival = time.perf_counter()
            srv.run_one(r)
        el = time.perf_counter() - t1
        so = latency_stats(solo)
        out_rates.append({"rate_req_s": lam if lam > 0 else "all at once", "requests": st["requests"], "p50_ms": 1e3 * st["p50_s"],
                      "p99_ms": 1e3 * st["p99_s"], "mean_ms": 1e3 * st["mean_s"], "throughput": st["throughput"],
                      "one_at_a_time": {"throughput": so["template_lags"] / el, "p50_ms": 1e3 * so["p50_s"],
                                        "p99_ms": 1e3 * so["p99_s"]}})
    # ring arm: the pool as the stations' recent samples in a device ring
    # (appended in chunks), requests naming windows of it, against the same
    # windows (no injected events) uploaded from the host
    ring = SignalRing(64, pool_n)
    for a in range(0, pool_n, 20_000):
        ring.append(pool[:, a:a + 20_000])
    lam = (rates if rates is not None else args.rates)[0] or 100.0
    rr = np.random.default_rng(900)
    specs = []
    for _ in range(requests if requests is not None else args.requests):
        n = int(rr.integers(6_000, 60_001))
        specs.append((banks[int(rr.integers(len(banks)))].name, rr.choice(64, int(rr.integers(1, 65)), replace=False),
                      int(rr.integers(0, pool_n - n)), n))
    ring_arm = {"rate_req_s": lam}
    for mode in ("ring", "upload"):
        objs = [DetectionRequest(b, ring=ring, channels=ch, n=n, end=o + n) if mode == "ring"
                else DetectionRequest(b, pool[ch, o:o + n]) for b, ch, o, n in specs]
        arr = np.cumsum(np.random.default_rng(901).exponential(1.0 / lam, len(objs)))
        base = time.perf_counter() + 0.05
        for r, a in zip(objs, arr):
            d = base + a - time.perf_counter()
            if d > 0:
                time.sleep(d)
            r.t_arrival = base + a
            srv.submit(r)
        for r in objs:
            r.wait(600)
        st = latency_stats(objs)
        ring_arm[mode] = {"p50_ms": 1e3 * st["p50_s"], "p99_ms": 1e3 * st["p99_s"], "mean_ms": 1e3 * st["mean_s"],
                          "h2d_bytes_per_request": 0 if mode == "ring" else
                          float(np.mean([4 * len(ch) * n for _, ch, _, n in specs]))}
    ring.close()
    srv.close()
    line = {"metric": "served detection requests: p50/p99 latency and template-lag correlations/s",
            "unit": "template-lag correlations/s; ms", "n_gpus": 1, "dtype": "f32",
            "data": "synthetic band-passed noise windows with injected template copies",
            "config": {"workload": "Poisson arrivals, windows 6,000-60,000 samples on 1-64 channels, banks of "
                                   "100/500/2,000/5,000 templates of 200-3,000 samples, 120 GB budget",
                       "slots": args.serving_slots, "buckets": list(srv.buckets),
                       "threshold": args.serving_threshold, "min_distance": 250},
            "rates": out_rates, "ring_windows": ring_arm, "objects_created": srv.created, "evicted": srv.evicted,
            "peak_device_bytes": srv.peak_held, "warm_s": warm_s}
    return line


def run_detector(args):
    """Single-channel detector timing: one 24 h channel (8.64 M samples of
    band-passed noise with injected copies) against 192 templates of 500
    samples; a step is Detector.detect (reduction of the 192 traces to their
    per-lag maximum and argmax, PeakFinder at rho > 0.5 with separation 250,
    quadratic refinement, amplitudes) on the traces of one apply, timed with
    CUDA events on the library's stream."""
    import torch
    import mflib_gb300 as mf
    w = make_workload(n_samples=args.samples, n_stations=1, n_events=64)
    x = w["signals"][0]
    p = mf.SingleChannel.MatchedFilterParameters()
    for tp in w["templates"][:192]:
        wt = mf.WaveformTemplate()
        wt.set_signal(tp)
        wt.set_sampling_rate(FS)
        p.add_template(wt)
    p.set_signal_size(x.size)
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p)
    f.set_signal(x)
    f.apply()
    prm = mf.SingleChannel.DetectorParameters()
    prm.set_detection_threshold(0.5)
    prm.set_minimum_detection_spacing(250)
    prm.set_matched_filtered_signal_detector_policy(mf.MatchedFilteredSignalDetectorPolicy.reduce)
    det = mf.SingleChannel.Detector()
    det.initialize(prm)
    import ctypes as C
    from mflib_gb300 import _lib
    dp = _lib.MfgpuDetectParams()
    dp.threshold, dp.min_distance, dp.absolute_maximum, dp.single = 0.5, 250, 0, 0
    dp.interpolation, dp.lanczos_alpha, dp.lanczos_points, dp.sampling_rate, dp.amplitudes = 1, 51, 100, FS, 1
    nd = C.c_int()

    def abi_detect():
        _lib.call("mfgpu_mf_detect", f._h, C.byref(dp), C.byref(nd))

    stream = torch.cuda.ExternalStream(f.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        f.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            fn()
        ev1.record(stream)
        f.synchronize()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / args.steps

    ms = timed(abi_detect)  # the C ABI call: device work, detections copied to host structs
    py_ms = timed(lambda: det.detect(f))  # plus the Python Detection objects
    nt = len(w["templates"][:192])
    ln = f.get_filtered_signal_length()
    alg = 4.0 * nt * ln + 8.0 * ln  # traces read, reduced trace and argmax written
    peak, kind = measured_peak()
    line = {"metric": "detector step through the C ABI (reduce + peaks + refinement + amplitudes)", "value": ms,
            "unit": "ms",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
            "config": {"workload": "1 channel x %d samples, %d templates x 500, REDUCED, quadratic" % (x.size, nt)},
            "detections": det.get_number_of_detections(), "python_api_ms": py_ms,
            "roofline_bound_ms": alg / (peak * 1e9) * 1e3, "algorithmic_bytes": alg, "peak_gbs": peak,
            "peak_source": kind}
    print(json.dumps(line), flush=True)


def run_stress(args):
    """Precision stress: 512 templates of 1,000 samples against 16 channels of
    4.32 M samples (all pairs: each channel against every template, one
    single-channel object reused per channel).  Signals: a DC offset
    U(1e3, 1e5) plus band-passed noise under a piecewise-constant envelope
    (segments of 10-60 min, levels log-uniform in [1e-3, 1e3]) with injected
    template copies at 0.2-1 x the local RMS.  For the FP32 FFT correlator
    and the split-precision tensor-core correlator (FP16 hi+lo operands):
    template-lags/s of the applies (CUDA events) and max |drho| against the
    FP64 oracle on sampled lags of 8 templates per channel, over all sampled
    lags and over lags whose window and FFT blocks stay inside one envelope
    segment; for the tensor-core correlator, with FP16 and with BF16 hi+lo
    operands, also the raw error (the accuracy fix-up skipped)."""
    import torch
    import mflib_gb300 as mf
    from scipy.signal import butter, sosfilt
    from scipy.signal.windows import hann
    from oracle.orc import Oracle
    rng = np.random.default_rng(300)
    nt, nch, L, n = 512, 16, 1000, args.samples if args.samples != N_SAMPLES else 4_320_000
    tps = []
    for _ in range(nt):
        lo = rng.uniform(1.0, 7.0)
        hi = rng.uniform(lo + 2.0, 15.0)
        tps.append(sosfilt(butter(4, [lo, hi], btype="bandpass", fs=FS, output="sos"), rng.standard_normal(L))
                   * hann(L))
    sos = butter(4, [1.0, 10.0], btype="bandpass", fs=FS, output="sos")
    chans, edges_all = [], []
    for c in range(nch):
        r = np.random.default_rng(3000 + c)
        noise = sosfilt(sos, r.standard_normal(n))
        env = np.empty(n)
        edges = [0]
        while edges[-1] < n:
            edges.append(min(n, edges[-1] + int(r.integers(60_000, 360_001))))
        for a, b in zip(edges[:-1], edges[1:]):
            env[a:b] = 10.0 ** r.uniform(-3, 3)
        x = env * noise
        for o in r.integers(0, n - L, 40):
            t = int(r.integers(nt))
            lvl = env[o] * np.std(noise[o:o + L])
            x[o:o + L] += r.uniform(0.2, 1.0) * lvl * tps[t] / np.std(tps[t])
        chans.append((x + r.uniform(1e3, 1e5)).astype(np.float32))
        edges_all.append(np.array(edges))
    o = Oracle()
    out = {}
    def errors(f, c, xs, e):
        lr = np.random.default_rng(7 + c)
        wa, wf = 0.0, 0.0
        for t in lr.choice(nt, 8, replace=False):
            lags = np.sort(lr.choice(n - L + 1, 500, replace=False))
            truth = o.pearson_naive(tps[t], xs, lags)
            got = f.get_matched_filtered_signal(int(t)).astype(np.float64)[lags]
            err = np.abs(got - truth)
            wa = max(wa, float(err.max()))
            seg = np.searchsorted(e, lags, side="right") - 1
            flat = (lags - 8192 >= e[seg]) & (lags + L + 8192 <= e[seg + 1])
            if flat.any():
                wf = max(wf, float(err[flat].max()))
        return wa, wf

    for name, variant, bf16 in (("fft", 3, False), ("tensor", 4, False), ("tensor_bf16", 4, True)):
        p = mf.SingleChannel.MatchedFilterParameters()
        for tp in tps:
            wt = mf.WaveformTemplate()
            wt.set_signal(tp)
            wt.set_sampling_rate(FS)
            p.add_template(wt)
        p.set_signal_size(n)
        f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
        f.initialize(p, correlator_variant=variant, tc_bf16=bf16)
        stream = torch.cuda.ExternalStream(f.stream_handle())
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total_ms, worst_all, worst_flat, fixups, raw_all, raw_flat = 0.0, 0.0, 0.0, 0, 0.0, 0.0
        for c in range(nch):
            f.set_signal(chans[c])
            f.apply()  # warm
            f.synchronize()
            ev0.record(stream)
            f.apply()
            ev1.record(stream)
            f.synchronize()
            torch.cuda.synchronize()
            total_ms += ev0.elapsed_time(ev1)
            fixups += f.get_fixup_runs()
            xs = chans[c].astype(np.float64)
            wa, wf = errors(f, c, xs, edges_all[c])
            worst_all, worst_flat = max(worst_all, wa), max(worst_flat, wf)
            if variant == 4:
                f.test_skip_fixup(True)
                f.apply()
                wa, wf = errors(f, c, xs, edges_all[c])
                raw_all, raw_flat = max(raw_all, wa), max(raw_flat, wf)
                f.test_skip_fixup(False)
        lags_total = float(nch) * nt * (n - L + 1)
        res = {"template_lags_per_s": lags_total / (total_ms * 1e-3), "apply_ms_per_channel": total_ms / nch,
               "max_abs_drho_all": worst_all, "max_abs_drho_away_from_envelope_steps": worst_flat,
               "fixup_runs": fixups, "runs": nch * ((n - L + 1 + 31) // 32),
               "correlator": f.get_plan()["correlator"], "operands": "bf16 hi+lo" if bf16 else
               ("fp16 hi+lo" if variant == 4 else "fp32")}
        if variant == 4:
            res["raw_max_abs_drho_all"] = raw_all
            res["raw_max_abs_drho_away_from_envelope_steps"] = raw_flat
        out[name] = res
        f.clear()
    line = {"metric": "precision stress: template-lag correlations/s and max |drho| vs FP64 oracle", "n_gpus": 1,
            "dtype": "f32", "config": {"workload": "512 templates x 1,000 against 16 channels x %d samples, all pairs,"
                                                   " DC 1e3..1e5, envelope 1e-3..1e3" % n},
            "paths": out, "tensor_over_fft": out["tensor"]["template_lags_per_s"] / out["fft"]["template_lags_per_s"]}
    return line


class Ctx:
    """Ranks of the job (torchrun: one per GPU) and the job-wide helpers."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.gloo = None  # host-tensor group for the gather of detections

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, v):
        return max_over_ranks(v, self.dist, "cuda")


def run_uneven_day(args, ctx):
    """The headline: the uneven bank over a whole day.  A step is apply
    (CUDA-graph replay after the first) plus the batched peak finder with
    candidates gathered in the correlator (rho > 0.7, separation 250) and the
    peaks copied to the host.  value: K steps with the channels resident,
    CUDA events on the library's stream; e2e: the same K steps with every
    step's channels staged from pinned host memory under the previous step.
    --fp64 runs the same bank in double precision (the reference's default
    type)."""
    import torch
    import mflib_gb300 as mf
    fp64 = bool(getattr(args, "fp64", False))
    npt, tdt, es = (np.float64, torch.float64, 8) if fp64 else (np.float32, torch.float32, 4)
    w = make_uneven_workload(n_samples=args.samples)
    n, nch, lens = w["n"], w["nch"], w["lens"]
    nt = len(w["templates"])
    p = mf.MultiChannel.MatchedFilterParameters()
    for tp in w["templates"]:
        wt = mf.WaveformTemplate()
        wt.set_signal(tp)
        wt.set_sampling_rate(FS)
        p.add_template(wt)
    p.set_signal_size(n)
    f = mf.MultiChannel.MatchedFilter(dtype=npt)
    f.initialize(p, template_channels=[int(c) for c in w["tchan"]], n_channels=nch,
                 correlator_variant=args.correlator_variant, length_buckets=args.length_buckets)
    pinned = torch.empty((nch, n), dtype=tdt, pin_memory=True)
    pinned.numpy()[:] = w["signals"]
    host = pinned.numpy()
    f.set_channel_signals(host)
    f.set_peak_threshold(UNEVEN_THR)
    tune = None
    if args.autotune:
        # measured per-bucket plan choice (1-3 buckets, FFT length and
        # organisation per bucket) before anything is timed
        t0 = time.perf_counter()
        res = f.autotune(w["signals"], repeats=1, max_buckets=3)
        ok = [t for t in res["trials"] if t["apply_ms"] is not None]
        tune = {"seconds": time.perf_counter() - t0, "trials": len(ok),
                "model_apply_ms": ok[0]["apply_ms"], "tuned_apply_ms": res["apply_ms"],
                "chosen": res["plan"]["bucket_plans"]}
        f.set_channel_signals(host)
    f.set_graph(True)  # the day-long apply replayed as a CUDA graph after its first run
    lags = float(sum(n - int(L) + 1 for L in lens))

    def run_steps(k, stage=False):
        xms, out = [], None
        if stage:
            f.stage_channel_signals(host)
        for i in range(k):
            f.apply()
            if stage and i + 1 < k:
                f.stage_channel_signals(host)
            f.find_peaks(UNEVEN_THR, UNEVEN_SEP)
            out = f.get_all_peaks()
            xms.append(f.last_timings()["xcorr_ms"])
        return out, xms

    run_steps(args.warmup)
    f.synchronize()
    stream = torch.cuda.ExternalStream(f.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = f.launch_count()
    clocks = ClockSampler(ctx.local)
    clocks.start()
    ctx.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    (counts, idx), xms = run_steps(args.steps)
    ev1.record(stream)
    f.synchronize()
    torch.cuda.synchronize()
    ctx.barrier()
    el = ctx.max(1e-3 * ev0.elapsed_time(ev1))
    clk = clocks.stop()
    launches = f.launch_count() - launches0

    # end to end through the C ABI: every step's channels copied from pinned
    # host memory (staged under the previous step), peaks copied back; the
    # staged applies replay their own pair of CUDA graphs, captured in an
    # untimed warm-up
    run_steps(2, stage=True)
    f.synchronize()
    ctx.barrier()
    t0 = time.perf_counter()
    (c2, i2), _ = run_steps(args.steps, stage=True)
    e2e_el = ctx.max(time.perf_counter() - t0)
    h2d = nch * n * es
    d2h = int(4 * (c2.size + i2.size))
    # the host link's rate for one step's upload alone (the e2e steps overlap
    # it with the previous apply, so it bounds them when it is the longer)
    f.synchronize()
    t1 = time.perf_counter()
    f.stage_channel_signals(host)
    f.synchronize()
    h2d_gbs = h2d / (time.perf_counter() - t1) / 1e9

    plan = f.get_plan()
    P = plan["fft_length"] // 2
    x_ms = float(np.mean(xms))
    alg = es * lags + es * nch * n + 2.0 * es * (P + 1) * nt
    peak, kind = measured_peak()
    traffic = profile_traffic("xcorr_fp32_uneven_traffic.txt")
    default = (n == N_SAMPLES and args.correlator_variant == 0 and args.length_buckets == 0 and not args.autotune
               and not fp64)
    roof = {"bound": "hbm", "achieved": alg / (x_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": alg / (x_ms * 1e-3) / 1e9 / peak, "traffic": traffic if default else None,
            "kernel": "xcorr_kernel<%s,%d,per-template normalisation>" % ("double" if fp64 else "float", P),
            "kernel_ms": x_ms,
            "algorithmic_bytes": alg, "peak_source": kind}
    line = {"metric": METRIC, "value": ctx.world * lags / (el / args.steps), "unit": METRIC, "n_gpus": ctx.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if fp64 else "f32",
            "data": "synthetic seeded seismograms (band-passed noise, Hann-tapered band-passed templates)",
            "config": {"workload": "uneven bank: 2,000 templates of 200-3,000 samples on 96 channels x %d samples, "
                                   "peaks %.1f/%d" % (n, UNEVEN_THR, UNEVEN_SEP),
                       "template_lags": lags, "fft_length": plan["fft_length"], "buckets": plan["buckets"],
                       "lags_per_block": plan["lags_per_block"], "correlator": plan["correlator"],
                       "graph": True,
                       "l2": "inputs (%.2f GB) and outputs (%.0f GB) exceed the 129 MB L2; no flush needed"
                             % (4e-9 * nch * n, 4e-9 * lags)},
            "e2e": {"value": ctx.world * lags / (e2e_el / args.steps), "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_el / args.steps,
                    "h2d_gbs_one_upload": h2d_gbs,
                    "api": "stage_channel_signals (async H2D of step i+1 under step i), apply, find_peaks, "
                           "get_all_peaks"},
            "roofline": roof, "gpu_launches": int(launches), "clocks": clk, "detections": int(idx.size),
            "graph_replays": f.graph_launches()}
    if ctx.world > 1:  # after the timed regions; every rank takes part
        line["gathered_detections"] = gather_detections_to_rank0(counts, idx, FS, ctx.gloo)
    # The split-precision tensor-core form on this bank, by arithmetic: per
    # template-lag it executes 3 products (hi*hi, hi*lo, lo*hi) over the
    # template's K padded to 16 (K = L + 7 for the 8 phases of a row), 2 flops
    # each; even at the measured dense BF16/FP16 peak that takes longer than
    # the FFT form's measured step.
    if tune is not None:
        line["config"]["autotune"] = tune
    if fp64:  # the split-precision form is an FP32 path
        f.clear()
        return line, w
    kp = ((lens.astype(np.int64) + 7 + 15) // 16) * 16
    tc_flops = float(np.sum(3.0 * 2.0 * kp * (n - lens + 1)))
    bf16, bf16_kind = measured_peak("bf16_tflops")
    tc_ms = tc_flops / (bf16 * 1e12) * 1e3
    line["split_precision_ceiling"] = {
        "executed_flops": tc_flops, "ms_at_tensor_peak": tc_ms, "peak_tflops": bf16, "peak_source": bf16_kind,
        "fft_ms_per_step": 1e3 * el / args.steps, "best_possible_ratio_over_fft": (1e3 * el / args.steps) / tc_ms}
    f.clear()
    return line, w


def run_day24(args, ctx, steps=None, warmup=None, cpu=True):
    """The 24-channel day: apply + peaks + DBSCAN association per step
    (software-pipelined: step i's association beside step i + 1's apply)."""
    import torch
    import mflib_gb300 as mf
    steps = steps or args.steps
    warmup = warmup or args.warmup
    samples = args.samples if args.day24 else N_SAMPLES
    w = make_workload(n_samples=samples, seed=10 + 97 * ctx.rank, n_events=args.events,
                      template_length=args.template_length)
    f = build_filter(mf, w, correlator_variant=args.correlator_variant)
    # the correlator gathers the peak candidates as it stores the traces
    f.set_peak_threshold(PEAK_THR)
    db = mf.DBSCAN()
    db.initialize(DB_EPS, DB_MINPTS)
    nt = len(w["templates"])
    n = w["n"]
    lags_per_step = sum(n - tp.size + 1 for tp in w["templates"])

    # pinned host copies of the channel samples for the end-to-end leg
    pinned = torch.empty((w["nch"], n), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = w["signals"]
    host = pinned.numpy()

    def load_all():
        f.set_channel_signals(host)

    def step():
        f.apply()
        f.find_peaks(PEAK_THR, PEAK_SEP)
        counts, idx = f.get_all_peaks()
        labels, ncl = associate(db, counts, idx, w)
        return counts, idx, labels, ncl

    def run_steps(k, stage=False):
        """k steps, software-pipelined: the association of step i (host
        grouping + DBSCAN on the clustering object's own stream) runs while
        step i + 1's apply runs on the matched filter's stream; every step's
        association has finished when this returns.  stage: each step's
        channels are uploaded asynchronously under the previous step."""
        pending, xms = None, []
        if stage:
            f.stage_channel_signals(host)
        for i in range(k):
            f.apply()
            if stage and i + 1 < k:
                f.stage_channel_signals(host)
            if pending is not None:
                associate(db, *pending, w)
            f.find_peaks(PEAK_THR, PEAK_SEP)
            pending = f.get_all_peaks()
            xms.append(f.last_timings()["xcorr_ms"])
        return pending + tuple(associate(db, *pending, w)), xms

    load_all()
    for _ in range(warmup):
        step()
    f.synchronize()

    # ---- device-resident timing (value): CUDA events on the library's
    #      stream, which carries every launch and copy of the matched filter;
    #      the last step's association (DBSCAN on the clustering object's
    #      stream) has returned to the host before the closing event
    stream = torch.cuda.ExternalStream(f.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = f.launch_count() + db.launch_count()
    clocks = ClockSampler(ctx.local)
    clocks.start()
    ctx.barrier()
    torch.cuda.synchronize()
    f.synchronize()
    ev0.record(stream)
    out, xcorr_ms = run_steps(steps)
    ev1.record(stream)
    f.synchronize()
    torch.cuda.synchronize()
    ctx.barrier()
    el = 1e-3 * ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches = f.launch_count() + db.launch_count() - launches0
    el = ctx.max(el)
    counts, idx, labels, ncl = out
    ms_step = 1e3 * el / steps

    # ---- end to end through the C ABI with host buffers.  Serial: copy all
    #      channels (one batched call, returns when copied), then the step.
    #      Pipelined (the headline): each step's channels are staged
    #      asynchronously while the previous step's correlation and peak
    #      finding run; every step still copies its 830 MB from pinned memory.
    def timed(fn):
        ctx.barrier()
        t0 = time.perf_counter()
        r = fn()
        return ctx.max(time.perf_counter() - t0), r

    def serial():
        r = None
        for _ in range(steps):
            load_all()
            r = step()
        return r

    serial_el, _ = timed(serial)
    e2e_el, (counts, idx, labels, ncl) = timed(lambda: run_steps(steps, stage=True)[0])
    last_pipelined = f.last_timings()  # correlator and apply of the last pipelined step
    h2d = w["nch"] * n * 4
    d2h = int(4 * (counts.size + idx.size + labels.size + ncl.size))

    # ---- roofline of the correlator
    x_ms = float(np.mean(xcorr_ms))
    plan = f.get_plan()
    P = plan["fft_length"] // 2
    if plan["correlator"] == 4:
        # tensor-core correlator: 2 L algorithmic flops per template-lag (one
        # multiply-add per template sample; the hi/lo split executes 3
        # products over the padded K, reported as executed_flops)
        alg_flops = 2.0 * args.template_length * lags_per_step
        peak, peak_kind = measured_peak("bf16_tflops")
        achieved = alg_flops / (x_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None, "kernel": "tc_xcorr_kernel",
                "kernel_ms": x_ms, "algorithmic_flops": alg_flops,
                "executed_flops": 6.0 * plan["tc_k"] * lags_per_step, "peak_source": peak_kind}
    else:
        alg_bytes = 4.0 * lags_per_step + 4.0 * w["nch"] * n + 8.0 * (P + 1) * nt
        peak, peak_kind = measured_peak()
        achieved = alg_bytes / (x_ms * 1e-3) / 1e9
        default = n == N_SAMPLES and args.template_length == TEMPLATE_LEN and args.events == N_EVENTS
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profile_traffic() if default else None,
                "kernel": "xcorr_kernel<float,%d,shared_den>" % P,
                "kernel_ms": x_ms, "algorithmic_bytes": alg_bytes, "peak_source": peak_kind}

    line = {"metric": METRIC, "value": ctx.world * lags_per_step / (el / steps), "unit": METRIC,
            "n_gpus": ctx.world, "steps": steps, "warmup": warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic seeded seismograms (band-passed noise + injected templates)",
            "config": {"workload": "%dch x %.2fM f32, %d templates x %d, peaks 0.5/250, dbscan 50/3"
                                   % (w["nch"], n / 1e6, nt, args.template_length),
                       "channels": w["nch"], "samples_per_channel": n, "templates": nt,
                       "template_length": args.template_length, "correlator": plan["correlator"],
                       "fft_length": plan["fft_length"],
                       "lags_per_block": plan["lags_per_block"],
                       "l2": "inputs (%.0f MB) and outputs (%.2f GB) exceed the 129 MB L2; no flush needed"
                             % (4e-6 * w["nch"] * n, 4e-9 * lags_per_step)},
            "e2e": {"value": ctx.world * lags_per_step / (e2e_el / steps), "unit": METRIC,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * e2e_el / steps,
                    "serial_value": ctx.world * lags_per_step / (serial_el / steps),
                    "last_step_xcorr_ms": last_pipelined["xcorr_ms"], "last_step_apply_ms": last_pipelined["apply_ms"],
                    "api": "stage_channel_signals (async H2D of step i+1 under step i), apply, find_peaks, "
                           "get_all_peaks, DBSCAN association (step i's beside step i+1's apply); "
                           "serial_value: set_channel_signals then the step, nothing overlapped"},
            "roofline": roof, "gpu_launches": int(launches), "clocks": clk,
            "detections": int(idx.size), "events_found": int(np.sum(ncl)),
            "events_injected": int(w["origins"].size)}
    if ctx.world > 1:  # after the timed regions; every rank takes part
        line["gathered_detections"] = gather_detections_to_rank0(counts, idx, FS, ctx.gloo)
    if cpu and ctx.rank == 0 and ctx.world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(w).items() if k != "seconds"}
    f.clear()
    return line


def _extra(fn):
    """An extra workload of the default run; its failure is recorded, not raised."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 -- the headline line must still print
        return {"error": "%s: %s" % (type(e).__name__, e)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 12 steps of the default uneven day time about 1.1 s (the clock sampler sees the load)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=N_SAMPLES, help="samples per channel (default 24 h)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default run: skip the 24-channel day, precision stress and serving extras")
    ap.add_argument("--day24", action="store_true",
                    help="the 24-channel day (peaks + DBSCAN association) as the headline line")
    ap.add_argument("--correlator-variant", type=int, default=0,
                    help="0 planner's choice, 1-3 FFT organisations, 4 tensor cores")
    ap.add_argument("--template-length", type=int, default=TEMPLATE_LEN,
                    help="24-channel day: samples per template (default %d)" % TEMPLATE_LEN)
    ap.add_argument("--events", type=int, default=N_EVENTS,
                    help="24-channel day: events, i.e. templates per channel (default %d)" % N_EVENTS)
    ap.add_argument("--serving", action="store_true", help="run the request loop instead of the day-long step")
    ap.add_argument("--autotune", action="store_true",
                    help="uneven bank: measured per-bucket plan choice before timing")
    ap.add_argument("--uneven", action="store_true", help="the uneven bank alone (the default headline, no extras)")
    ap.add_argument("--fp64", action="store_true", help="uneven bank: double precision (the reference's default type)")
    ap.add_argument("--detector", action="store_true", help="time the single-channel detector")
    ap.add_argument("--stress", action="store_true", help="precision stress: FFT and tensor-core paths")
    ap.add_argument("--length-buckets", type=int, default=0,
                    help="length buckets of a mixed-length bank (0 planner's choice, 1 one plan)")
    ap.add_argument("--rates", type=float, nargs="+", default=[50, 100, 200, 500, 0],
                    help="Poisson arrival rates in requests/s (0: all requests queued at once)")
    ap.add_argument("--requests", type=int, default=200, help="requests per arrival rate (serving)")
    ap.add_argument("--serving-slots", type=int, default=4)
    ap.add_argument("--serving-threshold", type=float, default=0.7)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.serving:
        print(json.dumps(run_serving(args)), flush=True)
        return
    if args.detector:
        run_detector(args)
        return
    if args.stress:
        print(json.dumps(run_stress(args)), flush=True)
        return

    ctx = Ctx()
    if ctx.world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if args.impl == "ours":
            torch.cuda.set_device(ctx.local)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        ctx.dist = dist
        if args.impl == "ours":
            ctx.gloo = dist.new_group(backend="gloo")

    if args.impl == "reference":
        run_reference(args, ctx.rank)
        if ctx.dist is not None:
            ctx.dist.destroy_process_group()
        return

    import mflib_gb300  # noqa: F401
    if ctx.world > 1:
        import torch
        torch.cuda.set_device(ctx.local)
    if args.day24:
        line = run_day24(args, ctx)
    else:
        # every rank runs the whole uneven day on its own GPU (weak scaling)
        line, w = run_uneven_day(args, ctx)
        if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu_baseline:
            # a short warm-up, then the mean of three timed samples (a single
            # cold sample had read well below the reference arm's steady mean)
            cdt = np.float64 if args.fp64 else np.float32
            cpu_baseline_uneven(w, channels=1, minutes=10.0, dtype=cdt)
            reps = [cpu_baseline_uneven(w, dtype=cdt) for _ in range(3)]
            cb = {k: v for k, v in reps[0].items() if k != "seconds"}
            cb["value"] = float(np.mean([r["value"] for r in reps]))
            cb["repeats"] = 3
            line["cpu_baseline"] = cb
        del w
        if ctx.rank == 0 and ctx.world == 1 and not args.no_extras and not args.uneven:
            line["multichannel_day"] = _extra(lambda: run_day24(args, ctx, steps=20, warmup=3, cpu=False))
            line["precision_stress"] = _extra(lambda: run_stress(args))
            line["serving"] = _extra(lambda: run_serving(args, rates=[100], requests=100))
    if ctx.rank == 0:
        print(json.dumps(line), flush=True)
    if ctx.dist is not None:
        ctx.dist.destroy_process_group()


if __name__ == "__main__":
    main()
