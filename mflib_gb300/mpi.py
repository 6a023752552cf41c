"""mflib_gb300.mpi -- MFLib::MPI (include/mflib/mpi.hpp, src/mpi.cpp) over a
torch.distributed process group: ``broadcast`` of a WaveformTemplate,
``send`` / ``recv`` of a Detection, and the one collective of the multi-rank
path, ``gather_detections``: every rank's detections to one rank.

The process group stands in for the MPI communicator.  Every tensor here is
a host tensor, so the group must carry CPU tensors (gloo; with an NCCL
default group pass ``dist.new_group(backend="gloo")``).  Ranks are global
ranks, as torch.distributed's send and recv take them.

Wire format of a detection: ``DETECTION_RECORD``, the reference's
MPIDetection struct (src/mpi.cpp:20-51) in its natural C layout -- eight
doubles, three 64-byte strings, the uint64 template id, the int32 signal
length and ten flags, 280 bytes, little-endian -- followed by the detected
signal's samples (float32 or float64) when it has one (src/mpi.cpp:386-414).
Differences from the reference, each deliberate:

* the record travels as its 280 bytes, so the two have-amplitude flags
  arrive (the reference's datatype lists the amplitudes' offsets in their
  place, src/mpi.cpp:95-96, and its receiver reads them uninitialised);
* byte 278, padding in the reference struct, carries the detection's
  polarity as int8 (a reference sender's zeroed padding reads as unknown);
* a received detection holds exactly the sent fields: it is cleared first
  (the reference's convertDetection, src/mpi.cpp:197-244, leaves the
  receiver's other fields in place).

The channel and location code of the template identifier do not travel in a
detection record (network, station and phase do, truncated to 64 bytes, as
in src/mpi.cpp:182-193).  A broadcast template carries all five identifier
fields at full length.
"""
import numpy as np
import torch
import torch.distributed as dist

from .detector import Detection, RelativeMagnitudeType
from .waveform import NetworkStationPhase, Polarity, WaveformTemplate

__all__ = ["DETECTION_RECORD", "TEMPLATE_HEADER", "pack_detection", "unpack_detection", "pack_detections",
           "unpack_detections", "pack_template", "unpack_template", "send", "recv", "broadcast",
           "gather_detections"]

# src/mpi.cpp:20-51, field for field; numpy's aligned layout is the C layout
DETECTION_RECORD = np.dtype({
    "names": ["amplitude1", "amplitude2", "correlation_coefficient", "detection_time",
              "interpolated_detection_time", "phase_onset_time", "interpolated_phase_onset_time", "travel_time",
              "network", "station", "phase", "template_id", "signal_length",
              "have_amplitude1", "have_amplitude2", "have_correlation_coefficient", "have_detected_signal",
              "have_detection_time", "have_interpolated_detection_time", "have_phase_onset_time",
              "have_interpolated_phase_onset_time", "have_travel_time", "have_template_id", "polarity"],
    "formats": ["<f8"] * 8 + ["S64"] * 3 + ["<u8", "<i4"] + ["?"] * 10 + ["i1"],
    "offsets": [0, 8, 16, 24, 32, 40, 48, 56, 64, 128, 192, 256, 264] + list(range(268, 278)) + [278],
    "itemsize": 280,
})

# WaveformTemplate broadcast header (the scalars of src/mpi.cpp:294-384 with a
# presence flag for each optional field); the identifier's five strings
# follow as one byte payload of the listed lengths, then the FP64 samples.
TEMPLATE_HEADER = np.dtype({
    "names": ["sampling_rate", "weight", "onset", "travel", "magnitude", "template_id", "n_samples",
              "string_bytes", "polarity", "have_magnitude", "have_identifier"],
    "formats": ["<f8"] * 5 + ["<u8", "<i8", ("<i4", (5,)), "<i4", "?", "?"],
    "offsets": [0, 8, 16, 24, 32, 40, 48, 56, 76, 80, 81],
    "itemsize": 88,
})

_AMP = (RelativeMagnitudeType.gibbons_ringdal_2006, RelativeMagnitudeType.schaff_richards_2014)
_TIMES = ("detection_time", "interpolated_detection_time", "phase_onset_time", "interpolated_phase_onset_time",
          "travel_time")
_TIME_ATTRS = (("detection_time", "_t"), ("interpolated_detection_time", "_ti"), ("phase_onset_time", "_po"),
               ("interpolated_phase_onset_time", "_poi"), ("travel_time", "_tt"))


def _str64(s):
    return str(s).encode("utf-8")[:64]


def _unstr(b):
    return bytes(np.asarray(b).item()).decode("utf-8", errors="replace")


def _fill_record(r, det):
    for i, t in enumerate(_AMP):
        if det.have_amplitude_scaling_factor(t):
            r["have_amplitude%d" % (i + 1)] = True
            r["amplitude%d" % (i + 1)] = det.get_amplitude_scaling_factor(t)
    if det.have_correlation_coefficient():
        r["have_correlation_coefficient"] = True
        r["correlation_coefficient"] = det.get_correlation_coefficient()
    for f in _TIMES:
        if getattr(det, "have_" + f)():
            r["have_" + f] = True
            r[f] = getattr(det, "get_" + f)()
    if det.have_detected_signal():
        r["have_detected_signal"] = True
        r["signal_length"] = det.get_detected_signal().size
    if det.have_template_identifier():
        nsp, wid = det.get_template_identifier()
        r["have_template_id"] = True
        r["template_id"] = int(wid)
        r["network"] = _str64(nsp.get_network())
        r["station"] = _str64(nsp.get_station())
        r["phase"] = _str64(nsp.get_phase())
    r["polarity"] = int(det.get_polarity())


def pack_detection(det):
    """The detection's wire record (a zeroed DETECTION_RECORD scalar with its
    fields and flags set, src/mpi.cpp:119-195)."""
    r = np.zeros((), DETECTION_RECORD)
    _fill_record(r, det)
    return r


def pack_detections(dets, dtype=np.float64):
    """Records of a list of detections and their detected signals
    concatenated in ``dtype`` (list order, each ``signal_length`` long)."""
    dtype = _check_dtype(dtype)
    recs = np.zeros(len(dets), DETECTION_RECORD)
    sigs = []
    for i, d in enumerate(dets):
        _fill_record(recs[i], d)
        if d.have_detected_signal():
            sigs.append(d.get_detected_signal().astype(dtype))
    return recs, (np.concatenate(sigs) if sigs else np.zeros(0, dtype))


def unpack_detection(rec, signal=None, det=None):
    """Detection holding the record's fields (``det`` cleared and filled, or a
    new one); ``signal`` is the detected signal that followed the record."""
    det = Detection() if det is None else det
    det.clear()
    r = np.asarray(rec)
    if r.dtype != DETECTION_RECORD:
        r = np.frombuffer(r.tobytes(), DETECTION_RECORD)[0]
    # the sent values as they are, assigned directly: a detector's refined
    # time may be slightly negative and its amplitude factor 0, which the
    # public setters refuse
    for i, t in enumerate(_AMP):
        if r["have_amplitude%d" % (i + 1)]:
            det._amp[t] = float(r["amplitude%d" % (i + 1)])
    if r["have_correlation_coefficient"]:
        det._xc = float(r["correlation_coefficient"])
    for f, attr in _TIME_ATTRS:
        if r["have_" + f]:
            setattr(det, attr, float(r[f]))
    if r["have_detected_signal"]:
        n = int(r["signal_length"])
        if signal is None or len(signal) != n:
            raise ValueError("detected signal of %d samples expected" % n)
        det.set_detected_signal(np.asarray(signal, dtype=np.float64))
    if r["have_template_id"]:
        nsp = NetworkStationPhase()
        nsp.set_network(_unstr(r["network"]))
        nsp.set_station(_unstr(r["station"]))
        nsp.set_phase(_unstr(r["phase"]))
        det.set_template_identifier((nsp, int(r["template_id"])))
    # a byte other than -1, 0, 1 (a sender's uninitialised padding) reads as unknown
    pol = int(r["polarity"])
    det.set_polarity(Polarity(pol) if pol in (-1, 0, 1) else Polarity.unknown)
    return det


def unpack_detections(recs, signals):
    """Inverse of pack_detections."""
    out, o = [], 0
    for r in recs:
        n = int(r["signal_length"]) if r["have_detected_signal"] else 0
        out.append(unpack_detection(r, signals[o:o + n] if n else None))
        o += n
    if o != len(signals):
        raise ValueError("%d signal samples for records that hold %d" % (len(signals), o))
    return out


def _bytes_tensor(a):
    return torch.from_numpy(np.frombuffer(np.ascontiguousarray(a).tobytes(), np.uint8).copy())


_TORCH = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


def _check_dtype(dtype):
    dtype = np.dtype(dtype)
    if dtype not in _TORCH:
        raise ValueError("dtype must be float32 or float64")
    return dtype


def send(detection, dest, tag=0, group=None, dtype=np.float64):
    """MPI::Send (src/mpi.cpp:386-414): the detection's record, then its
    detected signal in ``dtype`` when it has one."""
    dtype = _check_dtype(dtype)
    if not isinstance(detection, Detection):
        raise ValueError("detection must be a Detection")
    r = pack_detection(detection)
    dist.send(_bytes_tensor(r), dst=dest, group=group, tag=tag)
    if r["have_detected_signal"]:
        dist.send(torch.from_numpy(detection.get_detected_signal().astype(dtype)), dst=dest, group=group, tag=tag)


def recv(detection=None, source=None, tag=0, group=None, dtype=np.float64):
    """MPI::Recv (src/mpi.cpp:416-450): a detection from ``source`` (any rank
    when None).  Returns (detection, sender rank); ``detection`` is cleared
    and filled when given."""
    dtype = _check_dtype(dtype)
    buf = torch.empty(DETECTION_RECORD.itemsize, dtype=torch.uint8)
    src = dist.recv(buf, src=source, group=group, tag=tag)
    r = np.frombuffer(buf.numpy().tobytes(), DETECTION_RECORD)[0]
    sig = None
    if r["have_detected_signal"]:
        t = torch.empty(int(r["signal_length"]), dtype=_TORCH[dtype])
        dist.recv(t, src=src, group=group, tag=tag)
        sig = t.numpy()
    return unpack_detection(r, sig, detection), src


def pack_template(template):
    """A template's broadcast payload: (TEMPLATE_HEADER scalar, the
    identifier's network, station, channel, location code and phase as one
    UTF-8 byte string, FP64 samples)."""
    if not isinstance(template, WaveformTemplate):
        raise ValueError("template must be a WaveformTemplate")
    st = template.__getstate__()
    h = np.zeros((), TEMPLATE_HEADER)
    h["sampling_rate"] = st["fs"]
    h["weight"] = st["weight"]
    h["onset"] = st["onset"]
    h["travel"] = st["travel"]
    if st["mag"] is not None:
        h["have_magnitude"] = True
        h["magnitude"] = st["mag"]
    h["polarity"] = st["polarity"]
    x = np.zeros(0) if st["x"] is None else np.asarray(st["x"], dtype=np.float64)
    h["n_samples"] = x.size
    strings = b""
    if st["ident"] is not None:
        h["have_identifier"] = True
        h["template_id"] = int(st["ident"][1])
        parts = [f.encode("utf-8") for f in st["ident"][0]]
        h["string_bytes"] = [len(f) for f in parts]
        strings = b"".join(parts)
    return h, strings, x


def unpack_template(header, strings, samples, template=None):
    """Inverse of pack_template: ``template`` (or a new one) cleared and
    given the payload's fields."""
    h = np.asarray(header)
    if h.dtype != TEMPLATE_HEADER:
        h = np.frombuffer(h.tobytes(), TEMPLATE_HEADER)[0]
    lens = [int(v) for v in h["string_bytes"]]
    n = int(h["n_samples"])
    if len(samples) != n or len(strings) != sum(lens):
        raise ValueError("payload does not match its header")
    ident = None
    if h["have_identifier"]:
        o, parts = 0, []
        for k in lens:
            parts.append(bytes(strings[o:o + k]).decode("utf-8"))
            o += k
        ident = (tuple(parts), int(h["template_id"]))
    template = WaveformTemplate() if template is None else template
    template.__setstate__(dict(x=np.array(samples, dtype=np.float64) if n > 0 else None,
                               fs=float(h["sampling_rate"]), weight=float(h["weight"]), onset=float(h["onset"]),
                               travel=float(h["travel"]),
                               mag=float(h["magnitude"]) if h["have_magnitude"] else None,
                               polarity=int(h["polarity"]), ident=ident))
    return template


def broadcast(template, root, group=None):
    """MPI::Broadcast (src/mpi.cpp:294-384): on exit every rank's
    ``template`` equals the root's (non-root templates are cleared first;
    every optional field travels with a presence flag, so an onset time of
    0 arrives too).  Three broadcasts at most: header, identifier strings,
    samples."""
    if not isinstance(template, WaveformTemplate):
        raise ValueError("template must be a WaveformTemplate")
    me = dist.get_rank()
    if me == root:
        h, strings, x = pack_template(template)
    else:
        h, strings, x = np.zeros((), TEMPLATE_HEADER), b"", None
    hb = _bytes_tensor(h)
    dist.broadcast(hb, src=root, group=group)
    h = np.frombuffer(hb.numpy().tobytes(), TEMPLATE_HEADER)[0]
    nstr, n = int(h["string_bytes"].sum()), int(h["n_samples"])
    if nstr > 0:
        sb = torch.from_numpy(np.frombuffer(strings, np.uint8).copy()) if me == root else \
            torch.empty(nstr, dtype=torch.uint8)
        dist.broadcast(sb, src=root, group=group)
        strings = sb.numpy().tobytes()
    if n > 0:
        xt = torch.from_numpy(x) if me == root else torch.empty(n, dtype=torch.float64)
        dist.broadcast(xt, src=root, group=group)
        x = xt.numpy()
    if me == root:
        return template
    return unpack_template(h, strings, x if n > 0 else np.zeros(0), template)


def gather_detections(detections, dst=0, tag=0, group=None, dtype=np.float64):
    """Every rank's detections to rank ``dst``, in rank order: each rank
    sends (count, signal samples), its records and its signals in ``dtype``
    (three messages at most, none when it has no detections).  Returns the
    list on ``dst`` and None elsewhere.  The ``dst`` rank's own detections
    pass through the same records, so every entry holds the transmitted
    fields only."""
    dtype = _check_dtype(dtype)
    recs, sigs = pack_detections(list(detections), dtype)
    me = dist.get_rank()
    if me != dst:
        dist.send(torch.tensor([len(recs), sigs.size], dtype=torch.int64), dst=dst, group=group, tag=tag)
        if len(recs):
            dist.send(_bytes_tensor(recs), dst=dst, group=group, tag=tag)
        if sigs.size:
            dist.send(torch.from_numpy(sigs), dst=dst, group=group, tag=tag)
        return None
    ranks = dist.get_process_group_ranks(group) if group is not None else range(dist.get_world_size())
    out = []
    for r in ranks:
        if r == me:
            out += unpack_detections(recs, sigs)
            continue
        cnt = torch.empty(2, dtype=torch.int64)
        dist.recv(cnt, src=r, group=group, tag=tag)
        n, ns = int(cnt[0]), int(cnt[1])
        rr = np.zeros(0, DETECTION_RECORD)
        ss = np.zeros(0, dtype)
        if n:
            b = torch.empty(n * DETECTION_RECORD.itemsize, dtype=torch.uint8)
            dist.recv(b, src=r, group=group, tag=tag)
            rr = np.frombuffer(b.numpy().tobytes(), DETECTION_RECORD)
        if ns:
            t = torch.from_numpy(np.zeros(ns, dtype))
            dist.recv(t, src=r, group=group, tag=tag)
            ss = t.numpy()
        out += unpack_detections(rr, ss)
    return out
