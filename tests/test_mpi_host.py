"""Wire formats of the multi-rank path (mflib_gb300.mpi, the MFLib::MPI
functions of src/mpi.cpp over torch.distributed): the detection record's
layout is the C layout of the reference's MPIDetection struct, records
round-trip every field, and two gloo ranks exchange detections (send /
recv), broadcast a template and gather detections to either rank."""
import ctypes as C
import os
import shutil
import socket
import subprocess
import sys

import numpy as np
import pytest

from mflib_gb300 import NetworkStationPhase, Polarity, WaveformTemplate, mpi
from mflib_gb300.detector import Detection, RelativeMagnitudeType

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _CRecord(C.Structure):
    # src/mpi.cpp:20-51 restated with ctypes' C alignment rules
    _fields_ = ([(n, C.c_double) for n in ("a1", "a2", "xc", "t", "ti", "po", "poi", "tt")] +
                [(n, C.c_char * 64) for n in ("net", "sta", "pha")] +
                [("id", C.c_uint64), ("n", C.c_int32)] + [("h%d" % i, C.c_bool) for i in range(10)])


def test_record_layout_is_the_c_struct():
    assert C.sizeof(_CRecord) == mpi.DETECTION_RECORD.itemsize == 280
    names = [f[0] for f in _CRecord._fields_]
    for cname, (field, (_, off)) in zip(names, list(mpi.DETECTION_RECORD.fields.items())[:23]):
        assert getattr(_CRecord, cname).offset == off, field
    # the polarity byte sits in the struct's tail padding
    assert mpi.DETECTION_RECORD.fields["polarity"][1] == 278 > _CRecord.h9.offset


def _nsp(net, sta, pha, cha="", loc=""):
    n = NetworkStationPhase()
    n.set_network(net)
    n.set_station(sta)
    n.set_phase(pha)
    n.set_channel(cha)
    n.set_location_code(loc)
    return n


def _dets(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = Detection()
        if i % 2 == 0:
            d.set_template_identifier((_nsp("uu", "st%d" % i, "p" if i % 4 else "s"), int(rng.integers(2**63))))
        if i % 3 != 1:
            d.set_correlation_coefficient(float(rng.uniform(-1, 1)))
        if i % 3 != 2:
            d.set_detected_signal(rng.standard_normal(int(rng.integers(1, 40))))
        d.set_detection_time(float(rng.uniform(0, 1e5)))
        if i % 2:
            d.set_interpolated_detection_time(float(rng.uniform(0, 1e5)))
            d.set_phase_onset_time(0.0)
            d.set_amplitude_scaling_factor(float(rng.uniform(0.1, 5)), RelativeMagnitudeType.gibbons_ringdal_2006)
        else:
            d.set_interpolated_phase_onset_time(float(rng.uniform(0, 1e5)))
            d.set_travel_time(float(rng.uniform(0, 100)))
            d.set_amplitude_scaling_factor(float(rng.uniform(0.1, 5)), RelativeMagnitudeType.schaff_richards_2014)
        d.set_polarity((Polarity.compression, Polarity.dilatation, Polarity.unknown)[i % 3])
        out.append(d)
    return out


def _state(d, dtype=np.float64):
    st = d.__getstate__()
    if st["sig"] is not None:
        st["sig"] = np.asarray(st["sig"], dtype).tolist()
    return st


def test_record_round_trip_every_field():
    dets = _dets(1, 12)
    for d in dets:
        e = mpi.unpack_detection(mpi.pack_detection(d), d.get_detected_signal() if d.have_detected_signal() else None)
        assert _state(e) == _state(d)
    recs, sig = mpi.pack_detections(dets, np.float32)
    assert sig.dtype == np.float32 and recs.dtype == mpi.DETECTION_RECORD
    got = mpi.unpack_detections(recs, sig)
    assert [_state(g) for g in got] == [_state(d, np.float32) for d in dets]
    # the bytes alone carry the record
    assert not dets[2].have_detected_signal()
    e = mpi.unpack_detection(mpi.pack_detection(dets[2]).tobytes(), None)
    assert _state(e) == _state(dets[2])


def test_record_truncation_and_dropped_fields():
    d = Detection()
    d.set_template_identifier((_nsp("n" * 70, "sta", "p", cha="ehz", loc="01"), 7))
    e = mpi.unpack_detection(mpi.pack_detection(d))
    nsp, wid = e.get_template_identifier()
    # 64 bytes of a name travel (src/mpi.cpp:182-193); channel and location
    # code are not in the record
    assert wid == 7 and nsp.get_network() == "N" * 64 and nsp.get_station() == "STA"
    assert nsp.get_channel() == "" and nsp.get_location_code() == ""
    # the receiver's earlier fields are cleared
    tgt = Detection()
    tgt.set_detection_time(5.0)
    assert not mpi.unpack_detection(mpi.pack_detection(d), det=tgt).have_detection_time()
    with pytest.raises(ValueError):
        mpi.unpack_detection(mpi.pack_detection(_dets(2, 1)[0]), None)  # its signal is missing
    # a record carries what the detector computed, even where the public
    # setters would refuse it (a refined time just below 0)
    r = mpi.pack_detection(Detection())
    r["have_interpolated_detection_time"], r["interpolated_detection_time"] = True, -0.004
    assert mpi.unpack_detection(r).get_interpolated_detection_time() == -0.004
    # a polarity byte outside -1, 0, 1 reads as unknown
    r = mpi.pack_detection(_dets(3, 1)[0])
    r["polarity"] = 77
    assert mpi.unpack_detection(r, _dets(3, 1)[0].get_detected_signal()).get_polarity() == Polarity.unknown
    with pytest.raises(ValueError):
        mpi.pack_detections([Detection()], np.int32)
    with pytest.raises(ValueError):
        mpi.send(Detection(), 0, dtype=np.int32)  # refused before any message


def _template():
    wt = WaveformTemplate()
    wt.set_signal(np.sin(np.arange(300) / 7.0))
    wt.set_sampling_rate(100.0)
    wt.set_shift_and_stack_weight(0.25)
    wt.set_phase_onset_time_in_signal(0.0)
    wt.set_phase_travel_time(12.5)
    wt.set_magnitude(-0.5)
    wt.set_polarity(Polarity.dilatation)
    wt.set_identifier((_nsp("uu", "ctu", "p", cha="ehz", loc="01"), 2**64 - 3))
    return wt


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        res = {}
        dets = _dets(10 + rank, 3 if rank == 0 else 2)
        # point to point: rank 1 sends two detections, rank 0 takes them from
        # any source, the second in float32
        if rank == 1:
            mpi.send(dets[0], 0, tag=7)
            mpi.send(dets[1], 0, tag=8, dtype=np.float32)
        else:
            a, sa = mpi.recv(source=None, tag=7)
            b, sb = mpi.recv(Detection(), source=1, tag=8, dtype=np.float32)
            res["recv"] = (sa, sb, a.__getstate__(), b.__getstate__())
        # broadcast from rank 1; rank 0's template had other fields
        wt = _template() if rank == 1 else WaveformTemplate()
        if rank == 0:
            wt.set_signal(np.ones(5))
            wt.set_sampling_rate(40.0)
        mpi.broadcast(wt, root=1)
        res["bcast"] = wt.__getstate__()
        res["g0"] = mpi.gather_detections(dets, dst=0)
        res["g1"] = mpi.gather_detections(dets if rank == 1 else [], dst=1, dtype=np.float32)
        res["g0"] = None if res["g0"] is None else [d.__getstate__() for d in res["g0"]]
        res["g1"] = None if res["g1"] is None else [d.__getstate__() for d in res["g1"]]
        q.put((rank, res))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    d0, d1 = _dets(10, 3), _dets(11, 2)
    sa, sb, a, b = got[0]["recv"]
    assert (sa, sb) == (1, 1)
    assert a == _state(d1[0]) and b == _state(d1[1], np.float32)
    want = _template().__getstate__()
    assert got[0]["bcast"] == want and got[1]["bcast"] == want
    assert got[1]["g0"] is None and got[0]["g1"] is None
    assert got[0]["g0"] == [_state(d) for d in d0 + d1]
    assert got[1]["g1"] == [_state(d, np.float32) for d in d1]


def _fixed_detection():
    # the detection tests/cpp/test_mpi_wire.cpp writes (fixedDetection)
    d = Detection()
    d.set_template_identifier((_nsp("uu", "ctu", "p"), 12345678901234))
    d.set_correlation_coefficient(0.625)
    d.set_detection_time(101.25)
    d.set_interpolated_detection_time(101.3125)
    d.set_travel_time(7.5)
    d.set_amplitude_scaling_factor(2.5, RelativeMagnitudeType.gibbons_ringdal_2006)
    d.set_polarity(Polarity.dilatation)
    d.set_detected_signal([0.5, -1.25, 2.0])
    return d


def _fixed_template():
    # fixedTemplate of tests/cpp/test_mpi_wire.cpp
    wt = WaveformTemplate()
    wt.set_signal([1.0, -2.0, 3.5, 0.25])
    wt.set_sampling_rate(100.0)
    wt.set_shift_and_stack_weight(0.5)
    wt.set_phase_onset_time_in_signal(0.0)
    wt.set_phase_travel_time(3.0)
    wt.set_magnitude(1.5)
    wt.set_polarity(Polarity.compression)
    wt.set_identifier((_nsp("uu", "ctu", "p", cha="ehz", loc="01"), 42))
    return wt


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not found")
def test_cpp_wire_code_and_same_bytes(tmp_path):
    """The C++ header's Send / Recv / Broadcast / Gather pass their checks
    over the in-process MPI stand-in, and its records are the Python
    module's bytes."""
    exe = str(tmp_path / "test_mpi_wire")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "tests", "cpp", "fake_mpi"),
                        os.path.join(ROOT, "tests", "cpp", "test_mpi_wire.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and "ALL PASSED" in run.stdout, run.stdout + run.stderr
    assert (tmp_path / "detection.bin").read_bytes() == mpi.pack_detection(_fixed_detection()).tobytes()
    h, strings, x = mpi.pack_template(_fixed_template())
    assert (tmp_path / "template_header.bin").read_bytes() == h.tobytes()
    assert (tmp_path / "template_strings.bin").read_bytes() == strings == b"UUCTUEHZ01P"
    assert (tmp_path / "template_samples.bin").read_bytes() == x.tobytes()
    # and the C++ bytes unpack to the same objects in Python
    e = mpi.unpack_detection((tmp_path / "detection.bin").read_bytes(), [0.5, -1.25, 2.0])
    assert _state(e) == _state(_fixed_detection())
    t = mpi.unpack_template((tmp_path / "template_header.bin").read_bytes(), strings,
                            np.frombuffer((tmp_path / "template_samples.bin").read_bytes(), np.float64))
    assert t.__getstate__() == _fixed_template().__getstate__()
