"""Single-channel associator (mflib_gb300/associator.py: grouping on the
host, one segmented DBSCAN on the GPU) against the oracle's restatement of
Associator<T>::associate with the oracle DBSCAN."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _detections(mf, rng, nev=6, per=40, noise=60):
    from mflib_gb300.detector import Detection
    dets = []
    for e in range(nev):
        origins = rng.uniform(0, 3600, 3)
        for _ in range(per):
            o = rng.choice(origins) + rng.normal(0, 0.4)
            tt = rng.uniform(1, 30)
            d = Detection()
            d.set_template_identifier((mf.NetworkStationPhase(), 100 + e))
            d.set_travel_time(tt)
            d.set_phase_onset_time(o + tt)
            d.set_correlation_coefficient(float(rng.uniform(0.3, 1.0)))
            dets.append(d)
        for _ in range(noise // nev):
            d = Detection()
            d.set_template_identifier((mf.NetworkStationPhase(), 100 + e))
            tt = rng.uniform(1, 30)
            d.set_travel_time(tt)
            d.set_phase_onset_time(rng.uniform(0, 3600) + tt)
            d.set_correlation_coefficient(float(rng.uniform(0.3, 1.0)))
            dets.append(d)
    rng.shuffle(dets)
    return dets


@pytest.mark.parametrize("weighted", [False, True])
def test_associator_vs_oracle(gpu, oracle, rng, weighted):
    mf = gpu
    dets = _detections(mf, rng)
    prm = mf.SingleChannel.AssociatorParameters()
    prm.set_origin_time_tolerance(1.5)
    prm.set_minimum_number_of_picks_in_event(4 if not weighted else 2)
    if weighted:
        prm.enable_correlation_coefficient_weighting()
    asc = mf.SingleChannel.Associator()
    asc.initialize(prm)
    for d in dets:
        asc.add_detection(d)
    asc.associate()
    order, events = oracle.associate([d.get_template_identifier()[1] for d in dets],
                                     [d.get_phase_onset_time() for d in dets],
                                     [d.get_travel_time() for d in dets],
                                     [d.get_correlation_coefficient() for d in dets],
                                     prm.get_origin_time_tolerance(), prm.get_minimum_number_of_picks_in_event(),
                                     weighted)
    assert asc.get_number_of_events() == len(events) > 6
    for iev, (e, members) in enumerate(events):
        got = asc.get_detections_in_event(iev)
        assert asc.get_event_id(iev) == e
        assert [id(d) for d in got] == [id(dets[order[k]]) for k in members]


def test_associator_errors(gpu):
    mf = gpu
    from mflib_gb300.detector import Detection
    asc = mf.SingleChannel.Associator()
    with pytest.raises(RuntimeError):
        asc.add_detection(Detection())
    prm = mf.SingleChannel.AssociatorParameters()
    with pytest.raises(ValueError):
        prm.set_minimum_number_of_picks_in_event(0)
    with pytest.raises(ValueError):
        prm.set_origin_time_tolerance(-1.0)
    asc.initialize(prm)
    with pytest.raises(ValueError):
        asc.add_detection(Detection())  # no travel time
    asc.associate()
    assert asc.get_number_of_events() == 0
    assert asc.get_detections_in_event(0) == []  # pymflib: no events, nothing to return
