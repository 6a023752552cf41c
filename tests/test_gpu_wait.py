"""The bounded device waits' error path: a correlator whose segment copy is
never issued (test knob mfgpu_mf_test_wait_timeout; nothing is in flight)
gives up after its bounded wait, the apply reports MFGPU_ETIMEOUT at the next
synchronising call, and the same object's next apply is correct again."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("variant", [1, 2, 3])
def test_bounded_wait_times_out_and_recovers(gpu, oracle, rng, dtype, variant):
    mf = gpu
    from mflib_gb300 import _lib
    n = 30_000
    tps = [rng.standard_normal(300) for _ in range(3)]
    sig = rng.standard_normal(n)
    p = mf.SingleChannel.MatchedFilterParameters()
    for t in tps:
        wt = mf.WaveformTemplate()
        wt.set_signal(t)
        wt.set_sampling_rate(100.0)
        p.add_template(wt)
    p.set_signal_size(n)
    f = mf.SingleChannel.MatchedFilter(dtype=dtype)
    f.initialize(p, correlator_variant=variant)
    x = sig.astype(dtype)
    f.set_signal(x)
    _lib.call("mfgpu_mf_test_wait_timeout", f._h)
    f.apply()
    with pytest.raises(_lib.MfgpuTimeout):
        f.synchronize()
    assert not f.have_matched_filtered_signals()
    f.apply()
    ref = oracle.matched_filter(tps, [x], multi=False, fp64_from_f32=dtype == np.float32)
    tol = 1e-5 if dtype == np.float32 else 1e-11
    for t in range(len(tps)):
        rho = f.get_matched_filtered_signal(t).astype(np.float64)
        assert np.max(np.abs(rho - ref[t][: rho.size])) < tol


def test_wait_test_knob_rejected_for_tensor_cores(gpu, rng):
    mf = gpu
    from mflib_gb300 import _lib
    n = 20_000
    p = mf.SingleChannel.MatchedFilterParameters()
    wt = mf.WaveformTemplate()
    wt.set_signal(rng.standard_normal(200))
    wt.set_sampling_rate(100.0)
    p.add_template(wt)
    p.set_signal_size(n)
    f = mf.SingleChannel.MatchedFilter(dtype=np.float32)
    f.initialize(p, correlator_variant=4)
    with pytest.raises(ValueError):
        _lib.call("mfgpu_mf_test_wait_timeout", f._h)
