"""acum_find_pressure_time_history_noalloc: the tonal drop-in for callers that cannot
allocate memory (it keeps its scratch in a fixed device array instead of calling
cudaMalloc).  Its output must match the allocating entry point's, within the mixed-form
tolerance of the other tests, on two calls in a row (the second call reuses the scratch
the first one left behind).  Collected last on purpose."""
import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from oracle import oracle as O

from metrics import oaspl_db, per_bin_rms
from test_dropin_gpu import call_dropin

pytestmark = pytest.mark.gpu

MIXED_RMS_TOL = 1e-4


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    L = native.lib()
    d = synth.config_deck(3, replicate=80, scale=dict(n_span=5, n_chord_side=3, ntime=70, nobs=9))
    f = O.preprocess(d)
    rc, rT, rL, rA = call_dropin(L.acum_find_pressure_time_history, d, f, np.float32, torch)
    assert rc == 0, L.acum_last_global_error()
    for _ in range(2):
        rc, nT, nL, nA = call_dropin(L.acum_find_pressure_time_history_noalloc, d, f, np.float32, torch)
        assert rc == 0, L.acum_noalloc_last_error()
        for a, b in ((nT, rT), (nL, rL), (nA, rA)):
            assert per_bin_rms(a, b).max() < MIXED_RMS_TOL


def test_noalloc_long_period_on_the_wide_ring():
    """2048 steps at tip Mach 0.8: the records reach past the 512-slot ring (a live span of
    514 bins), so both drop-in entry points solve on the wide ring; they agree with each
    other, and with the oracle within the float interface's bound.  The scalars arrive as
    float32, as the reference passes them, so oM / dPsi (bins per second) carries a
    relative error of ~1e-7; an observer ~5000 bins of travel time away (20 radii at 2048
    steps) then has its whole signal shifted by ~5e-4 bins.  Measured against the oracle:
    the FP64 drop-in given the same float32 scalars 2.3e-3 of the observer RMS, with
    float32 fields and exact scalars 4e-7; the mixed drop-in 1.4e-3; the context entry
    point (FP64 scalars) 8.7e-5."""
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    L = native.lib()
    d = synth.config_deck(0, replicate=37, scale=dict(n_span=4, n_chord_side=3, ntime=2048, nobs=6, tip_mach=0.8,
                                                       minf=0.0))
    f = O.preprocess(d)
    _, _, oA, bad = O.tonal(d)
    assert bad == 0
    rc, rT, rL, rA = call_dropin(L.acum_find_pressure_time_history, d, f, np.float32, torch)
    assert rc == 0, L.acum_last_global_error()
    rc, nT, nL, nA = call_dropin(L.acum_find_pressure_time_history_noalloc, d, f, np.float32, torch)
    assert rc == 0, L.acum_noalloc_last_error()
    for a, b in ((nT, rT), (nL, rL), (nA, rA)):
        assert per_bin_rms(a, b).max() < MIXED_RMS_TOL
    assert per_bin_rms(nA, oA).max() < 3e-3
    assert np.abs(oaspl_db(nA) - oaspl_db(oA)).max() < 0.05


def test_noalloc_rejects_oversized_problems():
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    L = native.lib()
    # 4000 observers x 4096 steps of FP64 sums alone exceed the 128 MiB scratch
    d = synth.config_deck(0, replicate=81, scale=dict(n_span=1, n_chord_side=2, ntime=4096, nobs=4000))
    f = np.zeros((d.E, d.nTime, 18))
    f[:, :, 0] = 1.0
    rc, *_ = call_dropin(L.acum_find_pressure_time_history_noalloc, d, f, np.float32, torch)
    assert rc == -1
    assert b"maximum is" in L.acum_noalloc_last_error()


def test_noalloc_refuses_what_the_allocating_entry_point_refuses():
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    L = native.lib()
    d = synth.config_deck(0, replicate=82, scale=dict(n_span=2, n_chord_side=2, ntime=40, nobs=3))
    f = O.preprocess(d)
    # a bin grid other than t * dPsi: both entry points refuse it with ACUM_ERR_UNSUPPORTED
    tobs = np.arange(d.nTime, dtype=np.float32) * np.float32(d.derived()["dPsi"]) * np.float32(1.01)
    rc_a, *_ = call_dropin(L.acum_find_pressure_time_history, d, f, np.float32, torch, tobs=tobs)
    rc_n, *_ = call_dropin(L.acum_find_pressure_time_history_noalloc, d, f, np.float32, torch, tobs=tobs)
    assert rc_a == rc_n == -8
    assert b"tObs" in L.acum_noalloc_last_error()
    # the shortest period both accept: 4 steps
    d4 = synth.config_deck(0, replicate=83, scale=dict(n_span=2, n_chord_side=2, ntime=4, nobs=3))
    f4 = O.preprocess(d4)
    rc_a, aT, aL, aA = call_dropin(L.acum_find_pressure_time_history, d4, f4, np.float32, torch)
    rc_n, nT, nL, nA = call_dropin(L.acum_find_pressure_time_history_noalloc, d4, f4, np.float32, torch)
    assert rc_a == rc_n == 0, L.acum_noalloc_last_error()
    assert per_bin_rms(nA, aA).max() < MIXED_RMS_TOL
