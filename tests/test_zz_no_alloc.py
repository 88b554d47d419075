"""acum_find_pressure_time_history_noalloc: the tonal drop-in for callers that cannot
allocate memory (it keeps its scratch in a fixed device array instead of calling
cudaMalloc).  Its output must match the allocating entry point's, within the mixed-form
tolerance of the other tests, on two calls in a row (the second call reuses the scratch
the first one left behind).  Collected last on purpose."""
import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from oracle import oracle as O

from metrics import per_bin_rms
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
