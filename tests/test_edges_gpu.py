"""Edge cases of the tonal path: the smallest decks the readers accept, the longest period
the preprocessing supports (4096 steps, where the bin rows of one observer take 32 KB of
shared memory and the blocks hold few observers), and the decks the library refuses with
a status instead of running (no observers, too few or too many steps)."""
import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from oracle import oracle as O

from metrics import oaspl_db, per_bin_rel, per_bin_rms

pytestmark = pytest.mark.gpu

ERR_INVALID, ERR_UNSUPPORTED = -1, -8  # include/acum.h

F64_TOL = 1e-10
MIXED_RMS_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    from acum3_periodic_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _against_oracle(ctx, d, rms_norm=False):
    """rms_norm: the FP64 error normalised by the observer's RMS instead of by the bin's
    own value (a long period has bins near zero, where summation-order differences of
    ~1e-16 of the terms are large relative to the bin)."""
    from acum3_periodic_gb300 import native
    oT, oL, oA, bad = O.tonal(d)
    assert bad == 0
    ctx.set_deck(d, bb=False)
    _, _, pA = ctx.tonal(native.PLAIN_FP64)
    assert (per_bin_rms(pA, oA) if rms_norm else per_bin_rel(pA, oA)).max() < F64_TOL
    _, _, mA = ctx.tonal(native.MIXED)
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL
    assert np.abs(oaspl_db(mA) - oaspl_db(oA)).max() < 0.05
    assert ctx.error_word(reset=True) == 0
    return ctx.last_plan()


def test_smallest_deck(ctx):
    """One observer, one panel per blade side (two elements per blade), 8 steps."""
    d = synth.config_deck(0, replicate=80, scale=dict(n_span=1, n_chord_side=1, ntime=8, nobs=1))
    assert d.nObs == 1 and d.E == 4
    plan = _against_oracle(ctx, d)
    assert plan["obs_per_block"] == plan["obs_per_warp"]  # one warp


def test_longest_period(ctx):
    """4096 steps per period: the retarded times spread over more bins than the mixed
    ring holds (a live span of 671 bins), and the wide ring does the work; with whole rows
    asked for, the whole-row kernel's blocks hold only as many observer rows as fit in
    shared memory (fewer than 16).  Both match the oracle."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=81, scale=dict(n_span=2, n_chord_side=2, ntime=4096, nobs=9))
    plan = _against_oracle(ctx, d, rms_norm=True)
    assert plan["ring_used"] == 1024 and plan["wide_obs_per_block"] == 10  # 9 observers, two per warp
    _, _, oA, _ = O.tonal(d)
    ctx.set_tile(whole_rows=1)
    try:
        _, _, mA = ctx.tonal(native.MIXED)
        plan = ctx.last_plan()
    finally:
        ctx.set_tile()
    assert plan["ring_slots"] == 0 and plan["ring_used"] == 0 and plan["obs_per_block"] < 9
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL
    assert ctx.error_word(reset=True) == 0


def test_refused_decks(ctx):
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=82, scale=dict(n_span=2, n_chord_side=2, ntime=24, nobs=3))
    none = synth.config_deck(0, replicate=82, scale=dict(n_span=2, n_chord_side=2, ntime=24, nobs=3))
    none.obs_file = np.zeros((0, 3), np.float32)
    with pytest.raises(native.AcumError) as e:
        ctx.set_deck(none, bb=False)
    assert e.value.code == ERR_INVALID
    short = synth.config_deck(0, replicate=83, scale=dict(n_span=2, n_chord_side=2, ntime=5, nobs=3))
    with pytest.raises(native.AcumError) as e:
        ctx.set_deck(short, bb=False)
    assert e.value.code == ERR_INVALID
    long = synth.config_deck(0, replicate=84, scale=dict(n_span=1, n_chord_side=1, ntime=4097, nobs=2))
    ctx.set_deck(long, bb=False)
    with pytest.raises(native.AcumError) as e:
        ctx.tonal(native.MIXED)
    assert e.value.code == ERR_UNSUPPORTED
    # the context still solves a valid deck afterwards
    _against_oracle(ctx, d)
