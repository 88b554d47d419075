"""Failure detection without a GPU fault: the bounded barrier wait of the pipelined
kernels.  A block waits on a barrier that nothing completes; the wait gives up after its
limit, reports it, and the device stays usable (a deck solves afterwards)."""
import numpy as np
import pytest

from acum3_periodic_gb300 import synth

pytestmark = pytest.mark.gpu

LIMIT_S = 0.2


def test_wait_gives_up_after_its_limit():
    from acum3_periodic_gb300 import native
    timed_out, waited = native.selftest_wait(0, LIMIT_S, arrive=False)
    assert timed_out
    assert LIMIT_S <= waited < LIMIT_S + 1.0


def test_wait_returns_at_once_when_completed():
    from acum3_periodic_gb300 import native
    timed_out, waited = native.selftest_wait(0, LIMIT_S, arrive=True)
    assert not timed_out
    assert waited < 0.01


def test_device_usable_after_a_timeout():
    from acum3_periodic_gb300 import native
    native.selftest_wait(0, LIMIT_S, arrive=False)
    d = synth.config_deck(0, scale=dict(n_span=4, n_chord_side=3, ntime=24, nobs=4))
    ctx = native.Context(0)
    ctx.set_deck(d, bb=False)
    _, _, pA = ctx.tonal(native.MIXED)
    assert np.all(np.isfinite(pA)) and np.abs(pA).max() > 0
    assert ctx.error_word() == 0
    ctx.close()
