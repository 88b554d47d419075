"""Batched tonal solves (acum_batch_*): many decks in one persistent launch.

Cases are drawn like the 64-case batched workload (2-6 blades, uneven element, step and
observer counts, tip Mach 0.4-0.7, Minf 0-0.2) but shrunk so that the FP64 oracle
finishes in seconds.  Checks: every case of the persistent launch (direct and CUDA-graph
replay) against the same deck solved alone through the single-deck mixed path and
against the FP64 oracle; one launch per case (mode 1) against the persistent launch; all
tile shapes the autotuner may pick; the autotuner itself; and the error paths."""
import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from metrics import oaspl_db, per_bin_rms
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = (0, 5, 11, 17, 23, 42)
SHRINK = dict(n_span=12, n_chord_side=6, nobs=40)
# mixed form against FP64 (the tonal tests' bounds)
OASPL_DB = 0.05
BIN_RMS = 1e-4
# two mixed solves of the same deck that differ only in how the elements are cut into
# work items (FP32 partial sums flushed at different element boundaries)
SAME_FORM_RMS = 1e-5


def shrunk(case):
    d = synth.batch_deck(case, shrink=dict(SHRINK))
    return d


@pytest.fixture(scope="module")
def batch():
    from acum3_periodic_gb300 import native
    decks = [shrunk(c) for c in CASES]
    b = native.Batch(0)
    for d in decks:
        b.add(d)
    yield b, decks
    b.close()


@pytest.fixture(scope="module")
def singles(batch):
    from acum3_periodic_gb300 import native
    _, decks = batch
    ctx = native.Context(0)
    out = []
    for d in decks:
        ctx.set_deck(d, bb=False)
        out.append(ctx.tonal(native.MIXED)[2])
    ctx.close()
    return out


def test_shapes_are_uneven(batch):
    b, decks = batch
    assert b.count() == len(CASES)
    assert len({d.nTime for d in decks}) > 2
    assert len({d.E for d in decks}) > 2


def test_persistent_matches_single_deck_path(batch, singles):
    b, decks = batch
    b.set_tile(16, 4, 8)
    b.run(mode=0)
    for i, d in enumerate(decks):
        got = b.result(i)
        assert got.shape == (d.nTime, d.nObs)
        assert per_bin_rms(got, singles[i]).max() < SAME_FORM_RMS, i


def test_graph_replay_matches_and_repeats(batch, singles):
    b, decks = batch
    b.run(mode=2)
    first = [b.result(i) for i in range(len(decks))]
    b.run(mode=2)
    for i in range(len(decks)):
        assert per_bin_rms(first[i], singles[i]).max() < SAME_FORM_RMS
        assert per_bin_rms(b.result(i), first[i]).max() < 1e-12
    ms, launches = b.timing()
    assert ms > 0 and launches == 2


def test_one_launch_per_case_matches(batch, singles):
    b, decks = batch
    b.run(mode=1)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < 1e-12
        assert b.case_ms(i) > 0
    _, launches = b.timing()
    # per case the ring kernel, the wide-ring kernel (cases of more than 1024 steps), the
    # whole-row kernel, finalize
    assert launches == sum(4 if d.nTime > 1024 else 3 for d in decks)


def test_against_fp64_oracle(batch):
    b, decks = batch
    b.run(mode=0)
    for i in (0, 3, 5):
        _, _, ref, _ = O.tonal(decks[i], nthreads=8)
        got = b.result(i)
        assert np.max(np.abs(oaspl_db(got) - oaspl_db(ref))) < OASPL_DB
        assert per_bin_rms(got, ref).max() < BIN_RMS


@pytest.mark.parametrize("W,SE,ips,opw", [(8, 2, 4, 1), (12, 4, 16, 1), (16, 2, 8, 1), (5, 4, 1, 1), (16, 8, 8, 1),
                                         (7, 8, 2, 1), (32, 8, 8, 2), (16, 4, 4, 2), (24, 2, 8, 2), (6, 8, 1, 2)])
def test_tile_shapes_agree(batch, singles, W, SE, ips, opw):
    b, decks = batch
    b.set_tile(W, SE, ips, opw)
    assert b.tile() == (W, SE, ips) and b.obs_per_warp() == opw
    b.run(mode=0)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, (W, SE, ips, opw, i)


def test_tile_with_kept_values(batch, singles):
    """A shape of one observer per warp set with 0 observers per block after a shape of 32
    (two per warp) keeps 16, the most one-observer warps a block holds; 0 elements per stage
    and items per SM keep theirs."""
    b, decks = batch
    b.set_tile(32, 8, 8, 2)
    b.set_tile(0, 4, 0, 1)
    assert b.tile() == (16, 4, 8) and b.obs_per_warp() == 1
    b.run(mode=0)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, i


def test_autotune(batch, singles):
    b, decks = batch
    est = b.autotune()
    W, SE, ips = b.tile()
    if b.obs_per_warp() == 1:
        assert W in (8, 12, 16) and SE in (2, 4, 8)
    else:
        assert b.obs_per_warp() == 2 and W in (16, 24, 32) and SE in (2, 4, 8)
    assert ips in (4, 8, 16, 32)
    assert est > 0
    b.run(mode=2)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS


def test_ring_and_whole_row_cases_in_one_launch():
    """A batch whose cases take different forms: one in forward flight with an observer
    9 cm from the hub, which the bin ring's bound does not cover (its items run on whole
    rows), beside cases that run on the ring; every case matches its single-deck solve and
    the FP64 oracle."""
    from acum3_periodic_gb300 import native
    near = synth.config_deck(0, replicate=39, scale=dict(n_span=4, n_chord_side=3, ntime=72, nobs=5, minf=0.1))
    obs = near.obs_file.copy()
    obs[2] = np.array([0.0, 0.0, 0.09], np.float32) / np.float32(near.OBSscale)
    near.obs_file = obs
    decks = [shrunk(0), near, shrunk(5)]
    ctx = native.Context(0)
    singles, forms = [], []
    for d in decks:
        ctx.set_deck(d, bb=False)
        singles.append(ctx.tonal(native.MIXED)[2])
        forms.append(ctx.last_plan()["ring_used"])
    ctx.close()
    assert forms == [512, 0, 512]
    b = native.Batch(0)
    for d in decks:
        b.add(d)
    for W, SE, ips, opw in ((32, 8, 8, 2), (16, 8, 8, 1)):
        b.set_tile(W, SE, ips, opw)
        b.run(mode=0)
        for i, d in enumerate(decks):
            got = b.result(i)
            assert per_bin_rms(got, singles[i]).max() < SAME_FORM_RMS, (W, i)
    _, _, ref, _ = O.tonal(near, nthreads=8)
    assert per_bin_rms(b.result(1), ref).max() < BIN_RMS
    b.close()


def test_errors():
    from acum3_periodic_gb300 import native
    b = native.Batch(0)
    with pytest.raises(native.AcumError):
        b.run(mode=0)  # no cases
    b.add(shrunk(0))
    with pytest.raises(native.AcumError):
        b.run(mode=0, precision=native.PLAIN_FP64)
    with pytest.raises(native.AcumError):
        b.run(mode=3)
    with pytest.raises(native.AcumError):
        b.set_tile(17, 4, 8)
    with pytest.raises(native.AcumError):
        b.set_tile(8, 3, 8)
    with pytest.raises(native.AcumError):
        b.result(0)  # no run yet
    b.run(mode=0)
    with pytest.raises(native.AcumError):
        b.result(1)
    with pytest.raises(native.AcumError):
        b.case_ms(0)  # last run was not one launch per case
    b.close()


def test_wide_ring_case_in_a_batch():
    """A case whose records reach past the bin ring (2048 steps at tip Mach 0.8: a live
    span of 514 bins) runs on the wide ring of 1024 slots beside a case on the ring.  The
    default shape then holds fewer than 32 observers per block, an explicit shape whose
    rows do not fit is refused, and every case matches its single-deck solve and the FP64
    oracle."""
    from acum3_periodic_gb300 import native
    wide = synth.config_deck(0, replicate=37, scale=dict(n_span=4, n_chord_side=3, ntime=2048, nobs=6, tip_mach=0.8,
                                                         minf=0.0))
    decks = [shrunk(0), wide]
    ctx = native.Context(0)
    singles, forms = [], []
    for d in decks:
        ctx.set_deck(d, bb=False)
        singles.append(ctx.tonal(native.MIXED)[2])
        forms.append(ctx.last_plan()["ring_used"])
    ctx.close()
    assert forms == [512, 1024]
    b = native.Batch(0)
    for d in decks:
        b.add(d)
    b.run(mode=0)
    assert b.tile()[0] < 32
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, i
    b.set_tile(32, 8, 8, 2)
    with pytest.raises(native.AcumError):
        b.run(mode=0)
    b.set_tile(16, 8, 8, 1)
    b.run(mode=0)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, (16, i)
    _, _, ref, _ = O.tonal(wide, nthreads=8)
    assert per_bin_rms(b.result(1), ref).max() < BIN_RMS
    b.close()


def test_cases_on_every_ring_in_one_launch():
    """Cases on the ring (512 slots), the wide ring (1024: 2048 steps at tip Mach 0.8) and
    the widest (2048: 4096 steps at tip Mach 0.9) in one launch of the default shape, which
    then holds 12 observers per block, one per warp; each case matches its single-deck
    solve."""
    from acum3_periodic_gb300 import native
    decks = [shrunk(0)] + [synth.config_deck(0, replicate=37, scale=dict(n_span=4, n_chord_side=3, ntime=T, nobs=6,
                                                                           tip_mach=tip, minf=0.0))
                           for T, tip in ((2048, 0.8), (4096, 0.9))]
    ctx = native.Context(0)
    singles, forms = [], []
    for d in decks:
        ctx.set_deck(d, bb=False)
        singles.append(ctx.tonal(native.MIXED)[2])
        forms.append(ctx.last_plan()["ring_used"])
    ctx.close()
    assert forms == [512, 1024, 2048]
    b = native.Batch(0)
    for d in decks:
        b.add(d)
    b.run(mode=0)
    assert b.tile()[0] == 12 and b.obs_per_warp() == 1
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, i
    b.close()


def test_autotune_with_rows_no_probed_shape_holds():
    """A case whose records need whole rows of 4096 steps (an observer 9 cm from the hub in
    forward flight, outside every ring's bound) leaves room for at most 6 observer rows per
    block, fewer than any shape the autotuner probes: it keeps the default shape shrunk to
    fit, and every case matches its single-deck solve."""
    from acum3_periodic_gb300 import native
    near = synth.config_deck(0, replicate=39, scale=dict(n_span=4, n_chord_side=3, ntime=4096, nobs=3, minf=0.1))
    obs = near.obs_file.copy()
    obs[1] = np.array([0.0, 0.0, 0.09], np.float32) / np.float32(near.OBSscale)
    near.obs_file = obs
    decks = [near, shrunk(5)]
    ctx = native.Context(0)
    singles, forms = [], []
    for d in decks:
        ctx.set_deck(d, bb=False)
        singles.append(ctx.tonal(native.MIXED)[2])
        forms.append(ctx.last_plan()["ring_used"])
    ctx.close()
    assert forms == [0, 512]
    b = native.Batch(0)
    for d in decks:
        b.add(d)
    assert b.autotune() > 0
    assert b.tile()[0] <= 6
    b.run(mode=2)
    for i in range(len(decks)):
        assert per_bin_rms(b.result(i), singles[i]).max() < SAME_FORM_RMS, i
    b.close()
