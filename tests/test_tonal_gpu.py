"""Tonal path on the GPU (through the C ABI) against the oracle and the golden vectors
of the reference's FP64 build.

Tolerances: the plain FP64 form must agree per bin to 1e-10 relative, normalised as
|p - ref| / max(|ref|, 1e-6 max_t|ref|); the mixed form is held to a per-bin error of
1e-4 of the observer's RMS and to the OASPL bound of 0.05 dB (observed: far below)."""
import os

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from acum3_periodic_gb300.deck import read_deck
from oracle import oracle as O

from conftest import GOLDEN
from metrics import oaspl_db, per_bin_rel, per_bin_rms

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
MIXED_RMS_TOL = 1e-4
# The mixed form at 4096 steps per revolution: its FP32 observer-time offsets carry a
# relative error of a few 1e-7, i.e. an absolute error that grows with the records' reach
# in bins (up to ~500 here), and the bins of a long period resolve the sharp thickness
# pulses of a fast blade; measured 1.3e-4 (tip Mach 0.6) to 3.9e-4 (0.8) of the observer
# RMS, alike on the ring, the wide ring and whole rows (the FP64 form: < 4e-11).
LONG_PERIOD_RMS_TOL = 6e-4
# a ring form against whole rows on the same deck (summation orders differ)
SAME_DECK_RMS_TOL = 1e-5
OASPL_TOL_DB = 0.05

TONAL = ["tonal_hover", "tonal_flight_lowpass", "bb_tdel2", "bb_tdel1_lbl_cw", "bb_tdel0_hover"]


@pytest.fixture(scope="module")
def ctx():
    from acum3_periodic_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _golden(name):
    return read_deck(os.path.join(GOLDEN, "decks", name)), np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", TONAL)
def test_preprocess_fields_match_reference(ctx, name):
    d, g = _golden(name)
    ctx.set_deck(d, bb=False)
    f = ctx.fields()
    np.testing.assert_array_equal(f[:, :, 0:3], g["fields_X"][:, :, 0:3])
    for sl, key in ((slice(3, 4), None), (slice(4, 10), "fields_N"), (slice(10, 16), "fields_V"),
                    (slice(16, 18), "fields_P")):
        want = g["fields_X"][:, :, 3:4] if key is None else g[key]
        np.testing.assert_allclose(f[:, :, sl], want, rtol=0, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("name", TONAL)
def test_fp64_matches_reference_build(ctx, name):
    from acum3_periodic_gb300 import native
    d, g = _golden(name)
    ctx.set_deck(d, bb=False)
    pT, pL, pA = ctx.tonal(native.PLAIN_FP64)
    for k, v in (("pT", pT), ("pL", pL), ("pA", pA)):
        err = per_bin_rel(v, g[k + "_f64"]).max()
        assert err < F64_TOL, (k, err)
    assert ctx.error_word(reset=True) == 0


@pytest.mark.parametrize("name", TONAL)
def test_mixed_against_fp64_reference(ctx, name):
    from acum3_periodic_gb300 import native
    d, g = _golden(name)
    ctx.set_deck(d, bb=False)
    pT, pL, pA = ctx.tonal(native.MIXED)
    ref = g["pA_f64"]
    assert per_bin_rms(pA, ref).max() < MIXED_RMS_TOL
    assert np.abs(oaspl_db(pA) - oaspl_db(ref)).max() < OASPL_TOL_DB
    np.testing.assert_allclose(pA, pT + pL, rtol=0, atol=1e-12 * np.abs(pA).max())


@pytest.mark.parametrize("cfg,rep,scale", [
    (0, 31, dict(n_span=7, n_chord_side=5, ntime=45, nobs=13)),        # T not a multiple of 32
    (1, 32, dict(n_span=5, n_chord_side=3, ntime=64, nobs=37, bb_nsect=4, bb_small=True, n_bb=1)),
    (3, 33, dict(n_span=9, n_chord_side=4, ntime=90, nobs=21)),
])
def test_random_decks_against_oracle(ctx, cfg, rep, scale):
    from acum3_periodic_gb300 import native
    d = synth.config_deck(cfg, replicate=rep, scale=scale)
    oT, oL, oA, bad = O.tonal(d)
    assert bad == 0
    ctx.set_deck(d, bb=False)
    pT, pL, pA = ctx.tonal(native.PLAIN_FP64)
    assert per_bin_rel(pA, oA).max() < F64_TOL
    assert per_bin_rel(pT, oT).max() < F64_TOL
    mT, mL, mA = ctx.tonal(native.MIXED)
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL
    assert np.abs(oaspl_db(mA) - oaspl_db(oA)).max() < OASPL_TOL_DB


def test_config0_full_size(ctx):
    """Workload 0 at its full size (2 x 1200 elements, 360 steps, 16 observers)."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0)
    oT, oL, oA, bad = O.tonal(d)
    ctx.set_deck(d, bb=False)
    pT, pL, pA = ctx.tonal(native.PLAIN_FP64)
    assert per_bin_rel(pA, oA).max() < F64_TOL
    mT, mL, mA = ctx.tonal(native.MIXED)
    assert np.abs(oaspl_db(mA) - oaspl_db(oA)).max() < OASPL_TOL_DB
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL


def test_linearity_in_cp_and_blade_periodicity(ctx):
    """pL is linear in Cp and pT does not depend on it (scaling by 4 is exact in float32);
    a second blade that is exactly the first one half a revolution later makes pA repeat
    every half revolution."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=40, scale=dict(n_span=4, n_chord_side=3, ntime=48, nobs=5))
    ctx.set_deck(d, bb=False)
    pT, pL, pA = ctx.tonal(native.PLAIN_FP64)
    for s in d.surfaces:
        s[:, :, 3] *= 4.0
    ctx.set_deck(d, bb=False)
    qT, qL, qA = ctx.tonal(native.PLAIN_FP64)
    np.testing.assert_allclose(qT, pT, rtol=0, atol=1e-12 * np.abs(pT).max())
    np.testing.assert_allclose(qL, 4.0 * pL, rtol=0, atol=1e-12 * np.abs(pL).max())
    # make_periodic fits a cubic at the series seam, so only a Cp series that is already
    # periodic (here: constant in time) is left untouched by it
    s0 = d.surfaces[0]
    s0[:, :, 3] = s0[0:1, :, 3]
    d.surfaces[1] = np.ascontiguousarray(np.roll(s0, -(d.nTime // 2), axis=0))
    ctx.set_deck(d, bb=False)
    _, _, rA = ctx.tonal(native.PLAIN_FP64)
    np.testing.assert_allclose(rA, np.roll(rA, d.nTime // 2, axis=0), rtol=0, atol=1e-11 * np.abs(rA).max())


def test_element_permutation_invariance(ctx):
    from acum3_periodic_gb300 import native
    d = synth.config_deck(3, replicate=41, scale=dict(n_span=5, n_chord_side=3, ntime=40, nobs=6))
    ctx.set_deck(d, bb=False)
    _, _, pA = ctx.tonal(native.PLAIN_FP64)
    perm = np.array(synth.uniform(5, 1, d.surfaces[0].shape[1]).argsort())
    d.surfaces[0] = np.ascontiguousarray(d.surfaces[0][:, perm, :])
    ctx.set_deck(d, bb=False)
    _, _, qA = ctx.tonal(native.PLAIN_FP64)
    np.testing.assert_allclose(qA, pA, rtol=0, atol=1e-12 * np.abs(pA).max())


def test_load_deck_and_write_outputs(ctx, tmp_path):
    """The file-format drop-in: load a deck directory, write pT/pL/pA.out."""
    from acum3_periodic_gb300 import native
    import shutil
    src = os.path.join(GOLDEN, "decks", "tonal_hover")
    dst = tmp_path / "deck"
    shutil.copytree(src, dst)
    ctx.load_deck(str(dst))
    pT, pL, pA = ctx.tonal(native.PLAIN_FP64)
    ctx.write_outputs(str(dst))
    g = np.load(os.path.join(GOLDEN, "tonal_hover.npz"))
    lines = open(dst / "pA.out").read().splitlines()
    assert lines[0] == "# ntime nobs"
    T, Ob = (int(x) for x in lines[1].split())
    assert (T, Ob) == g["pA_f64"].shape
    vals = np.array([[float(x) for x in l.split()] for l in lines[2:]])
    np.testing.assert_allclose(vals[:, 1:], g["pA_f64"], rtol=1e-8, atol=1e-8 * np.abs(g["pA_f64"]).max())
    assert lines[3].startswith(" ") and "E" in lines[3]


def test_timing_and_launch_count(ctx):
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=42, scale=dict(n_span=4, n_chord_side=3, ntime=36, nobs=4))
    ctx.set_deck(d, bb=False)
    ctx.tonal(native.MIXED)
    ms, launches = ctx.timing(0)
    assert ms > 0 and launches >= 3


@pytest.mark.parametrize("W,SE,opw,tm,rows", [
    # the ring kernel
    (32, 8, 2, 2, 0), (32, 4, 2, 2, 0), (32, 2, 2, 2, 0), (16, 8, 2, 2, 0), (6, 4, 2, 2, 0),
    (16, 8, 1, 2, 0), (16, 4, 1, 2, 0), (16, 2, 1, 2, 0), (7, 8, 1, 2, 0),
    # whole rows only
    (16, 8, 1, 2, 1), (16, 4, 1, 2, 1), (16, 2, 1, 2, 1), (7, 8, 1, 2, 1),
    # whole rows with the record stages in tensor memory
    (16, 8, 1, 1, 0), (16, 4, 1, 1, 0), (16, 2, 1, 1, 0), (5, 8, 1, 1, 0)])
def test_mixed_tile_shapes_against_oracle(ctx, W, SE, opw, tm, rows):
    """Every tile shape of the mixed kernels (observers per block, elements per stage,
    observers per warp; the bin ring or whole rows; record stages in shared or tensor
    memory) on a deck whose observers, steps and elements are not multiples of the tile;
    the plan reports the shape that ran."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=34, scale=dict(n_span=7, n_chord_side=5, ntime=75, nobs=29))
    oT, oL, oA, bad = O.tonal(d)
    assert bad == 0
    ctx.set_deck(d, bb=False)
    try:
        ctx.set_tile(W, SE, 0, opw, tm, rows)
        _, _, mA = ctx.tonal(native.MIXED)
        plan = ctx.last_plan()
    finally:
        ctx.set_tile()
    assert (plan["obs_per_block"], plan["elems_per_stage"], plan["obs_per_warp"]) == (W, SE, opw)
    assert plan["tensor_memory"] == (1 if tm == 1 else 0)
    ring = tm != 1 and not rows
    assert plan["ring_slots"] == (512 if ring else 0)
    assert plan["ring_used"] == (512 if ring else 0)
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL
    assert np.abs(oaspl_db(mA) - oaspl_db(oA)).max() < OASPL_TOL_DB
    assert ctx.error_word(reset=True) == 0


def test_observer_near_the_origin_in_forward_flight(ctx):
    """An observer 9 cm from the hub of a rotor in forward flight (Mach 0.1): the ring
    kernel's bound on the observer-time offset needs every observer farther from the
    origin than 1.01 x |x|max x M / sqrt(1 - M^2) (10 cm here), so the whole-row kernel,
    which checks every sample's range, does the work; it matches the oracle."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=38, scale=dict(n_span=4, n_chord_side=3, ntime=72, nobs=4, minf=0.1))
    obs = d.obs_file.copy()
    obs[1] = np.array([0.0, 0.0, 0.09], np.float32) / np.float32(d.OBSscale)
    d.obs_file = obs
    oT, oL, oA, bad = O.tonal(d)
    assert bad == 0
    ctx.set_deck(d, bb=False)
    _, _, mA = ctx.tonal(native.MIXED)
    plan = ctx.last_plan()
    assert plan["ring_slots"] == 512 and plan["ring_used"] == 0
    assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL
    assert ctx.error_word(reset=True) == 0
    far = d.subset_observers([0, 2, 3])
    ctx.set_deck(far, bb=False)
    ctx.tonal(native.MIXED)
    assert ctx.last_plan()["ring_used"] == 512


def test_records_reaching_past_the_ring(ctx):
    """Hovering rotors whose retarded times spread over more bins than a ring holds: the
    reach of a source point is |x| x (bins per second) / a0, and the live span of a
    window 2 x reach + 40 bins (with the largest |x| of these blades, 0.90 of the tip
    radius: 588 x tip Mach bins either side at 4096 steps per revolution, 294 x tip Mach
    at 2048).  Each runs on the kernel the span selects, and matches the oracle:
    * 180 steps at tip Mach 0.8 (span 85) and 2048 at 0.68 (444 of 512): the ring;
    * 2048 steps at tip Mach 0.8 (514, just past the ring) and 4096 at 0.8 (984 of the
      wide ring's 1024): the 1024-slot wide ring launched behind it;
    * 4096 steps at tip Mach 0.9 (1102): the 2048-slot wide ring launched after that.
    Each agrees with whole rows asked for on the same deck."""
    from acum3_periodic_gb300 import native
    for T, tip, used in ((180, 0.8, 512), (2048, 0.68, 512), (2048, 0.8, 1024), (4096, 0.8, 1024),
                         (4096, 0.9, 2048)):
        d = synth.config_deck(0, replicate=37, scale=dict(n_span=4, n_chord_side=3, ntime=T, nobs=6, tip_mach=tip,
                                                           minf=0.0))
        oT, oL, oA, bad = O.tonal(d)
        assert bad == 0
        ctx.set_deck(d, bb=False)
        pT, pL, mA = ctx.tonal(native.MIXED)
        plan = ctx.last_plan()
        assert plan["ring_slots"] == 512 and plan["ring_used"] == used, T
        assert plan["wide_ring_slots"] == (1024 if T > 1024 else 0), T
        assert plan["wide2_ring_slots"] == (2048 if T > 2048 else 0), T
        assert plan["rows_obs_per_block"] > 0
        tol = LONG_PERIOD_RMS_TOL if T > 2048 else MIXED_RMS_TOL
        assert per_bin_rms(mA, oA).max() < tol, T
        assert np.abs(oaspl_db(mA) - oaspl_db(oA)).max() < OASPL_TOL_DB, T
        rms = np.sqrt(np.mean(oA ** 2, axis=0, keepdims=True))
        assert (np.abs(pT - oT) / rms).max() < tol, T
        assert ctx.error_word(reset=True) == 0
        if used:
            ctx.set_tile(whole_rows=1)
            try:
                _, _, rA = ctx.tonal(native.MIXED)
                assert ctx.last_plan()["ring_used"] == 0
            finally:
                ctx.set_tile()
            assert per_bin_rms(mA, rA).max() < SAME_DECK_RMS_TOL, T


def test_decks_in_sequence_on_one_context(ctx):
    """Decks of falling and rising sizes set one after the other on one context: each
    result matches the oracle, so nothing of a previous deck (its records in the padding
    of a reused buffer, its plan) reaches the next."""
    from acum3_periodic_gb300 import native
    for T, nobs, ns in [(96, 29, 7), (64, 29, 7), (45, 13, 7), (75, 29, 5), (45, 29, 7), (90, 29, 7)]:
        d = synth.config_deck(0, replicate=35, scale=dict(n_span=ns, n_chord_side=5, ntime=T, nobs=nobs))
        oT, oL, oA, bad = O.tonal(d)
        assert bad == 0
        ctx.set_deck(d, bb=False)
        _, _, pA = ctx.tonal(native.PLAIN_FP64)
        assert per_bin_rel(pA, oA).max() < F64_TOL, T
        _, _, mA = ctx.tonal(native.MIXED)
        assert per_bin_rms(mA, oA).max() < MIXED_RMS_TOL, T
        assert ctx.error_word(reset=True) == 0


def _observer_time_bins(d, fields):
    """u[o, e, tau]: observer time in bins of every sample (FP64, the retarded-time root
    of core.cu:261-279 and the observer time of core.cu:156)."""
    der = d.derived()
    x = fields[:, :, 0:3]
    v = np.asarray(der["vInf"], np.float64)
    a0 = float(der["a0"])
    alpha = a0 * a0 - v @ v
    out = []
    for o in d.observers().astype(np.float64):
        dd = o[None, None, :] - x
        c = np.sum(dd * dd, -1)
        beta = dd @ v
        tr = (np.sqrt(beta * beta + alpha * c) - beta) / alpha
        out.append((np.arange(d.nTime)[None, :] * float(der["dTau"]) + tr) * float(der["oM"]) / float(der["dPsi"]))
    return np.array(out)


def test_supersonic_intervals_of_three_bins(ctx):
    """A rotor at tip Mach 0.95 in a Mach 0.45 stream: the observer time advances by up
    to 2.5 bins per step on one side (intervals of three bins, the mixed kernel's
    per-stage extra pass) and runs backwards on the other (skipped and reported as
    ACUM_DEVERR_ORDER by both forms).  Near the Doppler singularity (1 - Mr -> 0) the
    integrand is unbounded and the two precisions part, so the forms are compared on the
    bins that no interval of less than 0.5 bins per step (or its neighbours) reaches;
    those bins include the three-bin intervals."""
    from acum3_periodic_gb300 import native
    d = synth.config_deck(0, replicate=36, scale=dict(n_span=6, n_chord_side=4, ntime=72, nobs=16,
                                                       tip_mach=0.95, minf=0.45))
    ctx.set_deck(d, bb=False)
    ctx.error_word(reset=True)
    _, _, ref = ctx.tonal(native.PLAIN_FP64)
    assert ctx.error_word(reset=True) & native.DEVERR_ORDER
    _, _, got = ctx.tonal(native.MIXED)
    assert ctx.error_word(reset=True) & native.DEVERR_ORDER
    assert np.all(np.isfinite(got))
    T = d.nTime
    u = _observer_time_bins(d, ctx.fields())                      # [O][E][T]
    ub = np.concatenate([u[:, :, -1:] - T, u], axis=2)             # interval k: (ub[k], ub[k+1]]
    du = np.diff(ub, axis=2)                                       # [O][E][T]
    near = du < 0.5
    near = near | np.roll(near, 1, axis=2) | np.roll(near, -1, axis=2)
    masked = np.zeros((T, d.nObs), bool)
    three = np.zeros((T, d.nObs), bool)
    for o, e, k in zip(*np.nonzero(near)):
        lo, hi = sorted((ub[o, e, k], ub[o, e, k + 1]))
        masked[np.arange(int(np.floor(lo)) - 1, int(np.ceil(hi)) + 2) % T, o] = True
    for o, e, k in zip(*np.nonzero(du > 2.0)):
        three[np.arange(int(np.floor(ub[o, e, k])) + 1, int(np.floor(ub[o, e, k + 1])) + 1) % T, o] = True
    keep = ~masked
    assert (keep & three).sum() >= 20
    rms = np.sqrt(np.mean(ref ** 2, axis=0, keepdims=True))
    assert np.max(np.abs(got - ref)[keep] / np.broadcast_to(rms, ref.shape)[keep]) < 1e-4
