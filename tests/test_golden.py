"""The oracle against the committed golden vectors generated from the reference's own
FP64 build (tests/golden/make_golden.py).  Runs anywhere; no reference tree needed."""
import os

import numpy as np
import pytest

from acum3_periodic_gb300.deck import read_deck
from oracle import oracle as O

from conftest import GOLDEN

TONAL = ["tonal_hover", "tonal_flight_lowpass", "bb_tdel2", "bb_tdel1_lbl_cw", "bb_tdel0_hover"]
BB = ["bb_tdel2", "bb_tdel1_lbl_cw", "bb_tdel0_hover"]


def _load(name):
    return read_deck(os.path.join(GOLDEN, "decks", name)), np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", TONAL)
def test_preprocess_matches_reference_fp64(name):
    d, g = _load(name)
    f = O.preprocess(d)
    np.testing.assert_array_equal(f[:, :, 0:4], g["fields_X"])
    np.testing.assert_allclose(f[:, :, 4:10], g["fields_N"], rtol=0, atol=1e-12 * np.abs(g["fields_N"]).max())
    np.testing.assert_allclose(f[:, :, 10:16], g["fields_V"], rtol=0, atol=1e-12 * np.abs(g["fields_V"]).max())
    np.testing.assert_allclose(f[:, :, 16:18], g["fields_P"], rtol=0, atol=1e-12 * np.abs(g["fields_P"]).max())


@pytest.mark.parametrize("name", TONAL)
def test_tonal_matches_reference_fp64(name):
    d, g = _load(name)
    pT, pL, pA, bad = O.tonal(d, nthreads=2)
    assert bad == 0
    for k, v in (("pT", pT), ("pL", pL), ("pA", pA)):
        ref = g[k + "_f64"]
        scale = np.abs(ref).max(axis=0, keepdims=True)
        assert np.max(np.abs(v - ref) / scale) < 1e-12, k


@pytest.mark.parametrize("name", BB)
def test_bpm_matches_reference_fp64(name):
    """aa_mode=1: the golden build zero-initialises the unset `aa` of bb_core.cu:520."""
    d, g = _load(name)
    spl, oas = O.bpm(d, aa_mode=1, nthreads=2)
    np.testing.assert_allclose(spl, g["spl_f64"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(oas, g["oaspl_f64"], rtol=0, atol=1e-9)


def test_fp32_reference_is_close_but_not_the_target():
    """The as-written FP32 reference differs from its FP64 build by FP32 rounding; this
    records the size of that gap on the hover deck (informational bound)."""
    _, g = _load("tonal_hover")
    scale = np.abs(g["pA_f64"]).max()
    gap = np.abs(g["pA_f32"] - g["pA_f64"]).max() / scale
    assert 1e-9 < gap < 1e-3


def test_unit_vectors():
    u = np.load(os.path.join(GOLDEN, "units.npz"))
    for w, nm in enumerate(("a_min", "a_max", "b_min", "b_max")):
        np.testing.assert_allclose(O.bb_curve(w, u["x_ab"]), u[nm], rtol=1e-14, atol=1e-12)
    g5 = np.array([[O.g5comp(h, e) for e in u["g5_eta"]] for h in u["g5_h"]])
    np.testing.assert_allclose(g5, u["g5"], rtol=1e-14, atol=1e-12)
    np.testing.assert_allclose(O.make_periodic(u["series"]), u["make_periodic"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(O.lowpass(u["series"]), u["lowpass"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(O.differentiate(u["series"], 0.01), u["diff_periodic"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(O.differentiate(u["series"], 0.01, True), u["diff_biased"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("periodic,lowpass", [(1, 0), (0, 1)])
def test_permeable_preprocessing(periodic, lowpass):
    """The oracle's preprocess_per against the reference's FP64 build on a seeded rotating
    data surface (two surfaces): every output array bit for bit."""
    g = np.load(os.path.join(GOLDEN, "permeable.npz"))
    out = O.preprocess_per(g["X"], g["N"], g["U"], g["PR"], *g["scal"], periodic, lowpass)
    for nm, a in zip("XNVUP", out):
        want = g["%s_p%d_l%d" % (nm, periodic, lowpass)]
        np.testing.assert_array_equal(a, want)


def test_permeable_deck_preprocessing():
    """The oracle's preprocess_per on the golden permeable deck as the Python reader reads
    it (12-column rows) against the reference's FP64 build on the same directory, loaded
    with its own readers: every array bit for bit."""
    from acum3_periodic_gb300.deck import read_deck
    d = read_deck(os.path.join(GOLDEN, "decks", "permeable_deck"))
    assert d.impermeable == 0 and d.ncol == 12
    der = d.derived()
    rows = np.concatenate([s.transpose(1, 0, 2) for s in d.surfaces], axis=0).astype(np.float64)
    X = np.zeros(rows.shape[:2] + (4,))
    N = np.zeros(rows.shape[:2] + (6,))
    U = np.zeros(rows.shape[:2] + (6,))
    PR = np.zeros(rows.shape[:2] + (4,))
    X[..., 0:3], X[..., 3] = rows[..., 0:3], rows[..., 8]
    N[..., 0:3], U[..., 0:3] = rows[..., 9:12], rows[..., 3:6]
    PR[..., 0], PR[..., 2] = rows[..., 6], rows[..., 7]
    out = O.preprocess_per(X, N, U, PR, der["dTau"], der["a0"], der["rhoRef"], der["Mref"], der["CFDscale"],
                           der["periodic"], der["lowpass"])
    g = np.load(os.path.join(GOLDEN, "permeable_deck.npz"))
    for a, k in zip(out, ("X", "N", "V", "U", "PR")):
        np.testing.assert_array_equal(a, g[k])
