"""The oracle against the reference's own sources compiled here (oracle/_ref), on fresh
seeded decks beyond the committed fixtures.  Skipped on machines without the reference
build (oracle/_ref is built only where the reference source tree is present)."""
import os

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from acum3_periodic_gb300.deck import read_deck, write_deck
from oracle import oracle as O, ref as R

pytestmark = pytest.mark.skipif(not R.available("f64"), reason="reference build (oracle/_ref) not present")


@pytest.mark.parametrize("cfg,rep,lowpass,periodic", [(0, 1, 0, 1), (1, 2, 0, 1), (3, 3, 1, 1), (3, 4, 1, 0)])
def test_tonal_random_decks(tmp_path, cfg, rep, lowpass, periodic):
    d = synth.config_deck(cfg, replicate=rep, scale=dict(n_span=3, n_chord_side=3, ntime=30, nobs=7, bb_nsect=5,
                                                         bb_small=True, n_bb=2))
    d.lowpass, d.periodic = lowpass, periodic
    write_deck(d, str(tmp_path))
    rd = R.RefDeck(str(tmp_path), "f64")
    pT, pL, pA = rd.tonal()
    oT, oL, oA, bad = O.tonal(d, nthreads=3)
    assert bad == 0
    for a, b in ((pT, oT), (pL, oL), (pA, oA)):
        assert np.max(np.abs(a - b)) <= 1e-12 * np.abs(a).max()


def test_reader_matches_reference_reader(tmp_path):
    """The Python deck reader against read_inputs/read_observers/read_surf/read_BB_inputs."""
    d = synth.config_deck(1, replicate=5, scale=dict(n_span=2, n_chord_side=2, ntime=12, nobs=5, bb_nsect=4,
                                                     bb_small=True, n_bb=2))
    d.OBSscale = 1.5
    d.CFDscale = 0.5
    write_deck(d, str(tmp_path))
    rd = R.RefDeck(str(tmp_path), "f32")
    r = read_deck(str(tmp_path))
    np.testing.assert_array_equal(rd.observers(), r.observers().astype(np.float64))
    X, N, _, P = rd.fields()
    raw = np.concatenate([s.transpose(1, 0, 2) for s in r.surfaces], axis=0)  # [E][T][8]
    np.testing.assert_array_equal(X[:, :, :3], raw[:, :, :3])
    np.testing.assert_array_equal(X[:, :, 3], raw[:, :, 4])
    np.testing.assert_array_equal(N[:, :, :3], raw[:, :, 5:8])
    np.testing.assert_array_equal(P[:, :, 0], raw[:, :, 3])
    dv = r.derived()
    assert rd.scalars["dTau"] == pytest.approx(dv["dTau"], rel=1e-6)
    assert rd.scalars["vx"] == pytest.approx(dv["vInf"][0], rel=1e-6)


@pytest.mark.parametrize("t_del", [0, 1, 2])
def test_bpm_random_decks(tmp_path, t_del):
    d = synth.config_deck(1, replicate=20 + t_del, scale=dict(n_span=2, n_chord_side=2, ntime=20, nobs=4,
                                                              bb_nsect=5, bb_small=True, n_bb=2))
    d.t_del = t_del
    if t_del == 0:
        for b in d.bb:
            c = b.geom[:, 3] * b.span
            b.data[:, :, 0] = 0.013 * c
            b.data[:, :, 1] = 0.009 * c
            b.data[:, :, 2] = 0.0035 * c
            b.data[:, :, 3] = 0.002 * c
    d.bb[0].trip = 0
    write_deck(d, str(tmp_path))
    rd = R.RefDeck(str(tmp_path), "f64")
    spl, oas = rd.bpm()
    ospl, ooas = O.bpm(d, aa_mode=1, nthreads=2)
    np.testing.assert_allclose(ospl, spl, rtol=0, atol=1e-9)
    np.testing.assert_allclose(ooas, oas, rtol=0, atol=1e-9)


def test_bpm_core_random_inputs(tmp_path):
    d = synth.config_deck(1, replicate=6, scale=dict(n_span=2, n_chord_side=2, ntime=8, nobs=2, bb_nsect=4,
                                                     bb_small=True, n_bb=1))
    write_deck(d, str(tmp_path))
    rd = R.RefDeck(str(tmp_path), "f64")
    ff = rd.bands()
    u = synth.uniform(9, 3, 200 * 16).reshape(200, 16)
    for k in range(200):
        a = u[k]
        args = [5 + 45 * a[0], 0.01 + 3.1 * a[1], 0.01 + 3.1 * a[2], 0.05 + 0.15 * a[3], 0.01 + 0.09 * a[4],
                25 * a[5], 20 + 230 * a[6], 0.0000181206 / 1.22500, 340.0, 1e-4 + 5e-3 * a[7], 1e-4 + 5e-3 * a[8],
                1e-5 + 1e-3 * a[9], 1e-5 + 1e-3 * a[10], 0.1, 0.5 + 1.5 * a[11]]
        trip, isect = int(a[12] * 2), int(a[13] * 3)
        want = rd.core(args, trip, isect, 3)
        out = np.full(42 * 7, -100.0)
        O.lib().acumo_bpm_core(*args[:9], trip, *args[9:13], isect, 3, O._p(ff), 42, args[14], O._p(out))
        np.testing.assert_allclose(out.reshape(42, 7), want, rtol=0, atol=1e-9)


@pytest.mark.parametrize("rep,ntime,periodic,lowpass", [(31, 24, 1, 1), (32, 61, 0, 0), (33, 200, 1, 0),
                                                         (34, 6, 0, 1), (35, 7, 1, 1)])
def test_permeable_preprocessing_random(rep, ntime, periodic, lowpass):
    ne = [2 + rep % 3, 4, 1]
    X, N, U, PR = synth.permeable_rows(rep, ne, ntime)
    rng = np.random.default_rng(rep)
    PR[:, :, 0] += 0.05 * rng.standard_normal(PR.shape[:2])  # not smooth: the median filter acts
    args = (1.0 / (ntime * 7.3), 341.0, 1.18, 0.11, 2.5, periodic, lowpass)
    want = R.preprocess_per(ne, X, N, np.zeros_like(N), U, PR, *args)
    got = O.preprocess_per(X, N, U, PR, *args)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
