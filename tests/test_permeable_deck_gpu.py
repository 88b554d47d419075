"""Permeable decks (impermeable 0) through the context API and the host program, as the
reference driver runs them: read_surf reads 12-column rows (io.cu:263-293), main.cu:87
runs preprocess_per, main.cu:236 launches no acoustic kernel, so pT, pL and pA stay as
main.cu:123-130 zeroed them and writeTimeHistory writes zero files.

Checked against the golden deck tests/golden/decks/permeable_deck/ (generated by
tests/golden/make_golden.py with the reference's own readers and preprocessing): the
context's preprocessed arrays equal the reference's FP64 build bit for bit
(permeable_deck.npz) and the oracle's restatement; the written pT.out, pL.out and pA.out
equal the reference's files (expected/, written by its FP32 build) byte for byte, both
from acum_write_outputs and from the acum_gb300 program; the surface-row cache keeps
the 12-column rows."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from acum3_periodic_gb300.deck import read_deck
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DECK = os.path.join(GOLDEN, "decks", "permeable_deck")
FILES = ("pT.out", "pL.out", "pA.out")
ERR_UNSUPPORTED = -8


@pytest.fixture()
def deck_dir(tmp_path):
    p = tmp_path / "permeable_deck"
    shutil.copytree(DECK, p, ignore=shutil.ignore_patterns("expected"))
    return p


@pytest.fixture(scope="module")
def ctx():
    from acum3_periodic_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def oracle_fields(d):
    """preprocess_per of the oracle on the deck's rows as read_surf stores them."""
    der = d.derived()
    rows = np.concatenate([s.transpose(1, 0, 2) for s in d.surfaces], axis=0).astype(np.float64)
    X = np.zeros(rows.shape[:2] + (4,))
    N = np.zeros(rows.shape[:2] + (6,))
    U = np.zeros(rows.shape[:2] + (6,))
    PR = np.zeros(rows.shape[:2] + (4,))
    X[..., 0:3], X[..., 3] = rows[..., 0:3], rows[..., 8]
    N[..., 0:3], U[..., 0:3] = rows[..., 9:12], rows[..., 3:6]
    PR[..., 0], PR[..., 2] = rows[..., 6], rows[..., 7]
    return O.preprocess_per(X, N, U, PR, der["dTau"], der["a0"], der["rhoRef"], der["Mref"], der["CFDscale"],
                            der["periodic"], der["lowpass"])


def test_loaded_deck_preprocessing_equals_reference(ctx, deck_dir):
    from acum3_periodic_gb300 import native
    ctx.load_deck(str(deck_dir))
    got = ctx.permeable_fields()
    g = np.load(os.path.join(GOLDEN, "permeable_deck.npz"))
    for a, k in zip(got, ("X", "N", "V", "U", "PR")):
        assert np.array_equal(a, g[k]), k
    for a, b in zip(got, oracle_fields(read_deck(str(deck_dir)))):
        assert np.array_equal(a, b)
    # the impermeable-only paths refuse the deck with a status
    with pytest.raises(native.AcumError) as e:
        ctx.fields()
    assert e.value.code == ERR_UNSUPPORTED
    with pytest.raises(native.AcumError) as e:
        ctx.adjoint(native.PLAIN_FP64)
    assert e.value.code == ERR_UNSUPPORTED


def test_pressures_zero_and_files_equal_reference(ctx, deck_dir):
    from acum3_periodic_gb300 import native
    ctx.load_deck(str(deck_dir))
    for prec in (native.MIXED, native.PLAIN_FP64):
        pT, pL, pA = ctx.tonal(prec)
        assert not pT.any() and not pL.any() and not pA.any()
    out = deck_dir / "out"
    out.mkdir()
    ctx.write_outputs(str(out))
    for f in FILES:
        with open(out / f, "rb") as a, open(os.path.join(DECK, "expected", f), "rb") as b:
            assert a.read() == b.read(), f


def test_host_program_and_surface_cache(deck_dir):
    from acum3_periodic_gb300 import native
    from acum3_periodic_gb300.build import EXE
    r = subprocess.run([EXE, str(deck_dir)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout
    for f in FILES:
        with open(deck_dir / f, "rb") as a, open(os.path.join(DECK, "expected", f), "rb") as b:
            assert a.read() == b.read(), f
    # the binary cache of the 12-column rows gives the same preprocessed arrays
    c = native.Context(0)
    try:
        c.load_deck(str(deck_dir))
        text = c.permeable_fields()
        assert native.lib().acum_write_surface_cache(os.fsencode(str(deck_dir))) == 0
        assert (deck_dir / "surfaces" / "surfaces.acumbin").exists()
        c.load_deck(str(deck_dir))
        for a, b in zip(text, c.permeable_fields()):
            assert np.array_equal(a, b)
    finally:
        c.close()


def test_set_deck_from_memory_and_back_to_impermeable(ctx):
    """A permeable deck set from memory (synthetic, two surfaces), then an impermeable
    one on the same context: each gives its own results."""
    from acum3_periodic_gb300 import native
    d = synth.permeable_deck(23, [5, 7], 36, nobs=2, lowpass=0, periodic=1)
    ctx.set_deck(d, bb=False)
    for a, b in zip(ctx.permeable_fields(), oracle_fields(d)):
        assert np.array_equal(a, b)
    imp = synth.config_deck(0, replicate=86, scale=dict(n_span=2, n_chord_side=2, ntime=24, nobs=3))
    ctx.set_deck(imp, bb=False)
    _, _, pA = ctx.tonal(native.PLAIN_FP64)
    _, _, oA, _ = O.tonal(imp)
    assert np.abs(pA - oA).max() <= 1e-10 * np.abs(oA).max()
    with pytest.raises(native.AcumError):
        ctx.permeable_fields()
