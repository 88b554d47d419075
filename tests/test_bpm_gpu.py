"""Broadband (BPM) path on the GPU through the C ABI, against the golden vectors of the
reference's FP64 build and against the oracle.

Tolerances (dB): the FP32 spectral formulas with FP64 sums hold the total level of every
band and the OASPL to 0.01 dB, and each of the six component levels to 0.05 dB, of the
FP64 build.  aa_mode=1 reproduces the zero-initialised `aa` of bb_core.cu:520 (the golden
build); aa_mode=0 is the convected emission time the formula intends."""
import os

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from acum3_periodic_gb300.deck import read_deck
from oracle import oracle as O

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOTAL_DB = 0.01
COMP_DB = 0.05
BB = ["bb_tdel2", "bb_tdel1_lbl_cw", "bb_tdel0_hover"]


@pytest.fixture(scope="module")
def ctx():
    from acum3_periodic_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def _check(spl, oas, rspl, roas):
    assert np.all(np.isfinite(spl)) and np.all(np.isfinite(oas))
    assert np.abs(oas - roas).max() < TOTAL_DB
    assert np.abs(spl[:, :, 0] - rspl[:, :, 0]).max() < TOTAL_DB
    assert np.abs(spl - rspl).max() < COMP_DB


@pytest.mark.parametrize("name", BB)
def test_bpm_matches_reference_build(ctx, name):
    d = read_deck(os.path.join(GOLDEN, "decks", name))
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ctx.set_deck(d)
    spl, oas = ctx.bpm(aa_mode=1)
    _check(spl, oas, g["spl_f64"], g["oaspl_f64"])


@pytest.mark.parametrize("t_del,aa_mode", [(2, 0), (1, 0), (0, 1), (2, 1)])
def test_bpm_random_decks_against_oracle(ctx, t_del, aa_mode):
    d = synth.config_deck(1, replicate=50 + t_del, scale=dict(n_span=2, n_chord_side=2, ntime=48, nobs=37,
                                                              bb_nsect=9, bb_small=True, n_bb=3))
    d.t_del = t_del
    if t_del == 0:
        for b in d.bb:
            c = b.geom[:, 3] * b.span
            b.data[:, :, 0] = 0.013 * c
            b.data[:, :, 1] = 0.009 * c
            b.data[:, :, 2] = 0.0035 * c
            b.data[:, :, 3] = 0.002 * c
    d.bb[0].trip = 0
    d.bb[1].ccw = 0
    ospl, ooas = O.bpm(d, aa_mode=aa_mode)
    ctx.set_deck(d)
    spl, oas = ctx.bpm(aa_mode=aa_mode)
    _check(spl, oas, ospl, ooas)


def test_bpm_many_observers_and_sections(ctx):
    """More observers than one block and more (section, step) items than one split."""
    d = synth.config_deck(1, replicate=60, scale=dict(n_span=2, n_chord_side=2, ntime=90, nobs=70, bb_nsect=24,
                                                      bb_small=True, n_bb=2))
    ospl, ooas = O.bpm(d, aa_mode=0)
    ctx.set_deck(d)
    spl, oas = ctx.bpm(aa_mode=0)
    _check(spl, oas, ospl, ooas)
    ms, launches = ctx.timing(3)
    assert ms > 0 and launches == 6


def test_bpm_file_dropin_and_writer(ctx, tmp_path):
    import shutil
    src = os.path.join(GOLDEN, "decks", "bb_tdel2")
    dst = tmp_path / "deck"
    shutil.copytree(src, dst)
    ctx.load_deck(str(dst))
    spl, oas = ctx.bpm(aa_mode=1)
    ctx.tonal(0)
    ctx.write_outputs(str(dst))
    g = np.load(os.path.join(GOLDEN, "bb_tdel2.npz"))
    lines = open(dst / "bb_oaspl.out").read().splitlines()
    assert lines[0] == "nobs: %d" % len(g["oaspl_f64"])
    np.testing.assert_allclose([float(x) for x in lines[1:]], g["oaspl_f64"], atol=TOTAL_DB)
    txt = open(dst / "bb_spl.dat").read().splitlines()
    assert txt[0].strip() == "# nfrequency nobs"
    zones = [l for l in txt if "ZONE" in l]
    assert [z.split('"')[1] for z in zones] == ["TOTAL", "TBL_TE_P", "TBL_TE_S", "TBL_SS", "TEB_VS", "LBL-VS", "TVF"]
    first = [float(x) for x in txt[3].split()]
    assert first[0] == pytest.approx(1.0)
    np.testing.assert_allclose(first[1:], g["spl_f64"][:, 0, 0], atol=TOTAL_DB)


def test_find_bb_noise_dropin(tmp_path):
    """acum_find_bb_noise with the reference's 39 arguments (bb_core.cu:11)."""
    import ctypes as C
    from acum3_periodic_gb300 import native
    from acum3_periodic_gb300.deck import BB_BANDS
    d = synth.config_deck(1, replicate=61, scale=dict(n_span=2, n_chord_side=2, ntime=30, nobs=5, bb_nsect=6,
                                                      bb_small=True, n_bb=2))
    L = native.lib()
    bb = d.bb
    der = d.derived()
    f32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    i32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1))
    ns = [b.nsect for b in bb]
    xsPtr = np.cumsum([0] + [4 * n for n in ns[:-1]])
    dsPtr = np.cumsum([0] + [n * 7 * d.nTime for n in ns[:-1]])
    data = np.concatenate([b.data_as_read().reshape(-1) for b in bb])
    nst = [b.t_data.shape[0] for b in bb]; nm = [b.t_data.shape[1] for b in bb]
    nr = [b.t_data.shape[2] for b in bb]; na = [b.t_data.shape[3] for b in bb]
    sPtr = np.cumsum([0] + nst[:-1]); mPtr = np.cumsum([0] + nm[:-1]); rPtr = np.cumsum([0] + nr[:-1])
    aPtr = np.cumsum([0] + na[:-1])
    dPtr = np.cumsum([0] + [a * b * c * e * 7 for a, b, c, e in zip(nst, nm, nr, na)][:-1])
    args = dict(span=f32([b.span for b in bb]), omega=f32([b.omega for b in bb]), ccw=i32([b.ccw for b in bb]),
                psi=f32([b.psi_offset for b in bb]), trip=i32([b.trip for b in bb]),
                rot=f32([b.rotate for b in bb]), tra=f32([b.translate for b in bb]), xs=i32(xsPtr), ds=i32(dsPtr),
                nsect=i32(ns), xyz=f32([b.geom for b in bb]), data=f32(data), nst=i32(nst), nm=i32(nm), na=i32(na),
                nr=i32(nr), aP=i32(aPtr), mP=i32(mPtr), rP=i32(rPtr), sP=i32(sPtr), dP=i32(dPtr),
                sect=f32(np.concatenate([b.t_sect for b in bb])), mach=f32(np.concatenate([b.t_mach for b in bb])),
                aoa=f32(np.concatenate([b.t_aoa for b in bb])), re=f32(np.concatenate([b.t_re for b in bb])),
                tab=f32(np.concatenate([b.t_data.reshape(-1) for b in bb])), vinf=f32(der["vInf"]),
                robs=f32(d.observers()), tobs=f32(np.arange(d.nTime) * der["dPsi"]), ff=f32(BB_BANDS))
    spl = np.full((d.nObs, 42, 7), -100.0, np.float32)
    oas = np.full(d.nObs, -100.0, np.float32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    a = args
    rc = L.acum_find_bb_noise(len(bb), d.nObs, d.nTime, C.c_float(der["dTau"]), P(a["span"]), P(a["omega"]),
                              P(a["ccw"]), P(a["psi"]), P(a["trip"]), P(a["rot"]), P(a["tra"]), P(a["xs"]),
                              P(a["ds"]), P(a["nsect"]), P(a["xyz"]), P(a["data"]), P(a["nst"]), P(a["nm"]),
                              P(a["na"]), P(a["nr"]), P(a["aP"]), P(a["mP"]), P(a["rP"]), P(a["sP"]), P(a["dP"]),
                              P(a["sect"]), P(a["mach"]), P(a["aoa"]), P(a["re"]), P(a["tab"]), d.t_del,
                              P(a["vinf"]), P(a["robs"]), P(a["tobs"]), 42, P(a["ff"]), C.c_float(der["a0"]),
                              P(spl), P(oas))
    assert rc == 0, L.acum_last_global_error()
    ospl, ooas = O.bpm(d, aa_mode=0)
    # the drop-in takes float arguments (dTau, vInf rounded to float), so allow FP32 input rounding
    assert np.abs(oas - ooas).max() < 0.02
    assert np.abs(spl[:, :, 0] - ospl[:, :, 0]).max() < 0.02
