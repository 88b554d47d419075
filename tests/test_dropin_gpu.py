"""The reference-shaped drop-ins on the GPU: acum_find_pressure_time_history (FP32 arrays,
mixed kernel), acum_find_pressure_time_history_f64 (FP64 arrays, plain kernel) and
acum_preprocess_imper, called with the reference's AoS arrays (device memory for the
kernel entry points, as main.cu:156-236 passes them) and checked against the oracle."""
import ctypes as C

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from oracle import oracle as O

from metrics import oaspl_db, per_bin_rel, per_bin_rms

pytestmark = pytest.mark.gpu


def aos_arrays(deck, fields, dtype):
    """Xham/Nham/Vham/PRham and the XPtr/NPtr/VPtr/PRPtr/E arrays of variables.cu:54."""
    T = deck.nTime
    ne = deck.elements
    X = np.ascontiguousarray(fields[:, :, 0:4], dtype=dtype)
    N = np.ascontiguousarray(fields[:, :, 4:10], dtype=dtype)
    V = np.ascontiguousarray(fields[:, :, 10:16], dtype=dtype)
    P = np.ascontiguousarray(fields[:, :, 16:18], dtype=dtype)
    off = np.cumsum([0] + ne[:-1])
    ptr = {k: np.array(off * k * T, dtype=np.int32) for k in (4, 6, 2)}
    return X, N, V, P, ptr[4], ptr[6], ptr[6].copy(), ptr[2], np.array(ne, dtype=np.int32)


def call_dropin(fn, deck, fields, dtype, torch, tobs=None):
    """Calls a reference-shaped tonal entry point; `tobs` replaces the grid t * dPsi."""
    der = deck.derived()
    T, Ob = deck.nTime, deck.nObs
    X, N, V, P, XP, NP_, VP, PP, E = aos_arrays(deck, fields, dtype)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tX, tN, tV, tP = dev(X), dev(N), dev(V), dev(P)
    tXP, tNP, tVP, tPP, tE = dev(XP), dev(NP_), dev(VP), dev(PP), dev(E)
    robs = dev(np.asarray(deck.observers(), dtype=dtype))
    if tobs is None:
        tobs = (np.arange(T, dtype=dtype) * dtype(der["dPsi"])).astype(dtype)
    tobs = dev(np.asarray(tobs, dtype=dtype))
    vinf = dev(np.asarray(der["vInf"], dtype=dtype))
    z = lambda: torch.zeros((T, Ob), dtype=torch.float64 if dtype == np.float64 else torch.float32, device="cuda")
    pT, pL, pA = z(), z(), z()
    p = lambda t: C.c_void_p(t.data_ptr())
    R = C.c_double if dtype == np.float64 else C.c_float
    rc = fn(p(robs), p(tobs), p(pT), p(pL), p(pA), p(tX), p(tN), p(tV), p(tP), deck.nSurf, p(tXP), p(tNP), p(tVP),
            p(tPP), p(tE), Ob, T, R(der["dPsi"]), R(der["dTau"]), R(der["a0"]), R(der["rhoRef"]), p(vinf),
            R(der["oM"]), None)
    torch.cuda.synchronize()
    return rc, pT.cpu().numpy().astype(np.float64), pL.cpu().numpy().astype(np.float64), \
        pA.cpu().numpy().astype(np.float64)


@pytest.fixture(scope="module")
def deck_and_ref():
    d = synth.config_deck(1, replicate=70, scale=dict(n_span=4, n_chord_side=3, ntime=50, nobs=11, bb_nsect=4,
                                                      bb_small=True, n_bb=1))
    f = O.preprocess(d)
    oT, oL, oA, bad = O.tonal(d, fields=f)
    return d, f, oA


def test_find_pressure_time_history_f64(deck_and_ref):
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    d, f, oA = deck_and_ref
    rc, pT, pL, pA = call_dropin(native.lib().acum_find_pressure_time_history_f64, d, f, np.float64, torch)
    assert rc == 0, native.lib().acum_last_global_error()
    assert per_bin_rel(pA, oA).max() < 1e-10


def test_find_pressure_time_history_mixed_accumulates(deck_and_ref):
    torch = pytest.importorskip("torch")
    from acum3_periodic_gb300 import native
    d, f, oA = deck_and_ref
    fn = native.lib().acum_find_pressure_time_history
    rc, pT, pL, pA = call_dropin(fn, d, f, np.float32, torch)
    assert rc == 0, native.lib().acum_last_global_error()
    # inputs rounded to float32 (as the reference stores them): per-bin error vs the FP64
    # oracle within the mixed tolerance, OASPL well inside 0.05 dB
    assert per_bin_rms(pA, oA).max() < 1e-3
    assert np.abs(oaspl_db(pA) - oaspl_db(oA)).max() < 0.05


def test_preprocess_imper_dropin():
    from acum3_periodic_gb300 import native
    d = synth.config_deck(3, replicate=71, scale=dict(n_span=3, n_chord_side=2, ntime=40, nobs=3))
    d.lowpass = 1
    f = O.preprocess(d)
    T = d.nTime
    raw = np.concatenate([s.transpose(1, 0, 2) for s in d.surfaces], axis=0)  # [E][T][8]
    X = np.ascontiguousarray(np.concatenate([raw[:, :, 0:3], raw[:, :, 4:5]], axis=2), dtype=np.float32)
    N = np.zeros((d.E, T, 6), np.float32)
    N[:, :, 0:3] = raw[:, :, 5:8]
    V = np.zeros((d.E, T, 6), np.float32)
    P = np.zeros((d.E, T, 2), np.float32)
    P[:, :, 0] = raw[:, :, 3]
    off = np.cumsum([0] + d.elements[:-1])
    XP, NP_, PP = (np.array(off * k * T, np.int32) for k in (4, 6, 2))
    der = d.derived()
    E = np.array(d.elements, np.int32)
    fp = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = native.lib().acum_preprocess_imper(fp(X), fp(N), fp(V), fp(P), d.nSurf, fp(XP), fp(NP_), fp(NP_.copy()),
                                            fp(PP), fp(E), T, C.c_float(der["dTau"]), C.c_float(der["a0"]),
                                            C.c_float(der["rhoRef"]), C.c_float(der["Mref"]),
                                            C.c_float(der["CFDscale"]), d.periodic, d.lowpass)
    assert rc == 0, native.lib().acum_last_global_error()
    # float storage of the results; the step size arrives as float, as the reference passes it
    np.testing.assert_allclose(X[:, :, :3], f[:, :, 0:3], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(P[:, :, 0], f[:, :, 16], rtol=1e-5, atol=1e-5 * np.abs(f[:, :, 16]).max())
    np.testing.assert_allclose(V[:, :, 0:3], f[:, :, 10:13], rtol=1e-5, atol=1e-5 * np.abs(f[:, :, 10:13]).max())
    np.testing.assert_allclose(V[:, :, 3:6], f[:, :, 13:16], rtol=1e-4, atol=1e-4 * np.abs(f[:, :, 13:16]).max())
