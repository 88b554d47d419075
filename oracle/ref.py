"""ctypes binding of the reference's own sources compiled for the host by build_ref.sh
(oracle/_ref/libacumref_{f32,f64}.so).  TEST INFRASTRUCTURE ONLY.

The libraries exist only where the reference tree was present when `build_ref.sh` ran
(this development container); `available()` says whether they can be used.  The
reference keeps its state in globals, so each call to `load_deck` replaces the previously
loaded deck of that library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_libs = {}
_DP = C.POINTER(C.c_double)


def path(prec: str) -> str:
    return os.path.join(HERE, "_ref", "libacumref_%s.so" % prec)


def build() -> None:
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])


def available(prec: str = "f64") -> bool:
    p = path(prec)
    if not os.path.exists(p):
        return False
    try:
        lib(prec)
        return True
    except OSError:
        return False


def lib(prec: str = "f64"):
    if prec not in _libs:
        L = C.CDLL(path(prec))
        L.acumref_load.argtypes = [C.c_char_p, C.c_int]
        L.acumref_dims.argtypes = [C.POINTER(C.c_int)]
        L.acumref_surf_sizes.argtypes = [C.POINTER(C.c_int)]
        L.acumref_scalars.argtypes = [_DP]
        L.acumref_observers.argtypes = [_DP]
        L.acumref_field_sizes.argtypes = [C.POINTER(C.c_long)]
        L.acumref_fields.argtypes = [_DP, _DP, _DP, _DP]
        L.acumref_preprocess.argtypes = [C.c_int]
        L.acumref_tonal.argtypes = [C.c_int, C.c_int, _DP, _DP, _DP, C.c_int]
        L.acumref_bpm.argtypes = [C.c_int, C.c_int, _DP, _DP, C.c_int]
        L.acumref_bb_curve.argtypes = [C.c_int, _DP, _DP, C.c_int]
        L.acumref_g5comp.argtypes = [C.c_double, C.c_double]
        L.acumref_g5comp.restype = C.c_double
        L.acumref_make_periodic.argtypes = [_DP, C.c_int]
        L.acumref_lowpass.argtypes = [_DP, C.c_int]
        L.acumref_differentiate.argtypes = [_DP, _DP, C.c_double, C.c_int, C.c_int]
        L.acumref_core.argtypes = [_DP, C.c_int, C.c_int, C.c_int, _DP]
        L.acumref_bands.argtypes = [_DP]
        L.acumref_preprocess_per.argtypes = [C.c_int, C.POINTER(C.c_int), C.c_int, _DP, C.c_int, C.c_int] + \
            [_DP] * 5 + [C.c_int]
        L.acumref_preprocess_per_loaded.argtypes = [C.c_int]
        L.acumref_fields_per.argtypes = [_DP] * 5
        L.acumref_write_zero_history.argtypes = [C.c_char_p]
        _libs[prec] = L
    return _libs[prec]


def _p(a):
    return a.ctypes.data_as(_DP)


class RefDeck:
    """A deck directory loaded into one of the reference builds."""

    def __init__(self, deck_dir: str, prec: str = "f64"):
        self.L = lib(prec)
        rc = self.L.acumref_load(os.path.abspath(deck_dir).encode(), 1)
        if rc != 0:
            raise RuntimeError("acumref_load failed: %d" % rc)
        d = (C.c_int * 12)()
        self.L.acumref_dims(d)
        (self.nSurf, self.nTime, self.nObs, self.E, self.BB_noise, self.nSurf_BB, self.nf, self.t_del,
         self.impermeable, self.periodic, self.lowpass, self.nPRham) = list(d)
        s = np.zeros(15)
        self.L.acumref_scalars(_p(s))
        self.scalars = dict(zip(("a0", "rhoRef", "pRef", "oM", "dPsi", "dTau", "vx", "vy", "vz", "Minf", "Mref",
                                 "CFDscale", "OBSscale", "xy_angle", "xz_angle"), s.tolist()))
        self.preprocessed = False

    def observers(self) -> np.ndarray:
        r = np.zeros(3 * self.nObs)
        self.L.acumref_observers(_p(r))
        return r.reshape(-1, 3)

    def fields(self):
        """(Xham, Nham, Vham, PRham) reshaped [E][T][k] (AoS of variables.cu:54)."""
        n = (C.c_long * 4)()
        self.L.acumref_field_sizes(n)
        X, N, V, P = (np.zeros(int(k)) for k in n)
        self.L.acumref_fields(_p(X), _p(N), _p(V), _p(P))
        E, T = self.E, self.nTime
        return X.reshape(E, T, 4), N.reshape(E, T, 6), V.reshape(E, T, 6), P.reshape(E, T, self.nPRham)

    def permeable_fields(self):
        """A loaded permeable deck after preprocess_per (main.cu:87): (Xham, Nham, Vham,
        Uham, PRham) reshaped [E][T][k]."""
        if self.impermeable != 0:
            raise RuntimeError("not a permeable deck")
        if not self.preprocessed:
            if self.L.acumref_preprocess_per_loaded(1) != 0:
                raise RuntimeError("acumref_preprocess_per_loaded failed")
            self.preprocessed = True
        E, T = self.E, self.nTime
        out = [np.zeros(E * T * w) for w in (4, 6, 6, 6, 4)]
        self.L.acumref_fields_per(*[_p(a) for a in out])
        return tuple(a.reshape(E, T, -1) for a in out)

    def write_zero_history(self, out_dir: str) -> None:
        """pT.out, pL.out, pA.out as the reference writes them for a permeable deck."""
        rc = self.L.acumref_write_zero_history(os.path.abspath(out_dir).encode())
        if rc != 0:
            raise RuntimeError("acumref_write_zero_history failed: %d" % rc)

    def preprocess(self) -> None:
        if not self.preprocessed:
            self.L.acumref_preprocess(1)
            self.preprocessed = True

    def tonal(self, obs_range=None):
        self.preprocess()
        o0, o1 = obs_range or (0, self.nObs)
        n = o1 - o0
        pT, pL, pA = (np.zeros((self.nTime, n)) for _ in range(3))
        rc = self.L.acumref_tonal(o0, n, _p(pT), _p(pL), _p(pA), 1)
        if rc != 0:
            raise RuntimeError("acumref_tonal failed")
        return pT, pL, pA

    def bpm(self, obs_range=None):
        o0, o1 = obs_range or (0, self.nObs)
        n = o1 - o0
        spl = np.zeros((n, self.nf, 7))
        oas = np.zeros(n)
        rc = self.L.acumref_bpm(o0, n, _p(spl), _p(oas), 1)
        if rc != 0:
            raise RuntimeError("acumref_bpm failed")
        return spl, oas

    def core(self, args, trip, isect, nsect):
        out = np.zeros(self.nf * 7)
        a = np.ascontiguousarray(args, dtype=np.float64)
        self.L.acumref_core(_p(a), trip, isect, nsect, _p(out))
        return out.reshape(self.nf, 7)

    def bands(self):
        f = np.zeros(self.nf)
        self.L.acumref_bands(_p(f))
        return f


def bb_curve(which: int, x: np.ndarray, prec: str = "f64") -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib(prec).acumref_bb_curve(which, _p(x), _p(y), x.size)
    return y


def g5comp(h: float, eta: float, prec: str = "f64") -> float:
    return lib(prec).acumref_g5comp(h, eta)


def make_periodic(f, prec="f64"):
    g = np.array(f, dtype=np.float64)
    lib(prec).acumref_make_periodic(_p(g), g.size)
    return g


def lowpass(f, prec="f64"):
    g = np.array(f, dtype=np.float64)
    lib(prec).acumref_lowpass(_p(g), g.size)
    return g


def differentiate(u, dt, biased=False, prec="f64"):
    u = np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros_like(u)
    lib(prec).acumref_differentiate(_p(u), _p(du), dt, u.size, int(biased))
    return du


def preprocess_per(ne, X, N, V, U, PR, dTau, a0, rhoRef, Mref, CFDscale, periodic=1, lowpass=0,
                   prec: str = "f64"):
    """The reference's preprocess_per (preprocess.cu:8-226) on copies of the given arrays,
    [element][step][k] with the elements of all surfaces stacked (ne = elements per
    surface).  Returns the updated (X, N, V, U, PR)."""
    L = lib(prec)
    arrs = [np.array(a, dtype=np.float64, order="C") for a in (X, N, V, U, PR)]
    ne_c = (C.c_int * len(ne))(*[int(k) for k in ne])
    scal = np.array([dTau, a0, rhoRef, Mref, CFDscale], np.float64)
    rc = L.acumref_preprocess_per(len(ne), ne_c, arrs[0].shape[1], _p(scal), int(periodic), int(lowpass),
                                  *[_p(a) for a in arrs], 1)
    if rc != 0:
        raise RuntimeError("acumref_preprocess_per failed: %d" % rc)
    return tuple(arrs)
