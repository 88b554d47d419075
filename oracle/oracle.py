"""ctypes binding of oracle/acum_oracle.c (the FP64 CPU restatement of the path).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg.  `build()` compiles the C file with gcc into oracle/_build/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "acum_oracle.c")
LIB = os.path.join(HERE, "_build", "libacum_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", SRC, "-o", tmp,
                               "-lm"])
        os.replace(tmp, LIB)
    return LIB


class _Tonal(C.Structure):
    _fields_ = [("nsurf", C.c_int), ("ntime", C.c_int), ("nobs", C.c_int), ("nelem", C.POINTER(C.c_int)),
                ("a0", C.c_double), ("rho_ref", C.c_double), ("om", C.c_double), ("dpsi", C.c_double),
                ("dtau", C.c_double), ("vinf", C.c_double * 3), ("mref", C.c_double), ("cfd_scale", C.c_double),
                ("periodic", C.c_int), ("lowpass", C.c_int)]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


class _Bpm(C.Structure):
    _fields_ = [("nsurf", C.c_int), ("ntime", C.c_int), ("nobs", C.c_int), ("nf", C.c_int), ("t_del", C.c_int),
                ("dtau", C.c_double), ("a0", C.c_double), ("vinf", C.c_double * 3), ("ff", _DP),
                ("span", _DP), ("omega", _DP), ("psi_offset", _DP), ("rotate", _DP), ("translate", _DP),
                ("ccw", _IP), ("trip", _IP), ("nsect", _IP), ("xyzcR", _DP), ("bbdata", _DP),
                ("nsect_t", _IP), ("naoa_t", _IP), ("nmach_t", _IP), ("nre_t", _IP),
                ("sect_t", _DP), ("aoa_t", _DP), ("mach_t", _DP), ("re_t", _DP), ("bbdata_t", _DP),
                ("aa_mode", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.acumo_preprocess.argtypes = [C.POINTER(_Tonal), _DP, _DP]
        L.acumo_preprocess_per.argtypes = [C.c_int, C.c_int, _DP, C.c_int, C.c_int] + [_DP] * 5
        L.acumo_tonal_run.argtypes = [C.POINTER(_Tonal), _DP, _DP, C.c_int, C.c_int, _DP, _DP, _DP, C.c_int]
        L.acumo_bpm_run.argtypes = [C.POINTER(_Bpm), _DP, C.c_int, C.c_int, _DP, _DP, C.c_int]
        L.acumo_bpm_prep.argtypes = [C.POINTER(_Bpm), C.c_int, _DP, _DP, _DP, _DP]
        L.acumo_bpm_geom.argtypes = [C.POINTER(_Bpm), C.c_int, _DP, _DP]
        L.acumo_bb_curve.argtypes = [C.c_int, _DP, _DP, C.c_int]
        L.acumo_g5comp.argtypes = [C.c_double, C.c_double]
        L.acumo_g5comp.restype = C.c_double
        L.acumo_make_periodic.argtypes = [_DP, C.c_int]
        L.acumo_lowpass.argtypes = [_DP, C.c_int]
        L.acumo_differentiate.argtypes = [_DP, _DP, C.c_double, C.c_int, C.c_int]
        L.acumo_bpm_core.argtypes = [C.c_double] * 9 + [C.c_int] + [C.c_double] * 4 + [C.c_int, C.c_int, _DP,
                                                                                      C.c_int, C.c_double, _DP]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_IP)


class TonalInputs:
    """Keeps the arrays alive that the C struct points into."""

    def __init__(self, deck):
        d = deck.derived()
        self.nelem = np.array(deck.elements, dtype=np.int32)
        # widened without a float32 round trip, so float64 rows (finite-difference
        # perturbations) keep their precision
        self.raw = np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1) for x in deck.surfaces])
        self.obs = deck.observers().astype(np.float64).reshape(-1)
        s = _Tonal()
        s.nsurf, s.ntime, s.nobs = deck.nSurf, deck.nTime, deck.nObs
        s.nelem = _ip(self.nelem)
        s.a0, s.rho_ref, s.om, s.dpsi, s.dtau = d["a0"], d["rhoRef"], d["oM"], d["dPsi"], d["dTau"]
        s.vinf[0], s.vinf[1], s.vinf[2] = d["vInf"]
        s.mref, s.cfd_scale, s.periodic, s.lowpass = d["Mref"], d["CFDscale"], d["periodic"], d["lowpass"]
        self.s = s
        self.E, self.T, self.O = deck.E, deck.nTime, deck.nObs


def preprocess(deck, inputs: TonalInputs = None) -> np.ndarray:
    """fields [E][T][18] of preprocess_imper (x,y,z,ds,n,ndot,V,Vdot,P,Pdot), FP64."""
    I = inputs or TonalInputs(deck)
    out = np.zeros((I.E, I.T, 18), dtype=np.float64)
    lib().acumo_preprocess(C.byref(I.s), _p(I.raw), _p(out))
    return out


def tonal(deck, obs_range=None, nthreads: int = 0, fields: np.ndarray = None, inputs: TonalInputs = None):
    """(pT, pL, pA) each [nTime][n] for observers obs_range (default: all), FP64."""
    I = inputs or TonalInputs(deck)
    if fields is None:
        fields = preprocess(deck, I)
    o0, o1 = obs_range or (0, I.O)
    n = o1 - o0
    pT = np.zeros((I.T, n)); pL = np.zeros((I.T, n)); pA = np.zeros((I.T, n))
    nth = nthreads or min(os.cpu_count() or 1, 16)
    bad = lib().acumo_tonal_run(C.byref(I.s), _p(np.ascontiguousarray(fields)), _p(I.obs), o0, n, _p(pT), _p(pL),
                                _p(pA), nth)
    return pT, pL, pA, bad


class BpmInputs:
    def __init__(self, deck, aa_mode: int = 0):
        from acum3_periodic_gb300.deck import BB_BANDS
        d = deck.derived()
        bb = deck.bb
        self.ff = BB_BANDS.astype(np.float64)
        self.span = np.array([b.span for b in bb], np.float64)
        self.omega = np.array([b.omega for b in bb], np.float64)
        self.psi = np.array([b.psi_offset for b in bb], np.float64)
        self.rot = np.array([b.rotate for b in bb], np.float64).reshape(-1)
        self.tra = np.array([b.translate for b in bb], np.float64).reshape(-1)
        self.ccw = np.array([b.ccw for b in bb], np.int32)
        self.trip = np.array([b.trip for b in bb], np.int32)
        self.nsect = np.array([b.nsect for b in bb], np.int32)
        self.xyzcR = np.concatenate([b.geom.reshape(-1) for b in bb]).astype(np.float64)
        self.bbdata = np.concatenate([b.data_as_read().reshape(-1) for b in bb]).astype(np.float64)
        self.ns_t = np.array([b.t_data.shape[0] for b in bb], np.int32)
        self.nm_t = np.array([b.t_data.shape[1] for b in bb], np.int32)
        self.nr_t = np.array([b.t_data.shape[2] for b in bb], np.int32)
        self.na_t = np.array([b.t_data.shape[3] for b in bb], np.int32)
        self.sect_t = np.concatenate([b.t_sect for b in bb]).astype(np.float64)
        self.aoa_t = np.concatenate([b.t_aoa for b in bb]).astype(np.float64)
        self.mach_t = np.concatenate([b.t_mach for b in bb]).astype(np.float64)
        self.re_t = np.concatenate([b.t_re for b in bb]).astype(np.float64)
        self.data_t = np.concatenate([b.t_data.reshape(-1) for b in bb]).astype(np.float64)
        self.obs = deck.observers().astype(np.float64).reshape(-1)
        s = _Bpm()
        s.nsurf, s.ntime, s.nobs, s.nf, s.t_del = len(bb), deck.nTime, deck.nObs, len(self.ff), deck.t_del
        s.dtau, s.a0 = d["dTau"], d["a0"]
        s.vinf[0], s.vinf[1], s.vinf[2] = d["vInf"]
        s.ff = _p(self.ff); s.span = _p(self.span); s.omega = _p(self.omega); s.psi_offset = _p(self.psi)
        s.rotate = _p(self.rot); s.translate = _p(self.tra); s.ccw = _ip(self.ccw); s.trip = _ip(self.trip)
        s.nsect = _ip(self.nsect); s.xyzcR = _p(self.xyzcR); s.bbdata = _p(self.bbdata)
        s.nsect_t = _ip(self.ns_t); s.naoa_t = _ip(self.na_t); s.nmach_t = _ip(self.nm_t); s.nre_t = _ip(self.nr_t)
        s.sect_t = _p(self.sect_t); s.aoa_t = _p(self.aoa_t); s.mach_t = _p(self.mach_t); s.re_t = _p(self.re_t)
        s.bbdata_t = _p(self.data_t)
        s.aa_mode = aa_mode
        self.s = s
        self.O = deck.nObs
        self.nf = len(self.ff)


def bpm(deck, aa_mode: int = 0, obs_range=None, nthreads: int = 0, inputs: BpmInputs = None):
    """(BBspl [n][42][7], BBoaspl [n]) in dB for observers obs_range, FP64, seeded with
    -100 dB as the reference driver does."""
    I = inputs or BpmInputs(deck, aa_mode)
    o0, o1 = obs_range or (0, I.O)
    n = o1 - o0
    spl = np.full((n, I.nf, 7), -100.0)
    oas = np.full(n, -100.0)
    nth = nthreads or min(os.cpu_count() or 1, 16)
    lib().acumo_bpm_run(C.byref(I.s), _p(I.obs), o0, n, _p(spl), _p(oas), nth)
    return spl, oas


def bpm_prep(deck, surface: int, aa_mode: int = 0):
    I = BpmInputs(deck, aa_mode)
    ns = deck.bb[surface].nsect
    T = deck.nTime
    u = np.zeros((ns, T)); al = np.zeros((ns, T)); cla = np.zeros((ns, T)); bl = np.zeros((ns, T, 4))
    lib().acumo_bpm_prep(C.byref(I.s), surface, _p(u), _p(al), _p(cla), _p(bl))
    return u, al, cla, bl


def bpm_geom(deck, surface: int):
    """quarter-chord and trailing-edge positions [sect][step][3] of one BB surface."""
    I = BpmInputs(deck, 0)
    ns = deck.bb[surface].nsect
    xyz = np.zeros((ns, deck.nTime, 3)); xyzt = np.zeros((ns, deck.nTime, 3))
    lib().acumo_bpm_geom(C.byref(I.s), surface, _p(xyz), _p(xyzt))
    return xyz, xyzt


def bb_curve(which: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().acumo_bb_curve(which, _p(x), _p(y), x.size)
    return y


def g5comp(h: float, eta: float) -> float:
    return lib().acumo_g5comp(h, eta)


def make_periodic(f: np.ndarray) -> np.ndarray:
    g = np.array(f, dtype=np.float64)
    lib().acumo_make_periodic(_p(g), g.size)
    return g


def lowpass(f: np.ndarray) -> np.ndarray:
    g = np.array(f, dtype=np.float64)
    lib().acumo_lowpass(_p(g), g.size)
    return g


def differentiate(u: np.ndarray, dt: float, biased: bool = False) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    du = np.zeros_like(u)
    lib().acumo_differentiate(_p(u), _p(du), dt, u.size, int(biased))
    return du


def preprocess_per(X, N, U, PR, dTau, a0, rhoRef, Mref, CFDscale, periodic=1, lowpass_=0):
    """preprocess_per (preprocess.cu:8-226), the permeable surfaces' preprocessing, in FP64
    (acumo_preprocess_per in acum_oracle.c).

    Inputs are one element's series stacked as [element][step][k] (AoS of variables.cu:
    11-42): X (x, y, z, ds), N (n, ndot), U (u, udot), PR (P, Pdot, rho, rhodot); only the
    columns the reader fills (io.cu:286) are read.  Returns new arrays (X, N, V, U, PR):

    * scaling (preprocess.cu:50-68): x by CFDscale, ds by CFDscale^2, rho by rhoRef, u by
      a0, P by 0.5 rhoRef Mref^2 a0^2;
    * optional lowpass of rho, u, P (preprocess.cu:113-137): twice median3 + Gaussian,
      no make_periodic (commented out in the reference, preprocess.cu:105-109);
    * d/dtau of rho, u, P periodic or end-biased (preprocess.cu:150-163), of n periodic
      (166-168); V = d x/dtau and Vdot = d V/dtau, both periodic (172-180).
    """
    X, N, U, PR = (np.array(a, dtype=np.float64, order="C") for a in (X, N, U, PR))
    V = np.zeros(N.shape, np.float64)
    scal = np.array([dTau, a0, rhoRef, Mref, CFDscale], np.float64)
    lib().acumo_preprocess_per(X.shape[0], X.shape[1], _p(scal), int(periodic), int(lowpass_), _p(X), _p(N), _p(V),
                               _p(U), _p(PR))
    return X, N, V, U, PR
