"""ctypes binding of libacum.so (include/acum.h).

The library is built in-tree by `acum3_periodic_gb300.build.build()`.  Loading fails
loudly (RuntimeError) if it is missing or if no CUDA device is present: there is no CPU
fallback for any of these calls.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

PLAIN_FP64 = 0
MIXED = 1

DEVERR_DISC = 0x1
DEVERR_ORDER = 0x2
DEVERR_NONFINITE = 0x4
DEVERR_TIMEOUT = 0x8

ERRORS = {-1: "ACUM_ERR_INVALID", -2: "ACUM_ERR_IO", -3: "ACUM_ERR_CUDA", -4: "ACUM_ERR_NOMEM",
          -5: "ACUM_ERR_STATE", -6: "ACUM_ERR_TIMEOUT", -7: "ACUM_ERR_GEOMETRY", -8: "ACUM_ERR_UNSUPPORTED"}

_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int)


class AcumError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Inputs(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("a0", "rhoRef", "pRef", "oM", "dPsi", "Minf", "Mref", "xy_angle",
                                          "xz_angle", "CFDscale", "OBSscale")] + \
               [(k, C.c_int) for k in ("nTime", "impermeable", "periodic", "lowpass", "BB_noise")]


class BBDesc(C.Structure):
    _fields_ = [("nsurf", C.c_int), ("t_del", C.c_int),
                ("span", _DP), ("omega", _DP), ("psi_offset", _DP), ("rotate", _DP), ("translate", _DP),
                ("ccw", _IP), ("trip", _IP), ("nsect", _IP), ("geom", _FP), ("data", _FP),
                ("ns_t", _IP), ("na_t", _IP), ("nm_t", _IP), ("nr_t", _IP),
                ("sect_t", _FP), ("aoa_t", _FP), ("mach_t", _FP), ("re_t", _FP), ("table", _FP)]


_lib = None

# every symbol of include/acum.h with its ctypes signature (restype, argtypes)
SIGNATURES = {
    "acum_version": (C.c_int, []),
    "acum_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "acum_destroy": (C.c_int, [C.c_void_p]),
    "acum_last_error": (C.c_char_p, [C.c_void_p]),
    "acum_last_global_error": (C.c_char_p, []),
    "acum_load_deck": (C.c_int, [C.c_void_p, C.c_char_p]),
    "acum_set_deck": (C.c_int, [C.c_void_p, C.POINTER(Inputs), C.c_int, _FP, C.c_int, _IP, C.c_void_p, C.c_int]),
    "acum_update_surfaces": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "acum_set_bb": (C.c_int, [C.c_void_p, C.POINTER(BBDesc)]),
    "acum_get_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "acum_preprocess": (C.c_int, [C.c_void_p]),
    "acum_get_fields": (C.c_int, [C.c_void_p, _DP]),
    "acum_get_permeable_fields": (C.c_int, [C.c_void_p, _DP, _DP, _DP, _DP, _DP]),
    "acum_tonal": (C.c_int, [C.c_void_p, C.c_int, _DP, _DP, _DP]),
    "acum_tonal_from_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "acum_tonal_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "acum_surfaces_device_ptr": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "acum_mark_surfaces_changed": (C.c_int, [C.c_void_p]),
    "acum_sync": (C.c_int, [C.c_void_p]),
    "acum_tonal_from_host_async": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "acum_selftest_wait": (C.c_int, [C.c_int, C.c_double, C.c_int, _IP, _DP]),
    "acum_selftest_tmem": (C.c_int, [C.c_int, _IP, C.c_void_p]),
    "acum_read_deck_sizes": (C.c_int, [C.c_char_p, C.POINTER(C.c_longlong)]),
    "acum_write_surface_cache": (C.c_int, [C.c_char_p]),
    "acum_last_plan": (C.c_int, [C.c_void_p, _IP]),
    "acum_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "acum_bpm": (C.c_int, [C.c_void_p, C.c_int, _DP, _DP]),
    "acum_write_outputs": (C.c_int, [C.c_void_p, C.c_char_p]),
    "acum_tonal_adjoint": (C.c_int, [C.c_void_p, C.c_int, _DP, _DP, _DP, _DP, _DP]),
    "acum_device_error_word": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_int]),
    "acum_last_timing": (C.c_int, [C.c_void_p, C.c_int, _DP, C.POINTER(C.c_longlong)]),
    "acum_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "acum_set_obs_per_warp": (C.c_int, [C.c_void_p, C.c_int]),
    "acum_set_tensor_memory": (C.c_int, [C.c_void_p, C.c_int]),
    "acum_set_ring": (C.c_int, [C.c_void_p, C.c_int]),
    "acum_last_plan_ring": (C.c_int, [C.c_void_p, _IP]),
    "acum_measure_peak": (C.c_int, [C.c_int, C.c_int, _DP]),
    "acum_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "acum_host_free": (C.c_int, [C.c_void_p]),
    "acum_find_pressure_time_history": (C.c_int, [C.c_void_p] * 9 + [C.c_int] + [C.c_void_p] * 5 +
                                        [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p,
                                         C.c_float, C.c_void_p]),
    "acum_find_pressure_time_history_f64": (C.c_int, [C.c_void_p] * 9 + [C.c_int] + [C.c_void_p] * 5 +
                                            [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                             C.c_void_p, C.c_double, C.c_void_p]),
    "acum_find_pressure_time_history_noalloc": (C.c_int, [C.c_void_p] * 9 + [C.c_int] + [C.c_void_p] * 5 +
                                                [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                                 C.c_void_p, C.c_float, C.c_void_p]),
    "acum_noalloc_last_error": (C.c_char_p, []),
    "acum_preprocess_imper": (C.c_int, [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 5 +
                              [C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int]),
    "acum_preprocess_per": (C.c_int, [C.c_void_p] * 5 + [C.c_int] + [C.c_void_p] * 6 +
                            [C.c_int] + [C.c_float] * 5 + [C.c_int, C.c_int]),
    "acum_preprocess_per_f64": (C.c_int, [C.c_void_p] * 5 + [C.c_int] + [C.c_void_p] * 6 +
                                [C.c_int] + [C.c_double] * 5 + [C.c_int, C.c_int]),
    "acum_preprocess_per_device": (C.c_int, [C.c_void_p] * 5 + [C.c_int, C.c_int] + [C.c_void_p] * 6 +
                                   [C.c_int] + [C.c_double] * 5 + [C.c_int, C.c_int, C.c_void_p]),
    "acum_find_bb_noise": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_float] + [C.c_void_p] * 26 +
                           [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_float,
                            C.c_void_p, C.c_void_p]),
    "acum_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "acum_batch_destroy": (C.c_int, [C.c_void_p]),
    "acum_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "acum_batch_add": (C.c_int, [C.c_void_p, C.POINTER(Inputs), C.c_int, _FP, C.c_int, _IP, C.c_void_p, _IP]),
    "acum_batch_prepare": (C.c_int, [C.c_void_p]),
    "acum_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "acum_batch_result": (C.c_int, [C.c_void_p, C.c_int, _DP]),
    "acum_batch_timing": (C.c_int, [C.c_void_p, _DP, C.POINTER(C.c_longlong)]),
    "acum_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "acum_batch_get_tile": (C.c_int, [C.c_void_p, _IP, _IP, _IP]),
    "acum_batch_set_tile2": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "acum_batch_get_obs_per_warp": (C.c_int, [C.c_void_p, _IP]),
    "acum_batch_count": (C.c_int, [C.c_void_p, _IP]),
    "acum_batch_case_timing": (C.c_int, [C.c_void_p, C.c_int, _DP]),
    "acum_batch_autotune": (C.c_int, [C.c_void_p, C.c_int, _DP]),
}


def lib(build_if_missing: bool = True):
    """The loaded library.  Builds it in-tree first if it is not there."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            if not build_if_missing:
                raise RuntimeError("libacum.so is not built (%s); run __graft_entry__.build()" % LIB)
            from .build import build
            build()
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, t=_DP):
    return a.ctypes.data_as(t)


def inputs_of(deck) -> Inputs:
    s = Inputs()
    for k in ("a0", "rhoRef", "pRef", "oM", "dPsi", "Minf", "Mref", "xy_angle", "xz_angle", "CFDscale",
              "OBSscale"):
        setattr(s, k, float(np.float32(getattr(deck, k))))
    s.nTime, s.impermeable, s.periodic, s.lowpass, s.BB_noise = (
        deck.nTime, deck.impermeable, deck.periodic, deck.lowpass, deck.BB_noise)
    return s


class Context:
    """One acum_ctx on one GPU."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = C.c_void_p()
        rc = self.L.acum_create(C.byref(h), device)
        if rc != 0:
            raise AcumError(rc, self.L.acum_last_global_error().decode())
        self.h = h
        self.T = self.O = self.E = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.acum_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise AcumError(rc, self.L.acum_last_error(self.h).decode())

    def _sizes(self):
        s = (C.c_longlong * 6)()
        self._ck(self.L.acum_get_sizes(self.h, s))
        self.nsurf, self.T, self.O, self.E, self.nbb, self.has_bb = (int(v) for v in s)

    # ---- deck
    def set_deck(self, deck, bb: bool = True):
        obs = np.ascontiguousarray(deck.obs_file, dtype=np.float32)
        ne = np.array(deck.elements, dtype=np.int32)
        if any(s.shape[2] != deck.ncol for s in deck.surfaces):
            raise ValueError("surface rows must have %d columns for impermeable = %d" % (deck.ncol, deck.impermeable))
        raw = deck.raw_surfaces()
        inp = inputs_of(deck)
        self._ck(self.L.acum_set_deck(self.h, C.byref(inp), deck.nObs, _p(obs, _FP), deck.nSurf, _p(ne, _IP),
                                      raw.ctypes.data_as(C.c_void_p), 0))
        self._sizes()
        if bb and deck.BB_noise == 1:
            self.set_bb(deck)
        return self

    def set_deck_raw_device(self, deck, raw_dev_ptr: int):
        obs = np.ascontiguousarray(deck.obs_file, dtype=np.float32)
        ne = np.array(deck.elements, dtype=np.int32)
        inp = inputs_of(deck)
        self._ck(self.L.acum_set_deck(self.h, C.byref(inp), deck.nObs, _p(obs, _FP), deck.nSurf, _p(ne, _IP),
                                      C.c_void_p(raw_dev_ptr), 1))
        self._sizes()
        return self

    def load_deck(self, path: str):
        self._ck(self.L.acum_load_deck(self.h, os.fsencode(path)))
        self._sizes()
        return self

    def set_bb(self, deck):
        bb = deck.bb
        self._bb_keep = k = dict(
            span=np.array([b.span for b in bb], np.float64), omega=np.array([b.omega for b in bb], np.float64),
            psi=np.array([b.psi_offset for b in bb], np.float64),
            rot=np.array([b.rotate for b in bb], np.float64).reshape(-1),
            tra=np.array([b.translate for b in bb], np.float64).reshape(-1),
            ccw=np.array([b.ccw for b in bb], np.int32), trip=np.array([b.trip for b in bb], np.int32),
            nsect=np.array([b.nsect for b in bb], np.int32),
            geom=np.concatenate([b.geom.reshape(-1) for b in bb]).astype(np.float32),
            data=np.concatenate([b.data.reshape(-1) for b in bb]).astype(np.float32),
            ns=np.array([b.t_data.shape[0] for b in bb], np.int32),
            na=np.array([b.t_data.shape[3] for b in bb], np.int32),
            nm=np.array([b.t_data.shape[1] for b in bb], np.int32),
            nr=np.array([b.t_data.shape[2] for b in bb], np.int32),
            sect=np.concatenate([b.t_sect for b in bb]).astype(np.float32),
            aoa=np.concatenate([b.t_aoa for b in bb]).astype(np.float32),
            mach=np.concatenate([b.t_mach for b in bb]).astype(np.float32),
            re=np.concatenate([b.t_re for b in bb]).astype(np.float32),
            table=np.concatenate([b.t_data.reshape(-1) for b in bb]).astype(np.float32))
        d = BBDesc()
        d.nsurf, d.t_del = len(bb), deck.t_del
        d.span, d.omega, d.psi_offset = _p(k["span"]), _p(k["omega"]), _p(k["psi"])
        d.rotate, d.translate = _p(k["rot"]), _p(k["tra"])
        d.ccw, d.trip, d.nsect = _p(k["ccw"], _IP), _p(k["trip"], _IP), _p(k["nsect"], _IP)
        d.geom, d.data = _p(k["geom"], _FP), _p(k["data"], _FP)
        d.ns_t, d.na_t, d.nm_t, d.nr_t = (_p(k[x], _IP) for x in ("ns", "na", "nm", "nr"))
        d.sect_t, d.aoa_t, d.mach_t, d.re_t, d.table = (_p(k[x], _FP) for x in ("sect", "aoa", "mach", "re",
                                                                                  "table"))
        self._ck(self.L.acum_set_bb(self.h, C.byref(d)))
        self._sizes()

    # ---- runs
    def preprocess(self):
        self._ck(self.L.acum_preprocess(self.h))

    def fields(self) -> np.ndarray:
        out = np.zeros((self.E, self.T, 18))
        self._ck(self.L.acum_get_fields(self.h, _p(out)))
        return out

    def permeable_fields(self):
        """A permeable deck's preprocessed AoS arrays (X, N, V, U, PR), each [E][T][width],
        FP64 (acum_get_permeable_fields)."""
        out = [np.zeros((self.E, self.T, w)) for w in (4, 6, 6, 6, 4)]
        self._ck(self.L.acum_get_permeable_fields(self.h, *(_p(a) for a in out)))
        return tuple(out)

    def tonal(self, precision: int = MIXED):
        pT, pL, pA = (np.zeros((self.T, self.O)) for _ in range(3))
        self._ck(self.L.acum_tonal(self.h, precision, _p(pT), _p(pL), _p(pA)))
        return pT, pL, pA

    def tonal_from_host(self, precision: int, raw_ptr: int, pA_ptr: int):
        self._ck(self.L.acum_tonal_from_host(self.h, precision, C.c_void_p(raw_ptr), C.c_void_p(pA_ptr)))

    def tonal_from_host_async(self, precision: int, raw_ptr: int, pA_ptr: int):
        self._ck(self.L.acum_tonal_from_host_async(self.h, precision, C.c_void_p(raw_ptr), C.c_void_p(pA_ptr)))

    def tonal_device(self, precision: int, pT_ptr: int, pL_ptr: int, pA_ptr: int):
        self._ck(self.L.acum_tonal_device(self.h, precision, C.c_void_p(pT_ptr), C.c_void_p(pL_ptr),
                                          C.c_void_p(pA_ptr)))

    def mark_surfaces_changed(self):
        self._ck(self.L.acum_mark_surfaces_changed(self.h))

    def sync(self):
        self._ck(self.L.acum_sync(self.h))

    def stream_ptr(self) -> int:
        """The cudaStream_t the context issues its runs on, as an integer."""
        p = C.c_void_p()
        self._ck(self.L.acum_stream(self.h, C.byref(p)))
        return int(p.value or 0)

    def bpm(self, aa_mode: int = 0):
        spl = np.zeros((self.O, 42, 7))
        oas = np.zeros(self.O)
        self._ck(self.L.acum_bpm(self.h, aa_mode, _p(spl), _p(oas)))
        return spl, oas

    def adjoint(self, precision: int = PLAIN_FP64, dJ_dpA: np.ndarray = None):
        J = np.zeros(1)
        gcp = np.zeros((self.E, self.T))
        gx = np.zeros((self.E, self.T, 3))
        gn = np.zeros((self.E, self.T, 3))
        dj = None if dJ_dpA is None else np.ascontiguousarray(dJ_dpA, dtype=np.float64)
        self._ck(self.L.acum_tonal_adjoint(self.h, precision, None if dj is None else _p(dj), _p(J), _p(gcp),
                                           _p(gx), _p(gn)))
        return float(J[0]), gcp, gx, gn

    def write_outputs(self, path: str):
        self._ck(self.L.acum_write_outputs(self.h, os.fsencode(path)))

    def set_tile(self, obs_per_block=0, elems_per_stage=0, items_per_sm=0, obs_per_warp=0, tensor_memory=0,
                 whole_rows=0):
        self._ck(self.L.acum_set_tile(self.h, obs_per_block, elems_per_stage, items_per_sm))
        self._ck(self.L.acum_set_obs_per_warp(self.h, obs_per_warp))
        self._ck(self.L.acum_set_tensor_memory(self.h, tensor_memory))
        self._ck(self.L.acum_set_ring(self.h, whole_rows))

    def last_plan(self) -> dict:
        """The last tonal plan; for the mixed form also `ring_slots` (0: whole rows only),
        `wide_ring_slots` and `wide2_ring_slots` (the 1024- and 2048-slot wide rings; 0:
        not planned) and `ring_used` (the slots of the ring whose kernel did the work, 0:
        the whole-row kernel)."""
        v = (C.c_int * 8)()
        self._ck(self.L.acum_last_plan(self.h, v))
        keys = ("obs_per_block", "elems_per_stage", "stages", "elems_per_item", "element_chunks", "work_items",
                "obs_per_warp", "tensor_memory")
        out = dict(zip(keys, (int(x) for x in v)))
        r = (C.c_int * 11)()
        self._ck(self.L.acum_last_plan_ring(self.h, r))
        out.update(ring_slots=int(r[0]), rows_obs_per_block=int(r[1]), rows_elems_per_stage=int(r[2]),
                   rows_stages=int(r[3]), ring_used=int(r[4]), wide_ring_slots=int(r[5]),
                   wide_obs_per_block=int(r[6]), wide_stages=int(r[7]), wide2_ring_slots=int(r[8]),
                   wide2_obs_per_block=int(r[9]), wide2_stages=int(r[10]))
        return out

    def timing(self, which: int):
        ms = C.c_double()
        n = C.c_longlong()
        self._ck(self.L.acum_last_timing(self.h, which, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def error_word(self, reset: bool = False) -> int:
        w = C.c_uint32()
        self._ck(self.L.acum_device_error_word(self.h, C.byref(w), int(reset)))
        return w.value


def measure_peak(device: int, which: int) -> float:
    v = C.c_double()
    rc = lib().acum_measure_peak(device, which, C.byref(v))
    if rc != 0:
        raise AcumError(rc, "acum_measure_peak failed")
    return v.value


class Batch:
    """One acum_batch on one GPU: many decks solved by one persistent launch."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = C.c_void_p()
        rc = self.L.acum_batch_create(C.byref(h), device)
        if rc != 0:
            raise AcumError(rc, self.L.acum_last_global_error().decode())
        self.h = h
        self.shapes = []  # (nTime, nObs, evals) per case

    def close(self):
        if getattr(self, "h", None):
            self.L.acum_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            raise AcumError(rc, self.L.acum_batch_last_error(self.h).decode())

    def add(self, deck) -> int:
        """Uploads and preprocesses one deck; its rows are not kept on the device."""
        obs = np.ascontiguousarray(deck.obs_file, dtype=np.float32)
        ne = np.array([s.shape[1] for s in deck.surfaces], np.int32)
        raw = np.ascontiguousarray(deck.raw_surfaces(), dtype=np.float32)
        cid = C.c_int()
        inp = inputs_of(deck)
        self._ck(self.L.acum_batch_add(self.h, C.byref(inp), obs.shape[0], _p(obs, _FP), len(ne), _p(ne, _IP),
                                       raw.ctypes.data_as(C.c_void_p), C.byref(cid)))
        self.shapes.append((deck.nTime, deck.nObs, deck.tonal_evals()))
        return cid.value

    def count(self) -> int:
        n = C.c_int()
        self._ck(self.L.acum_batch_count(self.h, C.byref(n)))
        return n.value

    def prepare(self):
        self._ck(self.L.acum_batch_prepare(self.h))

    def set_tile(self, obs_per_block=0, elems_per_stage=0, items_per_sm=0, obs_per_warp=1):
        self._ck(self.L.acum_batch_set_tile2(self.h, obs_per_block, elems_per_stage, items_per_sm, obs_per_warp))

    def obs_per_warp(self) -> int:
        v = C.c_int()
        self._ck(self.L.acum_batch_get_obs_per_warp(self.h, C.byref(v)))
        return v.value

    def tile(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._ck(self.L.acum_batch_get_tile(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, probe_per_sm: int = 0) -> float:
        """Picks the tile shape; returns the predicted batch time in ms."""
        ms = C.c_double()
        self._ck(self.L.acum_batch_autotune(self.h, probe_per_sm, C.byref(ms)))
        return ms.value

    def run(self, mode: int = 2, precision: int = MIXED):
        self._ck(self.L.acum_batch_run(self.h, precision, mode))

    def result(self, case: int) -> np.ndarray:
        if not 0 <= case < len(self.shapes):
            raise AcumError(-1, "bad case index %d" % case)
        T, O, _ = self.shapes[case]
        out = np.empty((T, O), np.float64)
        self._ck(self.L.acum_batch_result(self.h, case, _p(out)))
        return out

    def timing(self):
        ms, n = C.c_double(), C.c_longlong()
        self._ck(self.L.acum_batch_timing(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def case_ms(self, case: int) -> float:
        ms = C.c_double()
        self._ck(self.L.acum_batch_case_timing(self.h, case, C.byref(ms)))
        return ms.value


def selftest_wait(device: int, limit_s: float, arrive: bool):
    """(timed_out, waited_s) of one bounded barrier wait on the device."""
    to, ws = C.c_int(), C.c_double()
    rc = lib().acum_selftest_wait(device, limit_s, 1 if arrive else 0, C.byref(to), C.byref(ws))
    if rc != 0:
        raise AcumError(rc, "acum_selftest_wait failed")
    return bool(to.value), ws.value


def selftest_tmem(device: int = 0):
    """(mismatching words, readback [4][32][40]) of the tensor-memory copy self-test."""
    mis = C.c_int()
    rb = np.zeros((4, 32, 40), np.uint32)
    rc = lib().acum_selftest_tmem(device, C.byref(mis), rb.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise AcumError(rc, "acum_selftest_tmem failed")
    return mis.value, rb


def preprocess_per(ne, X, N, V, U, PR, dTau, a0, rhoRef, Mref, CFDscale, periodic=1, lowpass=0,
                   dtype=np.float64):
    """preprocess_per (preprocess.cu:8-226) on the GPU through acum_preprocess_per(_f64).

    X [E][T][4], N, V, U [E][T][6], PR [E][T][4]: the reference's AoS rows with the
    elements of all surfaces stacked (ne = elements per surface).  Works on copies in
    `dtype` (float32: the FP32 storage form, float64: the FP64 build's) and returns the
    updated (X, N, V, U, PR)."""
    arrs = [np.array(a, dtype=dtype, order="C") for a in (X, N, V, U, PR)]
    T = arrs[0].shape[1]
    ne = np.asarray(ne, np.int32)
    off = np.concatenate([[0], np.cumsum(ne)[:-1]]).astype(np.int64)
    ptrs = [np.ascontiguousarray(off * T * w, dtype=np.int32) for w in (4, 6, 6, 6, 4)]
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    fn = lib().acum_preprocess_per_f64 if dtype == np.float64 else lib().acum_preprocess_per
    rc = fn(*[vp(a) for a in arrs], len(ne), *[vp(q) for q in ptrs], vp(ne), T, dTau, a0, rhoRef, Mref, CFDscale,
            int(periodic), int(lowpass))
    if rc != 0:
        raise AcumError(rc, lib().acum_last_global_error().decode())
    return tuple(arrs)


class PinnedBuffer:
    """Page-locked host memory from acum_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype):
        self.L = lib()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        rc = self.L.acum_host_alloc(C.byref(p), max(n, 1))
        if rc != 0:
            raise AcumError(rc, self.L.acum_last_global_error().decode())
        self.ptr = p.value
        buf = (C.c_char * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def close(self):
        if self.ptr:
            self.array = None
            self.L.acum_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
