"""In-memory form of an ACUM-3 input deck, and its text reader/writer.

A deck is what the reference reads from its working directory:

* ``input``                       key/value settings            (io.cu:12-101)
* ``obs.dat``                     observer positions            (io.cu:106-135)
* ``surfaces/surface_<i>.dat``    per-step panel rows           (io.cu:206-333)
* ``input_BB``, ``BB_inputs/BB_surface_<i>.dat``, ``BB_inputs/BB_table_<i>.dat``
                                  broadband inputs              (io.cu:337-700)

The reader keeps the reference's semantics: the same defaults (io.cu:27-38), the same
derived quantities (``dTau``, ``dPsi`` in radians, ``vInf``; io.cu:73-83), the observer
scaling (io.cu:123-128) and the ``cn``/``cc`` division by ``(r/R)^2`` of rotating
broadband surfaces (io.cu:509-512).  All arrays hold float32 values, as the reference
stores them; the FP64 paths widen them exactly.

The writer prints every real as ``%.17g`` of its float32 value widened to double: a double
reader (the FP64 build) then parses exactly that float32 value, and a float reader rounds
the 17-digit decimal back to the same float32.  (``%.9g`` would identify the float32 for a
float reader but hand a double reader a value about 1e-9 away.)
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# 1/3-octave band centres used by the broadband model (io.cu:693-699): 1 Hz ... 10 kHz,
# then 20 kHz.  These are the standard preferred frequencies of the 1/3-octave series.
# Held as the decimal values in double (the FP64 build's view of the table); the FP32
# kernels round them to float.
BB_BANDS = np.array(
    [1.0, 1.25, 1.6, 2.0, 2.5, 3.15, 4.0, 5.0, 6.3, 8.0, 10.0, 12.5, 16.0, 20.0, 25.0, 31.5, 40.0, 50.0, 63.0,
     80.0, 100.0, 125.0, 160.0, 200.0, 250.0, 315.0, 400.0, 500.0, 630.0, 800.0, 1000.0, 1250.0, 1600.0,
     2000.0, 2500.0, 3150.0, 4000.0, 5000.0, 6300.0, 8000.0, 10000.0, 20000.0], dtype=np.float64)

# Order of the seven broadband components in BBspl[obs][band][7] (bb_core.cu:850-1034).
BB_COMPONENTS = ("total", "tbl_alpha", "tbl_suction", "tbl_pressure", "lbl_vs", "teb_vs", "tip")

INPUT_KEYS_F = ("a0", "rhoRef", "pRef", "oM", "dPsi", "Minf", "Mref", "xy_angle", "xz_angle", "CFDscale",
                "OBSscale")
INPUT_KEYS_I = ("impermeable", "nSurf", "nTime", "periodic", "lowpass", "BB_noise")


def f32(x) -> float:
    return float(np.float32(x))


def fmt(x) -> str:
    return "%.17g" % float(np.float32(x))


@dataclass
class BBSurface:
    span: float = 1.0
    omega: float = 1.0
    ccw: int = 1
    psi_offset: float = 0.0
    trip: int = 0
    rotate: tuple = (0.0, 0.0, 0.0)
    translate: tuple = (0.0, 0.0, 0.0)
    # BB_surface file
    geom: np.ndarray = None      # [nsect, 4]  r/R, y/R, z/R, c/R
    data: np.ndarray = None      # [nTime, nsect, 7] as written in the file (cn, cc not divided)
    # BB_table file
    t_sect: np.ndarray = None    # [ns_t]
    t_aoa: np.ndarray = None     # [na]
    t_mach: np.ndarray = None    # [nm]
    t_re: np.ndarray = None      # [nr]
    t_data: np.ndarray = None    # [ns_t, nm, nr, na, 7]  cl cd cm bl_u bl_l disp_u disp_l

    @property
    def nsect(self) -> int:
        return int(self.geom.shape[0])

    def data_as_read(self) -> np.ndarray:
        """bbdata after read_BB_inputs, in FP64: cn and cc divided by (r/R)^2 when omega != 0
        (io.cu:509-512).  The division is kept in double, as the FP64 build does it; the
        fixed-point angle-of-attack solve downstream is sensitive to its last bits."""
        d = self.data.astype(np.float64)
        if np.float32(self.omega) != 0:
            rr = self.geom[:, 0].astype(np.float64)
            d[:, :, 4] = d[:, :, 4] / (rr[None, :] ** 2)
            d[:, :, 5] = d[:, :, 5] / (rr[None, :] ** 2)
        return d


@dataclass
class Deck:
    a0: float = 340.0
    rhoRef: float = 1.2
    pRef: float = 0.0
    oM: float = 0.0
    nTime: int = 360
    dPsi: float = 1.0           # degrees, as in the input file
    Minf: float = 0.0
    Mref: float = 0.08
    xy_angle: float = 0.0
    xz_angle: float = 0.0
    CFDscale: float = 0.0
    OBSscale: float = 0.0
    impermeable: int = 0
    periodic: int = 1
    lowpass: int = 1
    BB_noise: int = 0
    obs_file: np.ndarray = None                 # [nObs, 3] as in obs.dat
    # each [nTime, E_i, ncol]: 8 columns for impermeable decks (x y z Cp A nx ny nz,
    # io.cu:321), 12 for permeable ones (x y z u v w P rho ds nx ny nz, io.cu:286)
    surfaces: List[np.ndarray] = field(default_factory=list)
    t_del: int = 0
    bb: List[BBSurface] = field(default_factory=list)
    name: str = ""

    # ---- sizes
    @property
    def nSurf(self) -> int:
        return len(self.surfaces)

    @property
    def ncol(self) -> int:
        """columns per surface row: 12 for a permeable deck, 8 otherwise"""
        return 12 if self.impermeable == 0 else 8

    @property
    def nObs(self) -> int:
        return int(self.obs_file.shape[0])

    @property
    def elements(self) -> List[int]:
        return [int(s.shape[1]) for s in self.surfaces]

    @property
    def E(self) -> int:
        return int(sum(self.elements))

    def tonal_evals(self) -> int:
        return self.E * self.nTime * self.nObs

    def bpm_evals(self) -> int:
        return sum(b.nsect for b in self.bb) * self.nObs * self.nTime * len(BB_BANDS)

    # ---- derived quantities exactly as read_inputs computes them (io.cu:73-83), in FP64
    def derived(self) -> dict:
        om = abs(f32(self.oM))
        dpsi_deg = f32(self.dPsi)
        a0 = f32(self.a0)
        minf = f32(self.Minf)
        xy = f32(self.xy_angle) * math.pi / 180.0
        xz = f32(self.xz_angle) * math.pi / 180.0
        return dict(
            a0=a0, rhoRef=f32(self.rhoRef), oM=om, dTau=2 * math.pi * dpsi_deg / om / 360,
            dPsi=dpsi_deg * math.pi / 180.0,
            vInf=(minf * a0 * math.cos(xy) * math.cos(xz), minf * a0 * math.sin(xy), minf * a0 * math.cos(xy) * math.sin(xz)),
            Mref=f32(self.Mref), CFDscale=f32(self.CFDscale), periodic=int(self.periodic), lowpass=int(self.lowpass))

    def observers(self) -> np.ndarray:
        """rObs after read_observers (io.cu:123-128): scaled by OBSscale, float32."""
        s = np.float32(self.OBSscale)
        return (self.obs_file.astype(np.float32) * s).astype(np.float32)

    def raw_surfaces(self) -> np.ndarray:
        """All surfaces concatenated surface-major: [sum_i nTime*E_i*ncol] float32.  When the
        surfaces are consecutive float32 views of one buffer (as the synthetic decks are
        built) that buffer is returned without a copy."""
        ss = self.surfaces
        b = ss[0].base if ss and isinstance(ss[0], np.ndarray) else None
        if (b is not None and b.dtype == np.float32 and b.ndim == 1 and b.flags.c_contiguous
                and all(s.dtype == np.float32 and s.base is b and s.flags.c_contiguous for s in ss)
                and sum(s.size for s in ss) == b.size):
            off = 0
            ok = True
            for s in ss:
                if s.__array_interface__["data"][0] != b.__array_interface__["data"][0] + 4 * off:
                    ok = False
                    break
                off += s.size
            if ok:
                return b
        return np.concatenate([s.reshape(-1) for s in ss]).astype(np.float32)

    def subset_observers(self, idx) -> "Deck":
        d = Deck(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        d.obs_file = self.obs_file[np.asarray(idx)]
        return d


# ------------------------------------------------------------------ writing

def write_deck(deck: Deck, path: str) -> None:
    os.makedirs(os.path.join(path, "surfaces"), exist_ok=True)
    with open(os.path.join(path, "input"), "w") as f:
        f.write("ACUM-3_INPUTS\n***Environmental\n")
        f.write("a0 %s\nrhoRef %s\npRef %s\n" % (fmt(deck.a0), fmt(deck.rhoRef), fmt(deck.pRef)))
        f.write("***Geometric\n")
        f.write("oM %s\nnSurf %d\nnTime %d\ndPsi %s\n" % (fmt(deck.oM), deck.nSurf, deck.nTime, fmt(deck.dPsi)))
        f.write("Minf %s\nMref %s\nxy_angle %s\nxz_angle %s\n" % (fmt(deck.Minf), fmt(deck.Mref),
                                                                   fmt(deck.xy_angle), fmt(deck.xz_angle)))
        f.write("CFDscale %s\nOBSscale %s\n" % (fmt(deck.CFDscale), fmt(deck.OBSscale)))
        f.write("***Data\nimpermeable %d\nperiodic %d\nlowpass %d\nBB_noise %d\n" % (
            deck.impermeable, deck.periodic, deck.lowpass, deck.BB_noise))
    with open(os.path.join(path, "obs.dat"), "w") as f:
        f.write("%d\n" % deck.nObs)
        for r in deck.obs_file.astype(np.float32):
            f.write("%s %s %s\n" % (fmt(r[0]), fmt(r[1]), fmt(r[2])))
    for i, s in enumerate(deck.surfaces):
        _write_rows(os.path.join(path, "surfaces", "surface_%d.dat" % (i + 1)),
                    "%d %d\n" % (s.shape[1], s.shape[0]), s.reshape(-1, s.shape[2]))
    if deck.BB_noise == 1:
        os.makedirs(os.path.join(path, "BB_inputs"), exist_ok=True)
        with open(os.path.join(path, "input_BB"), "w") as f:
            f.write("ACUM-3_Broadband_Inputs\n")
            f.write("nSurf_BB %d\nt_del %d\n" % (len(deck.bb), deck.t_del))
            for i, b in enumerate(deck.bb):
                f.write("***Surface-%d\n" % (i + 1))
                f.write("span(m) %s\nomega(rad/s) %s\nccw %d\npsi_offset %s\ntrip %d\n" % (
                    fmt(b.span), fmt(b.omega), b.ccw, fmt(b.psi_offset), b.trip))
                f.write("Initial_Position\nrotate %s %s %s\ntranslate %s %s %s\n" % (
                    tuple(fmt(v) for v in b.rotate) + tuple(fmt(v) for v in b.translate)))
        for i, b in enumerate(deck.bb):
            with open(os.path.join(path, "BB_inputs", "BB_surface_%d.dat" % (i + 1)), "w") as f:
                f.write("%d %d\n" % (b.data.shape[0], b.nsect))
                for g in b.geom.astype(np.float32):
                    f.write(" ".join(fmt(v) for v in g) + "\n")
                _write_block(f, b.data.reshape(-1, 7))
            with open(os.path.join(path, "BB_inputs", "BB_table_%d.dat" % (i + 1)), "w") as f:
                f.write('VARIABLES="alpha","mach","cl","cd","cm","bl_upper","bl_lower","disp_upper","disp_lower","Re"\n')
                ns, nm, nr, na = b.t_data.shape[:4]
                f.write("%d %d %d %d\n" % (ns, na, nm, nr))
                for j in range(ns):
                    f.write(fmt(b.t_sect[j]) + "\n")
                    rows = np.empty((nm, nr, na, 10), dtype=np.float32)
                    rows[..., 0] = b.t_aoa[None, None, :]
                    rows[..., 1] = b.t_mach[:, None, None]
                    rows[..., 2:9] = b.t_data[j]
                    rows[..., 9] = b.t_re[None, :, None]
                    _write_block(f, rows.reshape(-1, 10))


def _write_rows(fname: str, header: str, rows: np.ndarray) -> None:
    with open(fname, "w") as f:
        f.write(header)
        _write_block(f, rows)


def _write_block(f, rows: np.ndarray, chunk: int = 200000) -> None:
    rows = np.asarray(rows, dtype=np.float32)
    ncol = rows.shape[1]
    line = " ".join(["%.17g"] * ncol) + "\n"
    for a in range(0, rows.shape[0], chunk):
        blk = rows[a:a + chunk].astype(np.float64)
        f.write("".join(line % tuple(r) for r in blk.tolist()))


# ------------------------------------------------------------------ reading

def read_deck(path: str) -> Deck:
    """Reads a deck directory with the reference readers' semantics (float32 values)."""
    d = Deck()
    vals = {}
    with open(os.path.join(path, "input")) as f:
        toks = f.read().split()
    i = 0
    skip = {"ACUM-3_INPUTS", "***Environmental", "***Geometric", "***Data"}
    while i < len(toks):
        t = toks[i]
        i += 1
        if t in skip:
            continue
        if t in INPUT_KEYS_F:
            vals[t] = f32(float(toks[i])); i += 1
        elif t in INPUT_KEYS_I:
            vals[t] = int(toks[i]); i += 1
        else:
            raise ValueError("Input parameter not defined: %r" % t)
    nsurf = vals.pop("nSurf", 0)
    for k, v in vals.items():
        setattr(d, k, v)
    with open(os.path.join(path, "obs.dat")) as f:
        toks = f.read().split()
    nobs = int(toks[0])
    d.obs_file = np.array([float(x) for x in toks[1:1 + 3 * nobs]], dtype=np.float32).reshape(nobs, 3)
    for i in range(nsurf):
        fn = os.path.join(path, "surfaces", "surface_%d.dat" % (i + 1))
        with open(fn) as f:
            e, nt = (int(x) for x in f.readline().split())
            vals = _floats(f.read())
        nc = d.ncol
        d.surfaces.append(vals[: d.nTime * e * nc].reshape(d.nTime, e, nc))
    if d.BB_noise == 1:
        _read_bb(d, path)
    d.name = os.path.basename(os.path.normpath(path))
    return d


def _floats(text: str) -> np.ndarray:
    """Whitespace-separated reals, each rounded to float32 as fscanf("%f") does."""
    return np.array(text.split(), dtype=np.float64).astype(np.float32)


def _read_bb(d: Deck, path: str) -> None:
    with open(os.path.join(path, "input_BB")) as f:
        toks = f.read().split()
    nbb = d.nSurf
    d.t_del = 0
    surfs: List[BBSurface] = [BBSurface() for _ in range(max(nbb, 1))]
    i, cur = 0, 0
    while i < len(toks):
        t = toks[i]
        i += 1
        if t == "ACUM-3_Broadband_Inputs" or t == "Initial_Position":
            continue
        if t == "nSurf_BB":
            nbb = int(toks[i]); i += 1
            surfs = [BBSurface() for _ in range(nbb)]
        elif t == "t_del":
            d.t_del = int(toks[i]); i += 1
        elif t == "***Surface-%d" % (cur + 1):
            cur += 1
        elif t == "span(m)":
            surfs[cur - 1].span = f32(toks[i]); i += 1
        elif t == "omega(rad/s)":
            surfs[cur - 1].omega = f32(toks[i]); i += 1
        elif t == "ccw":
            surfs[cur - 1].ccw = int(toks[i]); i += 1
        elif t == "psi_offset":
            surfs[cur - 1].psi_offset = f32(toks[i]); i += 1
        elif t == "trip":
            surfs[cur - 1].trip = int(toks[i]); i += 1
        elif t == "rotate":
            surfs[cur - 1].rotate = tuple(f32(x) for x in toks[i:i + 3]); i += 3
        elif t == "translate":
            surfs[cur - 1].translate = tuple(f32(x) for x in toks[i:i + 3]); i += 3
            if cur == nbb:
                break
        else:
            raise ValueError("Input parameter not defined: %r" % t)
    for k, b in enumerate(surfs[:nbb]):
        with open(os.path.join(path, "BB_inputs", "BB_surface_%d.dat" % (k + 1))) as f:
            nt, ns = (int(x) for x in f.readline().split())
            vals = _floats(f.read())
        b.geom = vals[:4 * ns].reshape(ns, 4).copy()
        b.data = vals[4 * ns:4 * ns + d.nTime * ns * 7].reshape(d.nTime, ns, 7).copy()
        with open(os.path.join(path, "BB_inputs", "BB_table_%d.dat" % (k + 1))) as f:
            f.readline()
            ns_t, na, nm, nr = (int(x) for x in f.readline().split())
            toks = f.read().split()
        pos = 0
        b.t_sect = np.zeros(ns_t, np.float32)
        b.t_data = np.zeros((ns_t, nm, nr, na, 7), np.float32)
        b.t_aoa = np.zeros(na, np.float32)
        b.t_mach = np.zeros(nm, np.float32)
        b.t_re = np.zeros(nr, np.float32)
        for j in range(ns_t):
            b.t_sect[j] = f32(toks[pos]); pos += 1
            blk = np.array(toks[pos:pos + nm * nr * na * 10], dtype=np.float64).astype(np.float32)
            pos += nm * nr * na * 10
            blk = blk.reshape(nm, nr, na, 10)
            b.t_data[j] = blk[..., 2:9]
            b.t_aoa[:] = blk[-1, -1, :, 0]
            b.t_mach[:] = blk[:, -1, -1, 1]
            b.t_re[:] = blk[-1, :, -1, 9]
    d.bb = surfs[:nbb]
