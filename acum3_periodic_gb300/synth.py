"""Seeded synthetic rotor decks for the five workloads of this path.

No public dataset is involved: every deck is built from a seed.  The random numbers come
from a counter-based splitmix64 hash evaluated with numpy integer arithmetic, so a seed
gives the same deck on every machine and numpy version (Box-Muller normals go through
libm ``log``/``cos`` and can differ in the last float32 bit between machines; committed
fixtures are therefore stored as files, not regenerated).

Geometry conventions follow the reference's HAMSTR converter (read_surface.py:106-153):
a panel's position is the mean of its 4 nodes, its area ``(s1*s2 + s3*s4)/2`` from the
side lengths, its normal the normalised cross product of the two diagonals.  The rotor
turns counter-clockwise about +z; blade ``b`` sits at azimuth ``2*pi*b/B`` and step ``t``
adds ``t*dPsi``.  Panels cover both sides of a NACA0012 section, cosine-spaced in chord.
The surface pressure coefficient is ``-/+0.4*sqrt((1-x/c)/(x/c+0.01))`` on the
suction/pressure side plus N(0, 0.01) noise (sigma 0.01), optionally scaled by the local
dynamic pressure ``(r/R)^2``; ``Mref`` is the tip Mach number.  Every real is rounded to
float32 before it is stored.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from .deck import Deck, BBSurface, f32

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        t = z >> np.uint64(30)
        z ^= t
        z *= np.uint64(0xBF58476D1CE4E5B9)
        np.right_shift(z, np.uint64(27), out=t)
        z ^= t
        z *= np.uint64(0x94D049BB133111EB)
        np.right_shift(z, np.uint64(31), out=t)
        z ^= t
        return z


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n doubles in (0, 1) from (seed, stream); platform independent."""
    key = _splitmix(np.array([(seed & 0xFFFFFFFF) * 1000003 + stream], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = np.arange(n, dtype=np.uint64)
        ctr *= np.uint64(0xD1B54A32D192ED03)
        ctr += key
    z = _splitmix(ctr)
    z >>= np.uint64(11)
    out = z.astype(np.float64)
    out += 0.5
    out *= 1.0 / 9007199254740992.0
    return out


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 7919, n)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


# ------------------------------------------------------------------ geometry

def naca0012_half_thickness(x: np.ndarray) -> np.ndarray:
    """NACA 4-digit thickness distribution for t/c = 0.12 (closed-trailing-edge form)."""
    return 5 * 0.12 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)


@dataclass
class RotorSpec:
    blades: int = 2
    radius: float = 1.0
    chord_root: float = 0.08
    chord_tip: float = 0.08
    root_cut: float = 0.2
    collective_deg: float = 8.0
    twist_deg: float = 0.0
    n_span: int = 30
    n_chord_side: int = 20
    tip_mach: float = 0.6
    a0: float = 340.0
    rho: float = 1.225
    pref: float = 101325.0
    minf: float = 0.0
    xy_angle: float = 0.0
    xz_angle: float = 0.0
    dpsi_deg: float = 1.0
    ntime: int = 360
    cp_local_q: bool = False
    lowpass: int = 0
    periodic: int = 1

    @property
    def omega(self) -> float:
        return f32(self.tip_mach * self.a0 / self.radius)


def blade_panels(spec: RotorSpec):
    """Panels of one blade in its own frame (blade along +x, leading edge toward +y,
    quarter chord on the x axis, pitched nose-up about x).  Returns centroid [E,3],
    area [E], unit normal [E,3], x/c at the centroid [E], side sign [E] (+1 suction),
    r/R [E]."""
    R = spec.radius
    rs = R * (spec.root_cut + (1.0 - spec.root_cut) * np.arange(spec.n_span + 1) / spec.n_span)
    xi = 0.5 * (1.0 - np.cos(math.pi * np.arange(spec.n_chord_side + 1) / spec.n_chord_side))
    frac = (rs - rs[0]) / (rs[-1] - rs[0])
    chord = spec.chord_root + (spec.chord_tip - spec.chord_root) * frac
    pitch = np.deg2rad(spec.collective_deg + spec.twist_deg * frac)
    yt = naca0012_half_thickness(xi)
    cents, areas, norms, xcs, sides, rrs = [], [], [], [], [], []
    for side in (+1, -1):
        # nodes [span+1, chord+1, 3]
        y = (0.25 - xi)[None, :] * chord[:, None]
        z = side * yt[None, :] * chord[:, None]
        cp_, sp_ = np.cos(pitch)[:, None], np.sin(pitch)[:, None]
        nodes = np.stack([np.broadcast_to(rs[:, None], y.shape), y * cp_ - z * sp_, y * sp_ + z * cp_], axis=-1)
        n1 = nodes[:-1, :-1]
        n2 = nodes[1:, :-1]
        n3 = nodes[1:, 1:]
        n4 = nodes[:-1, 1:]
        if side < 0:  # reversed winding so the normal points out of the lower surface
            n2, n4 = n4, n2
        cen = 0.25 * (n1 + n2 + n3 + n4)
        s1 = np.linalg.norm(n2 - n1, axis=-1)
        s2 = np.linalg.norm(n3 - n2, axis=-1)
        s3 = np.linalg.norm(n4 - n3, axis=-1)
        s4 = np.linalg.norm(n1 - n4, axis=-1)
        area = 0.5 * (s1 * s2 + s3 * s4)
        nrm = np.cross(n3 - n1, n4 - n2)
        nrm = nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)
        up = np.stack([np.zeros_like(pitch), -np.sin(pitch), np.cos(pitch)], axis=-1)[:-1, None, :]
        flip = np.sign(np.sum(nrm * up, axis=-1))[:, spec.n_chord_side // 2][:, None, None]
        nrm = nrm * (flip * side)
        xc = 0.5 * (xi[:-1] + xi[1:])[None, :] * np.ones((spec.n_span, 1))
        rmid = 0.5 * (rs[:-1] + rs[1:])[:, None] * np.ones((1, spec.n_chord_side))
        cents.append(cen.reshape(-1, 3))
        areas.append(area.reshape(-1))
        norms.append(nrm.reshape(-1, 3))
        xcs.append(xc.reshape(-1))
        sides.append(np.full(xc.size, side, dtype=np.float64))
        rrs.append((rmid / R).reshape(-1))
    return (np.concatenate(cents), np.concatenate(areas), np.concatenate(norms), np.concatenate(xcs),
            np.concatenate(sides), np.concatenate(rrs))


def rotor_surfaces(spec: RotorSpec, seed: int) -> List[np.ndarray]:
    cen, area, nrm, xc, side, rr = blade_panels(spec)
    E = cen.shape[0]
    T = spec.ntime
    cp0 = -side * 0.4 * np.sqrt((1.0 - xc) / (xc + 0.01))
    if spec.cp_local_q:
        cp0 = cp0 * rr ** 2
    psi_t = np.deg2rad(f32(spec.dpsi_deg)) * np.arange(T)
    # all blades in one buffer (surface-major, the layout the library takes), so the
    # concatenated rows need no second copy
    raw = np.empty(spec.blades * T * E * 8, dtype=np.float32)
    tmpl = np.zeros((E, 8), np.float32)
    tmpl[:, 2] = cen[:, 2]
    tmpl[:, 4] = area
    tmpl[:, 7] = nrm[:, 2]
    rot = np.stack([cen[:, 0], cen[:, 1], nrm[:, 0], nrm[:, 1]], 0)
    out = []
    for b in range(spec.blades):
        psi = psi_t + 2.0 * math.pi * b / spec.blades
        cs, sn = np.cos(psi), np.sin(psi)
        arr = raw[b * T * E * 8:(b + 1) * T * E * 8].reshape(T, E, 8)
        arr[:] = tmpl[None]
        for t in range(T):
            a = arr[t]
            a[:, 0] = rot[0] * cs[t] - rot[1] * sn[t]
            a[:, 1] = rot[0] * sn[t] + rot[1] * cs[t]
            a[:, 5] = rot[2] * cs[t] - rot[3] * sn[t]
            a[:, 6] = rot[2] * sn[t] + rot[3] * cs[t]
        noise = normal(seed, 100 + b, T * E).reshape(T, E) * 0.01
        arr[:, :, 3] = cp0[None, :] + noise
        out.append(arr)
    return out


def observers(kind: str, n: int, radius: float, elevation_deg: float = -30.0) -> np.ndarray:
    if kind == "circle":
        ph = 2.0 * math.pi * np.arange(n) / n
        el = math.radians(elevation_deg)
        pts = np.stack([math.cos(el) * np.cos(ph), math.cos(el) * np.sin(ph), np.full(n, math.sin(el))], -1)
    else:
        i = np.arange(n) + 0.5
        if kind == "hemisphere":     # lower hemisphere, z <= 0
            z = -i / n
        elif kind == "sphere":
            z = 1.0 - 2.0 * i / n
        else:
            raise ValueError(kind)
        rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        ph = i * math.pi * (3.0 - math.sqrt(5.0))
        pts = np.stack([rho * np.cos(ph), rho * np.sin(ph), z], -1)
    return (pts * radius).astype(np.float32)


def rotor_deck(spec: RotorSpec, obs: np.ndarray, seed: int, name: str = "") -> Deck:
    d = Deck(a0=f32(spec.a0), rhoRef=f32(spec.rho), pRef=f32(spec.pref), oM=spec.omega, nTime=spec.ntime,
             dPsi=f32(spec.dpsi_deg), Minf=f32(spec.minf), Mref=f32(spec.tip_mach), xy_angle=f32(spec.xy_angle),
             xz_angle=f32(spec.xz_angle), CFDscale=1.0, OBSscale=1.0, impermeable=1, periodic=spec.periodic,
             lowpass=spec.lowpass, BB_noise=0)
    d.obs_file = np.asarray(obs, dtype=np.float32)
    d.surfaces = rotor_surfaces(spec, seed)
    d.name = name
    return d


# ------------------------------------------------------------------ broadband inputs

def bb_table(spec: RotorSpec, n_sect_t: int = 5, small: bool = False):
    """Synthetic 2-D section table: thin-airfoil cl = 2*pi*alpha(rad), AoA -10..20 deg,
    Mach 0.05..0.9, Re 1e4..5e6, with cd, cm and boundary-layer columns filled.  `small`
    keeps 3 Mach and 3 Re entries (for the committed fixtures)."""
    sect = np.linspace(spec.root_cut, 1.0, n_sect_t).astype(np.float32)
    aoa = np.arange(-10.0, 20.0 + 1e-9, 2.0).astype(np.float32)
    mach = np.array([0.05, 0.4, 0.9] if small else [0.05, 0.2, 0.4, 0.6, 0.9], np.float32)
    re = np.array([1e4, 1e6, 5e6] if small else [1e4, 1e5, 1e6, 5e6], np.float32)
    ns, na, nm, nr = len(sect), len(aoa), len(mach), len(re)
    a = np.deg2rad(aoa.astype(np.float64))
    data = np.zeros((ns, nm, nr, na, 7), np.float64)
    beta = np.sqrt(1.0 - np.minimum(mach.astype(np.float64), 0.95) ** 2)
    lre = np.log10(re.astype(np.float64))
    data[..., 0] = 2 * math.pi * a[None, None, None, :] / beta[None, :, None, None]
    data[..., 1] = 0.008 + 0.02 * a[None, None, None, :] ** 2 + 0.0 * lre[None, None, :, None]
    data[..., 2] = -0.01
    data[..., 3] = (0.012 + 0.002 * np.abs(aoa))[None, None, None, :] * (6.0 / lre)[None, None, :, None]
    data[..., 4] = (0.010 + 0.0005 * np.abs(aoa))[None, None, None, :] * (6.0 / lre)[None, None, :, None]
    data[..., 5] = data[..., 3] * 0.3
    data[..., 6] = data[..., 4] * 0.25
    return sect, aoa, mach, re, data.astype(np.float32)


def add_bb(deck: Deck, spec: RotorSpec, nsect: int, t_del: int, trip: int, seed: int, n_sect_t: int = 5,
           small_table: bool = False, n_bb: Optional[int] = None) -> None:
    rr = np.linspace(spec.root_cut, 1.0, nsect)
    frac = (rr - rr[0]) / (rr[-1] - rr[0])
    chord = spec.chord_root + (spec.chord_tip - spec.chord_root) * frac
    theta = spec.collective_deg + spec.twist_deg * frac
    T = deck.nTime
    deck.BB_noise = 1
    deck.t_del = t_del
    deck.bb = []
    ts, ta, tm, tr, td = bb_table(spec, n_sect_t, small_table)
    for b in range(spec.blades if n_bb is None else n_bb):
        geom = np.stack([rr, np.zeros(nsect), np.zeros(nsect), chord / spec.radius], -1).astype(np.float32)
        data = np.zeros((T, nsect, 7), np.float32)
        # local section coefficients cn in [0.2, 0.8] and cc in [-0.02, 0.02]; the file holds
        # them normalised by the tip dynamic pressure, i.e. times (r/R)^2, which the reader
        # divides out again (io.cu:509-512).  (Taken literally as file values they would mean
        # cl ~ 20 at the root, where the reference's fixed-point angle-of-attack solve does not
        # converge and the result depends on the last bits of cos/sin.)
        cn = (0.2 + 0.6 * uniform(seed, 500 + b, nsect)) * rr ** 2
        cc = (-0.02 + 0.04 * uniform(seed, 600 + b, nsect)) * rr ** 2
        if t_del == 0:
            # boundary-layer thicknesses given directly (BLT/DT suction, pressure) [m]
            base = 0.01 * chord
            data[:, :, 0] = base[None, :] * 1.3
            data[:, :, 1] = base[None, :] * 0.9
            data[:, :, 2] = base[None, :] * 0.35
            data[:, :, 3] = base[None, :] * 0.2
        data[:, :, 4] = cn[None, :]
        data[:, :, 5] = cc[None, :]
        data[:, :, 6] = theta[None, :]
        deck.bb.append(BBSurface(span=f32(spec.radius), omega=spec.omega, ccw=1,
                                 psi_offset=f32(360.0 * b / spec.blades), trip=trip, geom=geom, data=data,
                                 t_sect=ts, t_aoa=ta, t_mach=tm, t_re=tr, t_data=td))


# ------------------------------------------------------------------ the five workloads

def config_spec(cfg: int) -> RotorSpec:
    if cfg == 0:
        return RotorSpec(blades=2, radius=1.0, chord_root=0.08, chord_tip=0.08, collective_deg=8.0, n_span=30,
                         n_chord_side=20, tip_mach=0.6, minf=0.0, dpsi_deg=1.0, ntime=360)
    if cfg in (1, 2):
        s = RotorSpec(blades=4, radius=1.5, chord_root=0.12, chord_tip=0.06, collective_deg=8.0, twist_deg=-10.0,
                      n_span=100, n_chord_side=40, tip_mach=0.55, minf=0.1, xy_angle=0.0, xz_angle=-5.0,
                      dpsi_deg=0.5, ntime=720, cp_local_q=True)
        if cfg == 2:
            s.dpsi_deg, s.ntime = 0.25, 1440
        return s
    if cfg == 3:
        return RotorSpec(blades=2, radius=1.0, chord_root=0.08, chord_tip=0.08, collective_deg=8.0, n_span=60,
                         n_chord_side=20, tip_mach=0.6, minf=0.05, dpsi_deg=1.0, ntime=360)
    raise ValueError(cfg)


def config_observers(cfg: int, n: Optional[int] = None) -> np.ndarray:
    if cfg == 0:
        return observers("circle", n or 16, 10.0, -30.0)
    if cfg == 1:
        return observers("hemisphere", n or 1024, 20.0 * 1.5)
    if cfg == 2:
        return observers("hemisphere", n or 4096, 20.0 * 1.5)
    if cfg == 3:
        return observers("sphere", n or 256, 10.0)
    raise ValueError(cfg)


def config_deck(cfg: int, replicate: int = 0, scale: Optional[dict] = None) -> Deck:
    """Deck of workload `cfg` (0..3) with seed 1000*cfg + replicate.  `scale` may shrink
    n_span, n_chord_side, ntime (dPsi keeps one revolution), nobs, bb_nsect for tests."""
    spec = config_spec(cfg)
    scale = dict(scale or {})
    nobs = scale.pop("nobs", None)
    bb_nsect = scale.pop("bb_nsect", 50)
    bb_small = scale.pop("bb_small", False)
    n_bb = scale.pop("n_bb", None)
    for k, v in scale.items():
        setattr(spec, k, v)
    if "ntime" in scale and "dpsi_deg" not in scale:
        spec.dpsi_deg = 360.0 / spec.ntime
    seed = 1000 * cfg + replicate
    d = rotor_deck(spec, config_observers(cfg, nobs), seed, name="config%d" % cfg)
    if cfg in (1, 2):
        add_bb(d, spec, nsect=bb_nsect, t_del=2, trip=1, seed=seed, n_sect_t=3 if bb_small else 5,
               small_table=bb_small, n_bb=n_bb)
    return d


def batch_specs(ncase: int = 64, seed0: int = 4000):
    """Per-case draws of the batched workload: 2-6 blades, 500-20000 elements per blade,
    180-1440 steps with dPsi = 360/nTime, 64-2048 observers on a 10R-30R sphere, tip Mach
    0.4-0.7, Minf 0-0.2; geometry and Cp recipe of workload 0."""
    steps = np.array([180, 240, 288, 360, 480, 576, 720, 960, 1152, 1440])
    out = []
    for c in range(ncase):
        s = seed0 + c
        u = uniform(s, 1, 8)
        B = 2 + int(u[0] * 5)
        E = 500 + int(u[1] * 19500)
        nc = max(4, int(round(math.sqrt(E / 1.5) / 2)))
        ns = max(2, int(round(E / (2 * nc))))
        T = int(steps[int(u[2] * len(steps))])
        O = 64 + int(u[3] * (2048 - 64 + 1))
        rad = 10.0 + 20.0 * u[4]
        tip = 0.4 + 0.3 * u[5]
        minf = 0.2 * u[6]
        spec = RotorSpec(blades=B, radius=1.0, chord_root=0.08, chord_tip=0.08, collective_deg=8.0, n_span=ns,
                         n_chord_side=nc, tip_mach=tip, minf=minf, dpsi_deg=360.0 / T, ntime=T)
        out.append((spec, ("sphere", O, rad), s))
    return out


def batch_deck(case: int, ncase: int = 64, shrink: Optional[dict] = None) -> Deck:
    spec, (kind, O, rad), s = batch_specs(ncase)[case]
    if shrink:
        for k, v in shrink.items():
            if k == "nobs":
                O = min(O, v)
            else:
                setattr(spec, k, min(getattr(spec, k), v))
        spec.dpsi_deg = 360.0 / spec.ntime
    return rotor_deck(spec, observers(kind, O, rad), s, name="batch%d" % case)


def permeable_rows(seed: int, ne, ntime: int, radius: float = 1.2, mach_tip: float = 0.55):
    """Seeded rows of a permeable data surface for preprocess_per (preprocess.cu:8-226):
    a ring of panels rotating about z (one rotor period over ntime steps) with a
    periodic flow field on it.  Returns X (x, y, z, ds), N (n, 0), U (u, 0), PR (P, 0,
    rho, 0), each [element][step][k], all surfaces' elements stacked (ne = elements per
    surface), values in the non-dimensional units the reader sees (io.cu:286)."""
    E = int(sum(ne))
    u = uniform(seed, 5, E * 8).reshape(E, 8)
    ph = 2.0 * np.pi * np.arange(ntime) / ntime
    az = 2.0 * np.pi * np.arange(E) / E
    X = np.zeros((E, ntime, 4))
    N = np.zeros((E, ntime, 6))
    U = np.zeros((E, ntime, 6))
    PR = np.zeros((E, ntime, 4))
    th = az[:, None] + ph[None, :]
    r = radius * (1.0 + 0.05 * (u[:, 0:1] - 0.5))
    z = 0.3 * (u[:, 1:2] - 0.5)
    X[:, :, 0] = r * np.cos(th)
    X[:, :, 1] = r * np.sin(th)
    X[:, :, 2] = z
    X[:, :, 3] = 0.01 * (1.0 + u[:, 2:3])
    N[:, :, 0] = np.cos(th)
    N[:, :, 1] = np.sin(th)
    harm = np.sin(3.0 * th + 6.0 * u[:, 3:4]) + 0.2 * np.cos(7.0 * th)
    U[:, :, 0] = -mach_tip * np.sin(th) * (1.0 + 0.1 * harm)
    U[:, :, 1] = mach_tip * np.cos(th) * (1.0 + 0.1 * harm)
    U[:, :, 2] = 0.05 * harm
    PR[:, :, 0] = 0.8 * harm + 0.1 * (u[:, 4:5] - 0.5)
    PR[:, :, 2] = 1.0 + 0.02 * harm
    return X, N, U, PR


def permeable_deck(seed: int, ne, ntime: int, nobs: int = 4, lowpass: int = 1, periodic: int = 1) -> Deck:
    """A permeable deck (impermeable 0): the data surface of permeable_rows written as the
    12-column rows read_surf reads for such decks, x y z u v w P rho ds nx ny nz
    (io.cu:286), with a few observers on a 10 m circle.  The reference preprocesses such
    a deck (preprocess_per, main.cu:87) and launches no acoustic kernel for it
    (main.cu:236), so its pressure outputs are zero."""
    X, N, U, PR = permeable_rows(seed, ne, ntime)
    rows = np.zeros((int(sum(ne)), ntime, 12), dtype=np.float32)
    rows[:, :, 0:3] = X[:, :, 0:3]
    rows[:, :, 3:6] = U[:, :, 0:3]
    rows[:, :, 6] = PR[:, :, 0]
    rows[:, :, 7] = PR[:, :, 2]
    rows[:, :, 8] = X[:, :, 3]
    rows[:, :, 9:12] = N[:, :, 0:3]
    surfs = []
    e0 = 0
    for n in ne:
        surfs.append(np.ascontiguousarray(rows[e0:e0 + n].transpose(1, 0, 2)))
        e0 += n
    obs = observers("circle", nobs, 10.0, elevation_deg=-20.0)
    return Deck(a0=340.0, rhoRef=1.2, pRef=101325.0, oM=150.0, nTime=ntime, dPsi=360.0 / ntime, Minf=0.0,
                Mref=0.5, CFDscale=1.0, OBSscale=1.0, impermeable=0, periodic=periodic, lowpass=lowpass,
                BB_noise=0, obs_file=obs.astype(np.float32), surfaces=surfs, name="permeable")
