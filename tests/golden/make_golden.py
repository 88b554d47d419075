"""Generates the committed golden fixtures of tests/golden/ from the reference's own
sources compiled for the host (oracle/build_ref.sh).  Run from the repository root where
the reference tree is available:

    python tests/golden/make_golden.py

It writes a few small seeded decks (the reference's text formats) under
tests/golden/decks/<name>/ and, for each, the FP64-build outputs (plus the as-written
FP32-build outputs, for information) into tests/golden/<name>.npz; and unit vectors of
the broadband shape curves and the preprocessing filters into tests/golden/units.npz; and
the permeable preprocessing of a seeded data surface into tests/golden/permeable.npz; and
a permeable deck directory with its preprocessed arrays (tests/golden/permeable_deck.npz)
and the reference's pressure files for it (decks/permeable_deck/expected/).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from acum3_periodic_gb300 import synth  # noqa: E402
from acum3_periodic_gb300.deck import write_deck  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def decks():
    out = {}
    # tonal, hover, config-0 geometry
    out["tonal_hover"] = synth.config_deck(0, replicate=11, scale=dict(n_span=4, n_chord_side=3, ntime=24, nobs=4))
    # tonal, forward flight (convected retarded time), lowpass filters, biased Pdot
    d = synth.config_deck(3, replicate=12, scale=dict(n_span=3, n_chord_side=3, ntime=36, nobs=5))
    d.lowpass, d.periodic, d.xy_angle = 1, 0, 20.0
    out["tonal_flight_lowpass"] = d
    # broadband, empirical boundary layer (config-1 recipe)
    d = synth.config_deck(1, replicate=13, scale=dict(n_span=2, n_chord_side=2, ntime=40, nobs=4, bb_nsect=6, bb_small=True, n_bb=2))
    out["bb_tdel2"] = d
    # broadband, table boundary layer, untripped (LBL-VS on), clockwise surface, rotated
    # and translated mounting, crossflow
    d = synth.config_deck(1, replicate=14, scale=dict(n_span=2, n_chord_side=2, ntime=32, nobs=3, bb_nsect=5, bb_small=True, n_bb=3))
    d.t_del, d.xy_angle = 1, 30.0
    for b in d.bb:
        b.trip = 0
    d.bb[1].ccw = 0
    d.bb[2].rotate = (2.0, -3.0, 10.0)
    d.bb[2].translate = (0.1, -0.2, 0.05)
    out["bb_tdel1_lbl_cw"] = d
    # broadband, thicknesses read from the surface file, hover
    d = synth.config_deck(1, replicate=15, scale=dict(n_span=2, n_chord_side=2, ntime=24, nobs=3, bb_nsect=4, bb_small=True, n_bb=2))
    d.t_del, d.Minf = 0, 0.0
    for b in d.bb:
        c = b.geom[:, 3] * b.span
        b.data[:, :, 0] = 0.013 * c
        b.data[:, :, 1] = 0.009 * c
        b.data[:, :, 2] = 0.0035 * c
        b.data[:, :, 3] = 0.002 * c
    out["bb_tdel0_hover"] = d
    return out


def main():
    if not ref.available("f64"):
        ref.build()
    os.makedirs(os.path.join(OUT, "decks"), exist_ok=True)
    for name, d in decks().items():
        path = os.path.join(OUT, "decks", name)
        write_deck(d, path)
        res = {}
        for prec in ("f64", "f32"):
            rd = ref.RefDeck(path, prec)
            pT, pL, pA = rd.tonal()
            res["pT_" + prec], res["pL_" + prec], res["pA_" + prec] = pT, pL, pA
            X, N, V, P = rd.fields()
            if prec == "f64":
                res["fields_X"], res["fields_N"], res["fields_V"], res["fields_P"] = X, N, V, P
            if d.BB_noise == 1:
                spl, oas = rd.bpm()
                res["spl_" + prec], res["oaspl_" + prec] = spl, oas
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **res)
        print("wrote", name, {k: v.shape for k, v in res.items()})
    # unit vectors
    x_ab = np.linspace(0.0, 0.6, 241)
    units = {"x_ab": x_ab}
    for w, nm in enumerate(("a_min", "a_max", "b_min", "b_max")):
        units[nm] = ref.bb_curve(w, x_ab)
    hh = np.array([0.01, 0.1, 0.25, 0.4, 0.62, 0.9, 1.15, 1.18, 2.0, 5.0])
    ee = np.linspace(-1.0, 0.3, 53)
    units["g5_h"], units["g5_eta"] = hh, ee
    units["g5"] = np.array([[ref.g5comp(h, e) for e in ee] for h in hh])
    rng_u = synth.uniform(77, 1, 3 * 50)
    series = np.sin(np.linspace(0, 2 * np.pi, 50, endpoint=False) * 3) + 0.3 * (rng_u[:50] - 0.5) + 0.2 * np.linspace(0, 1, 50)
    units["series"] = series
    units["make_periodic"] = ref.make_periodic(series)
    units["lowpass"] = ref.lowpass(series)
    units["diff_periodic"] = ref.differentiate(series, 0.01, False)
    units["diff_biased"] = ref.differentiate(series, 0.01, True)
    np.savez_compressed(os.path.join(OUT, "units.npz"), **units)
    print("wrote units")
    # permeable preprocessing (preprocess_per) of a seeded rotating data surface, two
    # surfaces; outputs for (periodic, lowpass) = (1, 0) and (0, 1)
    ne, T = [5, 3], 48
    X, N, U, PR = synth.permeable_rows(21, ne, T)
    per = {"ne": np.array(ne), "X": X, "N": N, "U": U, "PR": PR,
           "scal": np.array([0.0021, 340.0, 1.2, 0.08, 1.5])}
    for periodic, lowpass in ((1, 0), (0, 1)):
        outs = ref.preprocess_per(ne, X, N, np.zeros_like(N), U, PR, *per["scal"], periodic, lowpass)
        for nm, a in zip("XNVUP", outs):
            per["%s_p%d_l%d" % (nm, periodic, lowpass)] = a
    np.savez_compressed(os.path.join(OUT, "permeable.npz"), **per)
    print("wrote permeable")
    # a permeable deck directory (impermeable 0, 12-column surface rows, filters on),
    # loaded by the reference's own readers: its preprocess_per arrays (FP64 build) and the
    # pressure files the reference writes for it (FP32 build, the program as shipped)
    d = synth.permeable_deck(22, [6, 4], 40, nobs=3)
    path = os.path.join(OUT, "decks", "permeable_deck")
    write_deck(d, path)
    rd = ref.RefDeck(path, "f64")
    pd = dict(zip(("X", "N", "V", "U", "PR"), rd.permeable_fields()))
    np.savez_compressed(os.path.join(OUT, "permeable_deck.npz"), **pd)
    exp = os.path.join(path, "expected")
    os.makedirs(exp, exist_ok=True)
    ref.RefDeck(path, "f32").write_zero_history(exp)
    print("wrote permeable_deck")


if __name__ == "__main__":
    main()
