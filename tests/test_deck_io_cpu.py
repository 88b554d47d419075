"""The deck readers on the host (acum_read_deck_sizes: the readers and checks of
acum_load_deck without a device), on decks written in the reference's formats and on
broken copies of them.  The reference exits, or crashes, on most of these inputs
(io.cu:18-21, 66, 109-113, 234); the library returns ACUM_ERR_IO with a message."""
import ctypes as C
import os
import shutil

import pytest

from acum3_periodic_gb300 import synth
from acum3_periodic_gb300.deck import write_deck

IO_ERR = -2


def sizes(path):
    from acum3_periodic_gb300 import native
    L = native.lib()
    out = (C.c_longlong * 6)()
    rc = L.acum_read_deck_sizes(os.fsencode(str(path)), out)
    return rc, [int(v) for v in out], L.acum_last_global_error().decode()


@pytest.fixture(scope="module")
def tonal_deck(tmp_path_factory):
    d = synth.config_deck(0, scale=dict(n_span=4, n_chord_side=3, ntime=24, nobs=5))
    p = tmp_path_factory.mktemp("deck0")
    write_deck(d, str(p))
    return d, p


@pytest.fixture(scope="module")
def bb_deck(tmp_path_factory):
    d = synth.config_deck(1, scale=dict(n_span=4, n_chord_side=3, ntime=24, nobs=5, bb_nsect=4, bb_small=True))
    p = tmp_path_factory.mktemp("deck1")
    write_deck(d, str(p))
    return d, p


def copy_of(src, tmp_path):
    dst = tmp_path / "copy"
    shutil.copytree(src, dst)
    return dst


def test_good_decks(tonal_deck, bb_deck):
    d, p = tonal_deck
    rc, s, _ = sizes(p)
    assert rc == 0 and s == [d.nSurf, d.nTime, d.nObs, d.E, 0, 0]
    d, p = bb_deck
    rc, s, _ = sizes(p)
    assert rc == 0 and s[:4] == [d.nSurf, d.nTime, d.nObs, d.E]
    assert s[4] == sum(b.nsect for b in d.bb) and s[5] == 1


def test_unknown_input_key(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    with open(p / "input", "a") as f:
        f.write("speedOfSound 340\n")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "speedOfSound" in msg


def test_missing_value(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    with open(p / "input", "a") as f:
        f.write("oM")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "oM" in msg


def test_missing_input_and_observers(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    os.remove(p / "obs.dat")
    assert sizes(p)[0] == IO_ERR
    os.remove(p / "input")
    assert sizes(p)[0] == IO_ERR


def test_short_observer_file(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    lines = open(p / "obs.dat").read().splitlines()
    with open(p / "obs.dat", "w") as f:
        f.write("\n".join(lines[:-1]) + "\n")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "obs.dat" in msg


def test_missing_surface_file(tonal_deck, tmp_path):
    # the reference does not check the fopen and crashes here (io.cu:234)
    p = copy_of(tonal_deck[1], tmp_path)
    os.remove(p / "surfaces" / "surface_2.dat")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "surface_2" in msg


def test_truncated_surface_rows(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    fn = p / "surfaces" / "surface_1.dat"
    lines = open(fn).read().splitlines()
    with open(fn, "w") as f:
        f.write("\n".join(lines[:-3]) + "\n")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "surface_1" in msg


def test_bad_surface_header(tonal_deck, tmp_path):
    p = copy_of(tonal_deck[1], tmp_path)
    fn = p / "surfaces" / "surface_1.dat"
    body = open(fn).read().split("\n", 1)[1]
    with open(fn, "w") as f:
        f.write("x y\n" + body)
    assert sizes(p)[0] == IO_ERR


def test_missing_broadband_files(bb_deck, tmp_path):
    p = copy_of(bb_deck[1], tmp_path)
    os.remove(p / "BB_inputs" / "BB_table_1.dat")
    assert sizes(p)[0] == IO_ERR
    p2 = tmp_path / "copy2"
    shutil.copytree(bb_deck[1], p2)
    os.remove(p2 / "input_BB")
    assert sizes(p2)[0] == IO_ERR


def write_cache(path):
    from acum3_periodic_gb300 import native
    return native.lib().acum_write_surface_cache(os.fsencode(str(path)))


def test_surface_cache_used_and_refreshed(tonal_deck, tmp_path):
    d, src = tonal_deck
    p = copy_of(src, tmp_path)
    assert write_cache(p) == 0
    assert os.path.exists(p / "surfaces" / "surfaces.acumbin")
    rc, s, _ = sizes(p)
    assert rc == 0 and s == [d.nSurf, d.nTime, d.nObs, d.E, 0, 0]
    # a changed text file makes the cache stale: the text is parsed (and here found short)
    fn = p / "surfaces" / "surface_1.dat"
    lines = open(fn).read().splitlines()
    with open(fn, "w") as f:
        f.write("\n".join(lines[:-3]) + "\n")
    rc, _, msg = sizes(p)
    assert rc == IO_ERR and "surface_1" in msg


def test_foreign_surface_cache_ignored(tonal_deck, tmp_path):
    d, src = tonal_deck
    p = copy_of(src, tmp_path)
    with open(p / "surfaces" / "surfaces.acumbin", "wb") as f:
        f.write(b"not a cache" * 10)
    rc, s, _ = sizes(p)
    assert rc == 0 and s == [d.nSurf, d.nTime, d.nObs, d.E, 0, 0]


PERM_DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", "permeable_deck")


def test_permeable_deck_read(tmp_path):
    """A permeable deck (impermeable 0): 12-column rows (io.cu:263-293); a file cut short
    is refused; the surface cache keeps the 12-column rows and a cache of another row
    width is not used."""
    p = tmp_path / "perm"
    shutil.copytree(PERM_DECK, p, ignore=shutil.ignore_patterns("expected"))
    rc, s, msg = sizes(p)
    assert rc == 0, msg
    assert s == [2, 40, 3, 10, 0, 0]
    assert write_cache(p) == 0
    rc, s2, _ = sizes(p)
    assert rc == 0 and s2 == s
    # the same rows read as an impermeable deck (8 columns) do not match the cached width:
    # the text is parsed again, with 8 columns per row
    inp = open(p / "input").read().replace("impermeable 0", "impermeable 1")
    with open(p / "input", "w") as f:
        f.write(inp)
    rc, s3, _ = sizes(p)
    assert rc == 0 and s3 == s
    q = tmp_path / "perm_short"
    shutil.copytree(PERM_DECK, q, ignore=shutil.ignore_patterns("expected"))
    fn = q / "surfaces" / "surface_2.dat"
    lines = open(fn).read().splitlines()
    with open(fn, "w") as f:
        f.write("\n".join(lines[:-1]) + "\n")
    rc, _, msg = sizes(q)
    assert rc == IO_ERR and "surface_2" in msg
