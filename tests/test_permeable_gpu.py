"""Permeable-surface preprocessing (preprocess_per, preprocess.cu:8-226) on the GPU through
acum_preprocess_per / acum_preprocess_per_f64, against the reference's FP64 build
(tests/golden/permeable.npz) and the oracle.

The kernel computes in FP64 in the reference's order of operations without fused
multiply-adds, so the FP64 form is compared for equality, and the float form against the
oracle's FP64 results (on the same float inputs) rounded once to float, also for
equality."""
import ctypes as C
import os

import numpy as np
import pytest

from acum3_periodic_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ERR_INVALID, ERR_UNSUPPORTED = -1, -8  # include/acum.h


def _native():
    from acum3_periodic_gb300 import native
    return native


@pytest.mark.parametrize("periodic,lowpass", [(1, 0), (0, 1)])
def test_golden_f64_bit_exact(periodic, lowpass):
    native = _native()
    g = np.load(os.path.join(GOLDEN, "permeable.npz"))
    V0 = np.zeros_like(g["N"])
    got = native.preprocess_per(g["ne"], g["X"], g["N"], V0, g["U"], g["PR"], *g["scal"], periodic, lowpass)
    for nm, a in zip("XNVUP", got):
        np.testing.assert_array_equal(a, g["%s_p%d_l%d" % (nm, periodic, lowpass)], err_msg=nm)


@pytest.mark.parametrize("rep,ntime,periodic,lowpass", [(41, 6, 0, 1), (42, 97, 1, 1), (43, 360, 0, 0),
                                                         (44, 4096, 1, 1)])
def test_random_against_oracle(rep, ntime, periodic, lowpass):
    """Ragged surfaces (one empty), the shortest period accepted (6 steps), a long one
    (4096, 64 KB of shared memory per block); FP64 and float storage."""
    native = _native()
    ne = [3, 0, 7, 1] if ntime < 4096 else [2, 3]
    X, N, U, PR = synth.permeable_rows(rep, ne, ntime)
    rng = np.random.default_rng(rep)
    PR[:, :, 0] += 0.05 * rng.standard_normal(PR.shape[:2])
    U[:, :, 2] += 0.01 * rng.standard_normal(U.shape[:2])
    V0 = np.zeros_like(N)
    args = (1.0 / (ntime * 7.3), 341.0, 1.18, 0.11, 2.5, periodic, lowpass)
    want = O.preprocess_per(X, N, U, PR, *args)
    got = native.preprocess_per(ne, X, N, V0, U, PR, *args)
    for nm, a, b in zip("XNVUP", got, want):
        np.testing.assert_array_equal(a, b, err_msg=nm)
    # float storage: inputs and scalars rounded to float, results rounded once
    f = lambda a: np.asarray(a, np.float32).astype(np.float64)
    fargs = tuple(float(np.float32(x)) for x in args[:5]) + args[5:]
    want32 = O.preprocess_per(f(X), f(N), f(U), f(PR), *fargs)
    got32 = native.preprocess_per(ne, X, N, V0, U, PR, *args, dtype=np.float32)
    for nm, a, b in zip("XNVUP", got32, want32):
        np.testing.assert_array_equal(a, b.astype(np.float32), err_msg=nm)


def test_surface_offsets_are_honoured():
    """The surfaces stored in reverse order in the arrays (Ptr[] not increasing): each
    element is found through its surface's pointer, as the reference indexes them."""
    native = _native()
    lib = native.lib()
    ne, T = [4, 2, 5], 30
    X, N, U, PR = synth.permeable_rows(45, ne, T)
    args = (0.004, 340.0, 1.2, 0.08, 1.0, 1, 1)
    want = O.preprocess_per(X, N, U, PR, *args)
    # reversed storage: surface 2 first, then 1, then 0
    starts = np.concatenate([[0], np.cumsum(ne)[:-1]])
    order = [2, 1, 0]
    perm = np.concatenate([np.arange(starts[s], starts[s] + ne[s]) for s in order])
    arrs = [np.ascontiguousarray(a[perm]) for a in (X, N, np.zeros_like(N), U, PR)]
    pos = {}
    acc = 0
    for s in order:
        pos[s] = acc
        acc += ne[s]
    ptrs = [np.array([pos[s] * T * w for s in range(3)], np.int32) for w in (4, 6, 6, 6, 4)]
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    E = np.array(ne, np.int32)
    rc = lib.acum_preprocess_per_f64(*[vp(a) for a in arrs], 3, *[vp(q) for q in ptrs], vp(E), T, *args)
    assert rc == 0, lib.acum_last_global_error()
    inv = np.argsort(perm)
    for nm, a, b in zip("XNVUP", arrs, want):
        np.testing.assert_array_equal(a[inv], b, err_msg=nm)


def test_refused_sizes():
    native = _native()
    X, N, U, PR = synth.permeable_rows(46, [2], 5)
    with pytest.raises(native.AcumError) as e:  # at least 6 steps
        native.preprocess_per([2], X, N, np.zeros_like(N), U, PR, 0.01, 340.0, 1.2, 0.08, 1.0, 1, 0)
    assert e.value.code == ERR_INVALID
    X, N, U, PR = synth.permeable_rows(46, [2], 8)
    for bad_dt in (0.0, -0.01, float("inf")):
        with pytest.raises(native.AcumError) as e:
            native.preprocess_per([2], X, N, np.zeros_like(N), U, PR, bad_dt, 340.0, 1.2, 0.08, 1.0, 1, 0)
        assert e.value.code == ERR_INVALID
    X, N, U, PR = synth.permeable_rows(47, [1], 4097)
    with pytest.raises(native.AcumError) as e:
        native.preprocess_per([1], X, N, np.zeros_like(N), U, PR, 0.01, 340.0, 1.2, 0.08, 1.0, 1, 0)
    assert e.value.code == ERR_UNSUPPORTED


def test_device_entry_matches_host_entry():
    """acum_preprocess_per_device on arrays already in device memory (torch tensors, on a
    side stream) gives the host entry's results, float and double."""
    torch = pytest.importorskip("torch")
    native = _native()
    lib = native.lib()
    ne, T = [6, 9], 144
    X, N, U, PR = synth.permeable_rows(48, ne, T)
    args = (0.0031, 340.0, 1.2, 0.08, 1.3, 1, 1)
    off = np.concatenate([[0], np.cumsum(ne)[:-1]])
    ptrs = [np.ascontiguousarray(off * T * w, dtype=np.int32) for w in (4, 6, 6, 6, 4)]
    E = np.array(ne, np.int32)
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    for dt, tdt in ((np.float64, torch.float64), (np.float32, torch.float32)):
        if dt == np.float32:  # the float host entry takes float scalars
            args = tuple(float(np.float32(x)) for x in args[:5]) + args[5:]
        want = native.preprocess_per(ne, X, N, np.zeros_like(N), U, PR, *args, dtype=dt)
        dev = [torch.tensor(np.asarray(a, dt), device="cuda:0") for a in (X, N, np.zeros_like(N), U, PR)]
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            rc = lib.acum_preprocess_per_device(*[C.c_void_p(t.data_ptr()) for t in dev], int(dt == np.float64), 2,
                                                *[vp(q) for q in ptrs], vp(E), T, *args, C.c_void_p(s.cuda_stream))
        assert rc == 0, lib.acum_last_global_error()
        s.synchronize()
        for nm, t, w in zip("XNVUP", dev, want):
            np.testing.assert_array_equal(t.cpu().numpy(), w, err_msg=nm)


def test_signed_zeros_and_ties():
    """Series with exact zeros of both signs and repeated values: the median's integer keys
    treat -0 and +0 as equal (as the reference's comparisons do) and a zero difference
    keeps the sign the IEEE quotient gives it."""
    native = _native()
    ne, T = [3], 40
    X, N, U, PR = synth.permeable_rows(49, ne, T)
    U[0, :, 2] = 0.0
    U[0, ::3, 2] = -0.0
    U[1, :, 2] = np.where(np.arange(T) % 4 < 2, 1.0, -1.0)
    PR[2, :, 0] = np.round(PR[2, :, 0], 1)  # ties
    N[0, :, 2] = -0.0
    N[0, 5:9, 2] = 0.0
    args = (0.004, 340.0, 1.2, 0.08, 1.0)
    for periodic, lowpass in ((1, 1), (0, 1), (1, 0)):
        want = O.preprocess_per(X, N, U, PR, *args, periodic, lowpass)
        got = native.preprocess_per(ne, X, N, np.zeros_like(N), U, PR, *args, periodic, lowpass)
        for nm, a, b in zip("XNVUP", got, want):
            np.testing.assert_array_equal(a, b, err_msg=nm)
            assert np.array_equal(np.signbit(a), np.signbit(b)), nm
