"""The C ABI library on a machine without a GPU: it builds, loads, exports every symbol
include/acum.h declares, and fails loudly (no CPU fallback) when no device is present."""
import re

import pytest

from conftest import ROOT


def test_library_exports_every_declared_symbol():
    from acum3_periodic_gb300 import native
    L = native.lib()
    hdr = open(ROOT + "/include/acum.h").read()
    syms = sorted(set(re.findall(r"\b(acum_[a-z0-9_]+)\s*\(", hdr)))
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing
    assert set(syms) == set(native.SIGNATURES)
    assert L.acum_version() >= 1


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from acum3_periodic_gb300 import native
    with pytest.raises(native.AcumError) as e:
        native.Context(0)
    assert e.value.code == -3


def test_preprocess_per_argument_checks_on_the_host():
    """acum_preprocess_per validates its layout and scalars before any CUDA call: bad
    arguments come back as statuses on a machine without a GPU, and a layout without
    elements is a no-op.  With a valid layout and no GPU the call fails loudly."""
    import ctypes as C

    import numpy as np
    import torch
    from acum3_periodic_gb300 import native, synth
    L = native.lib()
    ne, T = [2], 12
    X, N, U, PR = synth.permeable_rows(3, ne, T)
    arrs = [np.ascontiguousarray(a, np.float32) for a in (X, N, np.zeros_like(N), U, PR)]
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    ptrs = [np.zeros(1, np.int32) for _ in range(5)]

    def call(E, T_, dt, arrays=arrs):
        return L.acum_preprocess_per(*[vp(a) if a is not None else None for a in arrays], 1,
                                     *[vp(q) for q in ptrs], vp(np.array(E, np.int32)), T_, dt, 340.0, 1.2, 0.08,
                                     1.0, 1, 1)

    ERR_INVALID, ERR_UNSUPPORTED = -1, -8
    assert call([2], 5, 0.01) == ERR_INVALID           # fewer than 6 steps
    assert call([2], T, 0.0) == ERR_INVALID            # dTau not positive
    assert call([2], T, -1.0) == ERR_INVALID
    assert call([2], T, float("nan")) == ERR_INVALID
    assert call([-1], T, 0.01) == ERR_INVALID          # negative element count
    assert call([2], 4097, 0.01) == ERR_UNSUPPORTED    # beyond the 4096-step rows
    assert call([2], T, 0.01, [None] + arrs[1:]) == ERR_INVALID
    assert call([0], T, 0.01) == 0                     # nothing to do
    if not torch.cuda.is_available():
        assert call([2], T, 0.01) not in (0, ERR_INVALID, ERR_UNSUPPORTED)
