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
