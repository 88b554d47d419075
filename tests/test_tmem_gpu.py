"""The tensor-memory path of the mixed kernel's record stages: a pattern laid out as one
element-pair tile goes from shared memory into tensor memory (ten 32x128b.warpx4
copies) and back into the registers of every warp of a block, unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_memory_copy_round_trip():
    from acum3_periodic_gb300 import native
    mismatches, rb = native.selftest_tmem(0)
    assert mismatches == 0
    lane = np.arange(32)[:, None]
    col = np.arange(40)[None, :]
    expected = 0x10000 + (col >> 2) * 128 + lane * 4 + (col & 3)
    for w in range(4):
        assert np.array_equal(rb[w], expected)
