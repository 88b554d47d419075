"""The oracle against a known answer (CPU): a rotor deck frozen at its first step with
constant Cp radiates steady loading noise only, the same value in every observer bin:
p = sum_e D1 ds a0 P (n . r_hat) / r^2 (core.cu:130-141 with every rate zero)."""
import numpy as np

from oracle import oracle as O
from test_properties_gpu import frozen_deck, steady_loading


def test_oracle_frozen_rotor_known_answer():
    d = frozen_deck()
    ref = steady_loading(d)
    pT, pL, pA, bad = O.tonal(d, nthreads=4)
    assert bad == 0
    assert np.max(np.abs(pT)) == 0.0
    assert np.max(np.abs(pA - ref[None, :]) / np.abs(ref[None, :])) < 1e-12
