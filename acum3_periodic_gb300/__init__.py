"""GB300-native implementation of ACUM-3's periodic acoustic hot path.

Tonal: impermeable Farassat-1A thickness and loading noise binned by retarded time into
periodic observer-time bins.  Broadband: BPM spectra per span section and observer.
The compute runs in hand-written sm_103a CUDA kernels behind a C ABI (include/acum.h);
this package holds the deck model, the synthetic rotor generator and the Python binding
of that ABI.
"""
from .deck import Deck, BBSurface, read_deck, write_deck, BB_BANDS, BB_COMPONENTS  # noqa: F401
