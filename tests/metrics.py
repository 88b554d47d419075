"""Error measures used by the parity tests (the conventions of the measurement plan)."""
import numpy as np


def per_bin_rel(p, ref, floor=1e-6):
    """|p - ref| / max(|ref|, floor * max_t |ref(obs)|), per (bin, observer)."""
    scale = np.maximum(np.abs(ref), floor * np.abs(ref).max(axis=0, keepdims=True))
    return np.abs(p - ref) / scale


def per_bin_rms(p, ref):
    """|p - ref| / rms_t(ref(obs)): the error normalised by the observer's RMS."""
    rms = np.sqrt(np.mean(ref ** 2, axis=0, keepdims=True))
    return np.abs(p - ref) / rms


def oaspl_db(p, pref=2e-5):
    """tonal OASPL per observer: 10 log10(mean_t(p^2) / pref^2)."""
    return 10.0 * np.log10(np.mean(p ** 2, axis=0) / pref ** 2)
