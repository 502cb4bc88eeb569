"""Shared comparison helpers for the parity tests."""
import numpy as np


def rel_err(x, ref):
    """max |x - ref| / max(|ref|, tiny) over the whole array."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = max(float(np.max(np.abs(ref))) if ref.size else 0.0, 1e-300)
    return float(np.max(np.abs(x - ref))) / scale if ref.size else 0.0


def sections(o, slab):
    """Split a slab into E0, one-body and two-body parts (oracle layout sizes)."""
    b = o.basis
    A = b.nholes
    P = b.norbits - A
    n1 = 1 + A * A + P * P + P * A
    return slab[0], slab[1:n1], slab[n1:]
