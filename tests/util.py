"""Error metrics shared by the parity tests."""
import numpy as np


def per_receiver_rel(test, ref):
    """Relative L2 per receiver seismogram over time and both components.

    test/ref: (nsave, nrecv, 2).  A receiver with a zero reference trace is
    compared in absolute terms."""
    num = np.linalg.norm((test - ref).transpose(1, 0, 2).reshape(ref.shape[1], -1), axis=1)
    den = np.linalg.norm(ref.transpose(1, 0, 2).reshape(ref.shape[1], -1), axis=1)
    return num / np.where(den > 0, den, 1.0)


def peak_rel(test, ref):
    """Peak-amplitude relative error per receiver (both components)."""
    pt = np.abs(test).max(axis=(0, 2))
    pr = np.abs(ref).max(axis=(0, 2))
    return np.abs(pt - pr) / np.where(pr > 0, pr, 1.0)


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)
