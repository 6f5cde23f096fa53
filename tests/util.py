"""Error metrics shared by the parity tests."""
import numpy as np


def per_receiver_rel(test, ref, floor=1e-3):
    """Relative L2 per receiver seismogram over time and both components.

    test/ref: (nsave, nrecv, 2).  A receiver the wave has not reached carries
    only round-off (FP32 denormals, ~1e-40): its error is measured against
    `floor` times the strongest receiver's norm instead of its own."""
    num = np.linalg.norm((test - ref).transpose(1, 0, 2).reshape(ref.shape[1], -1), axis=1)
    den = np.linalg.norm(ref.transpose(1, 0, 2).reshape(ref.shape[1], -1), axis=1)
    den = np.maximum(den, floor * den.max())
    return num / np.where(den > 0, den, 1.0)


def fp64_rel(test, ref):
    """Relative L2 per receiver seismogram with no floor: every receiver is
    measured against its own norm (a receiver whose reference trace is all
    zero is measured absolutely).  The bar for the plain FP64 form."""
    return per_receiver_rel(test, ref, floor=0.0)


def peak_rel(test, ref, floor=1e-3):
    """Peak-amplitude relative error per receiver (both components), with the
    same floor as per_receiver_rel."""
    pt = np.abs(test).max(axis=(0, 2))
    pr = np.abs(ref).max(axis=(0, 2))
    den = np.maximum(pr, floor * pr.max())
    return np.abs(pt - pr) / np.where(den > 0, den, 1.0)


def rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)
