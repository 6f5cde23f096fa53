"""The plain FP64 form against the CPU oracle on the benched configurations
at their full size and length, through the C ABI.

Tolerance: <= 1e-12 relative L2 on every receiver seismogram (both components
over time), each receiver against its own norm (no floor).  The runs are full
length so that every receiver records the whole pulse: a receiver that holds
only the leading tail of a pulse (amplitudes many orders below the others)
measures the round-off of the field around it, not the seismogram.
"""
import os

import numpy as np
import pytest

from exfem import workloads
from exfem.gpu import Solver
from oracle import oracle
from util import fp64_rel, rel

pytestmark = pytest.mark.gpu
TOL = 1e-12
NT = os.cpu_count() or 8


def gpu_run(m):
    with Solver(m) as s:
        mf = s.init_explicit()
        s.run()
        s.sync()
        return mf, s.seismograms(), [s.u(r) for r in range(s.nrhs)]


def test_full_size_canyon_every_rhs():
    """The canyon as configured: 192K elements, 680 hanging nodes, P at
    0/30/60 deg and SV at 0/15/25 deg, all 8000 steps."""
    m = workloads.build("canyon")
    assert m.problem.nrhs == 6 and m.problem.nsteps == 8000 and m.problem.nhanging > 0
    mf, seis, us = gpu_run(m)
    for r in range(m.problem.nrhs):
        o = oracle.run(m, rhs=r, nthreads=NT)
        assert np.array_equal(mf, o["mfull"])
        err = fp64_rel(seis[r], o["seis"])
        assert err.max() <= TOL, (r, err.max())
        assert rel(us[r], o["u"]) <= TOL


def test_full_size_valley_full_length():
    """The heterogeneous valley as configured: 1.53M elements, 3177 hanging
    nodes, four quadtree levels, SV fc 5 Hz, all 20000 steps (2.65 s: the
    pulse crosses the 400 m of 300 m/s infill to every surface receiver)."""
    m = workloads.build("valley")
    assert m.nelems > 1_400_000 and m.problem.nsteps == 20000
    o = oracle.run(m, nthreads=NT)
    mf, seis, us = gpu_run(m)
    assert np.array_equal(mf, o["mfull"])
    peak = np.abs(o["seis"]).max(axis=(0, 2))
    assert peak.min() > 1e-2 * peak.max()       # every receiver holds the pulse
    err = fp64_rel(seis[0], o["seis"])
    assert err.max() <= TOL, err.max()
    assert rel(us[0], o["u"]) <= TOL
