"""Point sources (POINTN force, POINTD displacement; setup_point_source,
point_reactions and point_displacements, model.f90:808-845, 1051-1078) on
the host model and the oracle, without a GPU."""
import math

import numpy as np
import pytest

from exfem import decks, workloads
from exfem.abi import EXFEM_POINT_DISP, EXFEM_POINT_FORCE, ExfemError
from exfem.model import Model
from oracle import oracle


def ricker_point(amp, sigma, t):
    """ricker (formulation.f90:53-59)."""
    return amp * math.exp(-t * t / (4 * sigma)) * (t * t - 2 * sigma) / (8 * math.sqrt(math.pi) * sigma ** 2.5)


def brute_force_nodes(model, pparams):
    xy = model.nodes().reshape(-1, 2)
    hit = np.zeros(len(xy), bool)
    dist = pparams[3]
    for j in range(4, len(pparams) - 1, 2):
        hit |= np.hypot(pparams[j] - xy[:, 0], pparams[j + 1] - xy[:, 1]) < dist
    return np.nonzero(hit)[0] + 1


@pytest.mark.parametrize("geom,kind", [("NONE", "POINTN"), ("CANYON", "POINTD")])
def test_point_nodes_are_the_nodes_within_the_distance(geom, kind):
    m = workloads.build("point_source", scale=0.15, steps=20, geom=geom, kind=kind)
    p = m.problem
    assert p.point_kind == (EXFEM_POINT_FORCE if kind == "POINTN" else EXFEM_POINT_DISP)
    assert p.nseismic == 0 and not p.waves and p.nrhs == 1
    deck = decks.point_source(scale=0.15, steps=20, geom=geom, kind=kind)
    line = deck.split("PROBLEM:\n")[1].split("\n")[1].split()
    pparams = [float(v) for v in line[1:]]
    assert np.array_equal(m.point_nodes(), brute_force_nodes(m, pparams))
    assert (p.point_amp, p.point_sigma, p.point_t0) == tuple(pparams[:3])
    if geom == "CANYON":   # the rim source reaches hanging nodes
        assert len(set(m.point_nodes()) & set(m.hanging()[:, 0])) > 0


def test_point_decks_reject_plane_wave_rhs_and_bad_sigma():
    d = decks.point_source(scale=0.15, steps=20)
    with pytest.raises(ExfemError):
        Model(d + "RHS:\n1\nWAVEP 0.0 1.0 2.0 1.0\n")
    bad = d.replace("PROBLEM:\nPOINTN\n6 1000000.0 0.01", "PROBLEM:\nPOINTN\n6 1000000.0 -0.01")
    assert bad != d
    with pytest.raises(ExfemError):
        Model(bad)


def test_vertical_surface_force_gives_a_mirror_symmetric_response():
    """A vertical force at the middle of a homogeneous rectangle's surface:
    u_x is odd and u_y even about the middle, at every receiver pair and
    every saved step (up to the summation-order rounding of mirrored dofs)."""
    m = workloads.build("point_source", scale=0.25, steps=600, save_every=2, geom="NONE", kind="POINTN")
    o = oracle.run(m, nthreads=4)
    s = o["seis"]                    # (nsave, nrecv, 2)
    xy, _ = m.receivers()            # x = (k + 1) * spacing (find_highest), source at x = 32 spacings
    nr = s.shape[1]
    assert nr == 64 and np.allclose(xy[:63, 0] + xy[62::-1, 0], 2 * xy[31, 0])
    peak = np.abs(s).max()
    assert peak > 0
    i = np.arange(63)
    assert np.abs(s[:, i, 0] + s[:, 62 - i, 0]).max() <= 1e-9 * peak
    assert np.abs(s[:, i, 1] - s[:, 62 - i, 1]).max() <= 1e-9 * peak
    assert np.abs(s[:, :, 1]).max() > 10 * np.abs(s[:, :, 0]).max() * 1e-3


@pytest.mark.parametrize("steps", [0, 37])
def test_prescribed_displacement_holds_the_pulse(steps):
    """POINTD: every non-hanging source node's vertical displacement is the
    pulse at t = steps*dt - start; the horizontal one is free."""
    m = workloads.build("point_source", scale=0.15, steps=60, geom="CANYON", kind="POINTD", save_every=1)
    p = m.problem
    o = oracle.run(m, nsteps=steps, nthreads=4)
    hang = set(m.hanging()[:, 0].tolist())
    want = ricker_point(p.point_amp, p.point_sigma, steps * p.deltat - p.point_t0)
    nodes = [n for n in m.point_nodes() if steps == 0 or n not in hang]
    got = o["u"][2 * (np.array(nodes) - 1) + 1]
    assert np.allclose(got, want, rtol=1e-14, atol=0)
