"""ANIMAT sampling on the GPU (exfem_gpu_sample_points) against visu_field
restated on the oracle's displacement: FP64 at 1e-12, FP32 at 1e-4 of the
field's peak; and the frame files of the driver."""
import os

import numpy as np
import pytest

from exfem import workloads
from exfem.abi import EXFEM_FP32_KAHAN
from exfem.animat import animate
from exfem.gpu import Solver
from oracle import oracle

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 8


def visu_field(m, u, pts, elem, time):
    """visu_field (visualization.f90:156-181) on a reference-order u."""
    xy = m.nodes().reshape(-1, 2)
    cor = m.corners() - 1
    p = m.problem
    out = np.zeros((len(pts), 2))
    w = m.waves()
    for i, (pt, e) in enumerate(zip(pts, elem)):
        if e == 0:
            continue
        c = cor[e - 1]
        r = 2 * (pt[0] - xy[c[0], 0]) / (xy[c[2], 0] - xy[c[0], 0]) - 1
        s = 2 * (pt[1] - xy[c[0], 1]) / (xy[c[2], 1] - xy[c[0], 1]) - 1
        r, s = min(1, max(-1, r)), min(1, max(-1, s))
        n = np.array([(1 - r) * (1 - s), (1 + r) * (1 - s), (1 + r) * (1 + s), (1 - r) * (1 + s)]) / 4
        out[i] = [n @ u[2 * c], n @ u[2 * c + 1]]
        if w and (pt[0] < p.wbox[0] - 1e-9 or pt[0] > p.wbox[1] + 1e-9 or pt[1] > p.wbox[2] + 1e-9):
            f = oracle.planewave(w[0].kind, w[0].amp, p.walpha, p.wbeta, w[0].angle, w[0].freq, time - w[0].t0,
                                 pt[0] - p.worigin[0], pt[1] - p.worigin[1])
            out[i] += f[:, 0]
    return out


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (EXFEM_FP32_KAHAN, 1e-4)])
@pytest.mark.parametrize("name", ["canyon", "point_source"])
def test_sampled_field_matches_visu_field_on_the_oracle_state(name, precision, tol):
    kw = {"geom": "CANYON"} if name == "point_source" else {}
    m = workloads.build(name, scale=0.15, steps=400, save_every=4, **kw)
    xy = m.nodes().reshape(-1, 2)
    g = m.grid(0.0, xy[:, 0].max(), 0.0, xy[:, 1].max(), 15.0)
    assert 0 < g["nfound"] < len(g["elem"])
    o = oracle.run(m, nthreads=NT)
    want = visu_field(m, o["u"], g["points"], g["elem"], m.problem.nsteps * m.problem.deltat)
    with Solver(m, precision=precision) as s:
        s.init_explicit()
        s.run()
        got = s.sample_points(g["points"], g["elem"])
    assert np.abs(want).max() > 0
    assert np.abs(got - want).max() <= tol * np.abs(want).max()
    assert (got[g["elem"] == 0] == 0).all()


def test_animate_writes_one_frame_per_saved_step(tmp_path):
    m = workloads.build("canyon", scale=0.12, steps=40, save_every=8)
    xy = m.nodes().reshape(-1, 2)
    g, frames = animate(m, tmp_path, 0.0, xy[:, 0].max(), 0.0, xy[:, 1].max(), 20.0)
    assert [os.path.basename(f) for f in frames] == ["exfem.%05d.vtu" % k for k in range(1, 40 // 8 + 2)]
    assert (tmp_path / "mater.vtu").exists()
    head = open(frames[-1]).read(400)
    assert 'NumberOfPoints="%d" NumberOfCells="%d"' % (len(g["elem"]), len(g["eptr"]) - 1) in head
