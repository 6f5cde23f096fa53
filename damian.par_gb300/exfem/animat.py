"""ANIMAT visualisation (create_visualization / visualize_solution,
visualization.f90:24-54, 192-284) from the device-resident state.

The reference samples every saved step.bin offline on a grid.  Here the grid
is located once on the host (exfem_model_grid), and the solver samples its
current state with exfem_gpu_sample_points every io_interval steps.  That is
the same visu_field interpolation at the same times, with no step.bin in
between.  Files are those of print_vtkun_mater/print_vtkun_field
(io_utils.f90:442-467): mater.vtu with (material, vp), then exfem.NNNNN.vtu
per saved step (frame = saved step + 1), written by exfem_write_vtu.
"""
from __future__ import annotations

import os

from .abi import EXFEM_FP64
from .gpu import Solver
from .model import write_vtu


def animate(model, outdir, xmin, xmax, ymin, ymax, dist, rhs=0, nsteps=None, precision=EXFEM_FP64, **opts):
    """Writes mater.vtu and one exfem.NNNNN.vtu per saved step into outdir;
    returns the grid (exfem.Model.grid) and the list of frame paths."""
    os.makedirs(outdir, exist_ok=True)
    g = model.grid(xmin, xmax, ymin, ymax, dist)
    write_vtu(os.path.join(outdir, "mater.vtu"), g["eptr"], g["eind"], g["points"], g["material"], "material")
    io = model.problem.io_interval
    total = model.problem.nsteps if nsteps is None else int(nsteps)
    frames = []
    with Solver(model, precision=precision, **opts) as s:
        s.init_explicit()
        save = 0
        while True:
            field = s.sample_points(g["points"], g["elem"], rhs)
            path = os.path.join(outdir, "exfem.%05d.vtu" % (save + 1))
            write_vtu(path, g["eptr"], g["eind"], g["points"], field, "displacements")
            frames.append(path)
            if s.steps_done + io > total:
                break
            s.run(io)
            save += 1
    return g, frames
