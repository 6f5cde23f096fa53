"""The oracle on a model handed over as plain arrays (oracle/model_arrays.py,
the reference arm's input path) gives the same results as on the built
model, and a process that loads the arrays maps the oracle and no product
library."""
import os
import subprocess
import sys

import numpy as np

from exfem import workloads
from oracle import model_arrays, oracle

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def test_array_model_runs_the_oracle_identically(tmp_path):
    m = workloads.build("canyon", scale=0.12, steps=60, save_every=2, refine_band=20)
    path = str(tmp_path / "m.npz")
    model_arrays.dump(m, path)
    a = model_arrays.ArrayModel(path)
    assert (a.nelems, a.nnodes, a.problem.nrhs) == (m.nelems, m.nnodes, m.problem.nrhs)
    for r in (0, m.problem.nrhs - 1):
        x = oracle.run(m, rhs=r, nthreads=2)
        y = oracle.run(a, rhs=r, nthreads=2)
        for k in ("mfull", "seis", "u"):
            assert np.array_equal(x[k], y[k]), (r, k)


def test_reference_arm_process_maps_no_product_library():
    code = ("import sys; sys.path[:0] = [%r, %r]; import bench; from oracle import oracle; "
            "m = bench.reference_model('homogeneous_rectangle', 0.125, 40); "
            "oracle.run(m, nsteps=4, nthreads=1, want_u=False); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libexfem_oracle' in maps; "
            "assert 'libexfem_host' not in maps and 'libexfem_gpu' not in maps; print('ok')"
            % (REPO, os.path.join(REPO, "damian.par_gb300")))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stderr[-2000:]
