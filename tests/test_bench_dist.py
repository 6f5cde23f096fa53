"""bench.py's multi-process path on CPU (gloo, world size 2).

`bench.py --gpus N` runs under torchrun as N independent replicas: each rank
reads RANK / WORLD_SIZE / MASTER_* from its environment, the ranks meet at a
barrier around the timed region, the reported time is the maximum over ranks,
and for `--impl reference` every rank but 0 exits without work.  Two
processes started with that environment exercise the same calls here.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, %(repo)r)
import bench
ws, rank, local, dist, torch = bench.dist_setup()
assert ws == 2 and dist is not None and rank == local
bench.barrier(dist)
t = bench.allreduce_max(dist, torch, 10.0 + 3.0 * rank)   # rank 1's time is the longer one
bench.barrier(dist)

class Args:
    workload = "homogeneous_rectangle"
    scale = 0.25
    steps = 1
    warmup = 1

if rank == 1:
    bench.run_reference(Args(), ws, rank, dist)   # the reference arm runs on rank 0 alone
print(json.dumps({"rank": rank, "t": t, "backend": dist.get_backend()}))
dist.destroy_process_group()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_share_the_max_time():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(r),
                   LOCAL_RANK=str(r), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD % {"repo": REPO}], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            outs.append(p.communicate(timeout=180))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = [json.loads(out.strip().splitlines()[-1]) for out, _ in outs]
    assert sorted(r["rank"] for r in res) == [0, 1]
    assert all(r["backend"] == "gloo" for r in res)
    assert all(r["t"] == 13.0 for r in res)


def test_burst_stream_is_the_documented_sample():
    """The saturated serving burst (and `--burst-request I`) is a fixed,
    seeded sample: 16 canyon/valley decks of 34K-855K elements, 1-16 angles,
    1000-2000 steps; requests 12 and 6 are the 13- and 12-RHS ones the
    served-request profiles cover."""
    import sys
    sys.path.insert(0, REPO)
    import bench
    from exfem.model import Model
    stream = bench.burst_stream(16)
    assert len(stream) == 16 and stream == bench.burst_stream(16)
    models = [Model(d, nsteps=n) for _, d, n in stream]
    sizes = [m.nelems for m in models]
    assert min(sizes) == 34368 and max(sizes) == 854616
    assert all(1 <= m.problem.nrhs <= 16 for m in models)
    assert all(1000 <= n <= 2000 for _, _, n in stream)
    assert (models[12].nelems, models[12].problem.nrhs) == (598038, 13)
    assert (models[6].nelems, models[6].problem.nrhs) == (742906, 12)
