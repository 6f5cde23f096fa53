"""Benchmark of the explicit time loop (damian.par run_explicit) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--form fp64|fp32] [--scale S]

A bench step is one time step of the whole batch of right-hand sides on the
workload's mesh.  Metric: element-steps x RHS per second (N_e * R * steps / s),
inputs resident in HBM, timed with CUDA events on the library's own stream.
Multi-GPU runs are independent replicas (the path shards but is not built
multi-GPU): weak scaling, value = sum over ranks.

--impl reference times the CPU oracle (the C++ restatement of the reference's
per-element loop; the Fortran/MPI reference cannot be built here) with every
host thread, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
for p in (HERE, os.path.join(HERE, "damian.par_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

FORMS = {"fp64": 0, "fp32": 1}
DEFAULT_WORKLOAD = ("valley_batched", "fp32")


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return ws, rank, local, dist, torch
    return 1, 0, local, None, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, torch, x):
    if dist is None:
        return x
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
        mine = [r for r in rows if r[0] == str(self.gpu)] or rows
        if not mine:
            return None
        sm = [float(r[1]) for r in mine if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in mine if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in mine for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(mine)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    except Exception:
        return 6800.0, "fallback"


def kernel_bytes(name, m, R, fp64):
    """Algorithmic bytes one launch of `name` must move (what the roofline uses).

    ne, nn: elements, nodes; ndof = 2 nn; s = state word (8 FP64, 4 FP32).
      k_elem_ref/k_elem64   read u, u- (2*ndof*s*R), element data (conn 16 +
                            (mu,lambda) 16 + mass 8 + damping slot 4), write
                            the element forces 8*s*R per element
      k_node_ref/k_node64   read the element forces once (8*s*R per element),
                            the gather lists (4 B per incidence), m_full 16 per
                            node, write u+ (ndof*s*R)
      k_drm*                read corner coordinates (64 B), write 16 forces*s*R
                            per DRM element
      k_hang*               hanging nodes 3 values in/1 out, receivers
      k_step32/_tile32/_pipe32
                            FP32 increment form, fused: read u_hi, Kahan term
                            and increment, write all three (6*ndof*4*R), read
                            element data (conn 16 + coef 16) and lists
    """
    ne, nn, ns = m.nelems, m.nnodes, m.problem.nseismic
    nh, nr = m.problem.nhanging, m.problem.nrecv
    ndof = 2 * nn
    s = 8 if fp64 else 4
    inc = 4 * ne
    if name in ("k_elem_ref", "k_elem64"):
        return 2 * ndof * s * R + ne * 44 + ne * 8 * s * R
    if name in ("k_node_ref", "k_node64"):
        return ne * 8 * s * R + 4 * inc + 16 * nn + ndof * s * R
    if name.startswith("k_drm"):
        return ns * (64 + 16 * s * R)
    if name.startswith("k_hang"):
        return nh * 2 * 3 * s * R + nr * (4 * 2 * s * R + 2 * 8 * R)
    if name.startswith(("k_step32", "k_tile32", "k_pipe32", "k_mma32")):
        return 6 * ndof * 4 * R + ne * 32 + 4 * inc
    return None


def ncu_traffic(kernel, workload):
    """Per-launch DRAM bytes from the committed ncu summary, if one exists."""
    try:
        with open(os.path.join(HERE, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        v = d.get(workload, {}).get(kernel.split("<")[0])
        return v.get("bytes_per_launch") if isinstance(v, dict) else v
    except Exception:
        return None


def input_bytes(m):
    p, L = m.problem, int(m.eptr()[-1]) - 1
    return (4 * (m.nelems + 1) + 4 * L + L + 16 * m.nnodes + 4 * m.nelems + 40 * p.nmat + 4 * m.nnodes
            + 12 * p.nhanging + 8 * p.nseismic + 40 * p.nrhs + 20 * p.nrecv)


def cpu_baseline(m, target_s=12.0, rhs=0):
    """Oracle on all host threads over a bounded sample (steps chosen for ~target_s)."""
    from oracle import oracle
    nt = os.cpu_count() or 1
    probe = oracle.run(m, rhs=rhs, nsteps=2, nthreads=nt, want_u=False)["seconds"]
    per_step = max(probe / 2.0, 1e-6)
    steps = int(max(1, min(m.problem.nsteps, target_s / per_step)))
    r = oracle.run(m, rhs=rhs, nsteps=steps, nthreads=nt, want_u=False)
    val = m.nelems * steps / r["seconds"]
    return {"value": val, "unit": "elem-steps*rhs/s", "cores": nt, "kind": "port",
            "sample": "oracle per-element FP64 loop, rhs %d, %d of %d steps, %d elements, %d threads"
                      % (rhs, steps, m.problem.nsteps, m.nelems, nt)}


def serving_leg(args, local):
    """Bounded serving sample: Poisson arrivals of uneven canyon/valley
    requests, FP32 with continuous batching, against the same requests run
    serially in plain FP64 (one context at a time)."""
    from exfem import decks
    from exfem.gpu import Solver
    from exfem.model import Model
    from exfem.serve import run_stream
    stream = decks.serving_stream(n=args.serve_requests, rate=20.0, seed=7, min_scale=0.2, max_scale=1.0,
                                  max_angles=16, step_range=(500, 2000))
    # requests arrive as problem.in text: the server meshes them on its worker
    # threads, inside the latency
    recs, summary, _ = run_stream(stream, server_kw={"max_active": 16, "chunk_steps": 128, "device": local})
    mesh_s = [r["t_meshed"] - r["t_submit"] for r in recs.values() if r.get("status") == 0]
    # plain FP64, serially, same requests (meshing included)
    t0 = time.perf_counter()
    work = 0
    sizes = []
    for _, d, n in stream:
        m = Model(d, nsteps=n)
        with Solver(m, device=local) as s:
            s.init_explicit()
            s.run(n)
            s.seismograms()
        work += m.nelems * m.problem.nrhs * n
        sizes.append(m.nelems)
    t64 = time.perf_counter() - t0
    summary.update({"serial_fp64_throughput": work / t64, "serial_fp64_s": t64,
                    "elements_min": min(sizes), "elements_max": max(sizes),
                    "mesh_s_median": float(np.median(mesh_s)) if mesh_s else None,
                    "note": "latency = finish - arrival of the problem.in text (the server meshes it); "
                            "%d requests, Poisson 20/s, 1-16 angles, 500-2000 steps" % len(stream)})
    return summary


def burst_stream(n):
    """The saturated serving burst: n decks sized like the serving config
    (canyons and valleys of 3e4-9e5 elements, 1-16 angles, 1000-2000 steps),
    as (arrival, problem.in text, steps)."""
    from exfem import decks
    return list(decks.serving_stream(n=n, rate=1e9, seed=5, min_scale=0.3, max_scale=1.0, max_angles=16,
                                     step_range=(1000, 2000), canyon_nperlen=25.0, valley_chper=0.07))


def saturated_serving_leg(args, local):
    """Server capacity: a burst of requests sized like the serving config
    (canyons and valleys of 3e4-9e5 elements, 1-16 angles) submitted at once,
    meshed before the clock, so the server stays saturated.  Served
    element-steps*RHS/s = total work / makespan (plan builds, uploads,
    admission and stepping included).  The plain FP64 GPU form is timed on
    every request (CUDA events over 10 steps after 3) and its throughput is
    the same total work over the sum of steps x ms/step."""
    from exfem.gpu import Solver
    from exfem.model import Model
    from exfem.serve import Server
    reqs = [(Model(d, nsteps=n), n) for _, d, n in burst_stream(args.serve_burst)]
    work = sum(m.nelems * m.problem.nrhs * n for m, n in reqs)
    with Server(max_active=16, chunk_steps=256, device=local) as srv:
        ids = [srv.submit(m, n) for m, n in reqs]
        res = srv.wait_all(len(ids))
    ok = [r for r in res if r["status"] == 0]
    makespan = max(r["t_done"] for r in ok) - min(r["t_submit"] for r in ok) if ok else None
    lat = sorted(r["t_done"] - r["t_submit"] for r in ok)
    t64 = 0.0
    for m, n in reqs:
        with Solver(m, device=local) as s:
            s.init_explicit()
            s.run(3)
            s.sync()
            ms = C.c_double(0)
            if s.lib.exfem_gpu_run_timed(s.h, 10, C.byref(ms)) != 0:
                return {"error": "fp64 timing failed"}
        t64 += n * ms.value / 10.0 / 1000.0
    served = work / makespan if makespan else None
    sizes = [m.nelems for m, _ in reqs]
    # algorithmic HBM bytes of the served steps (the FP32 step kernel's and the
    # hanging/receiver pass's, as in the roofline) over the makespan
    abytes = sum(n * ((kernel_bytes("k_step32", m, m.problem.nrhs, False) or 0) +
                      (kernel_bytes("k_hang32", m, m.problem.nrhs, False) or 0)) for m, n in reqs)
    peak, peak_kind = measured_peaks()
    served_gbs = abytes / makespan / 1e9 if makespan else None
    return {"requests": len(reqs), "ok": len(ok), "work": work, "makespan_s": makespan,
            "served_throughput": served, "fp64_throughput": work / t64, "unit": "elem-steps*rhs/s",
            "ratio_served_fp32_over_fp64": (served / (work / t64)) if served else None,
            "served_algorithmic_gbs": served_gbs,
            "served_hbm_frac": (served_gbs / peak) if (served_gbs and peak) else None, "peak_kind": peak_kind,
            "p50_s": lat[len(lat) // 2] if lat else None, "p99_s": lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
            "elements_min": min(sizes), "elements_max": max(sizes),
            "note": "burst of %d requests submitted at once (meshed beforehand), 1000-2000 steps, 1-16 angles; "
                    "fp64 = plain FP64 GPU form, per-request ms/step x steps" % len(reqs)}


def accuracy_leg(args, local, tuned):
    """Seismogram error of the FP32 form against the plain FP64 form (which
    matches the oracle to 1e-12), relative L2 and peak amplitude per receiver
    (the metrics of tests/util.py):
      - the timed workload itself, the 64-RHS valley, every RHS over
        `accuracy_batched_steps` steps with the bench's tuned shapes;
      - the valley with one SV wave at full length (20000 steps)."""
    from exfem import workloads
    from exfem.gpu import Solver
    sys.path.insert(0, os.path.join(HERE, "tests"))
    from util import peak_rel, per_receiver_rel

    def pair(m, kw32):
        """Seismograms of both forms over the whole run, and each form's
        device time per step (CUDA events around the run on its stream)."""
        seis, us = {}, {}
        for prec in (1, 0):
            with Solver(m, precision=prec, device=local, **(kw32 if prec == 1 else {})) as s:
                s.init_explicit()
                ms = C.c_double(0)
                if s.lib.exfem_gpu_run_timed(s.h, m.problem.nsteps, C.byref(ms)) != 0:
                    raise RuntimeError("timed run failed")
                s.sync()
                seis[prec] = s.seismograms()
                us[prec] = 1000.0 * ms.value / m.problem.nsteps
        return seis, us

    out = {"against": "plain FP64 GPU form (matches the oracle to 1e-12)", "tolerance": 1e-4}
    if args.accuracy_batched_steps > 0:
        mb = workloads.build(args.workload, scale=args.scale, steps=args.accuracy_batched_steps)
        seis, _ = pair(mb, tuned)
        l2 = [float(per_receiver_rel(seis[1][r], seis[0][r]).max()) for r in range(mb.problem.nrhs)]
        pk = [float(peak_rel(seis[1][r], seis[0][r]).max()) for r in range(mb.problem.nrhs)]
        out.update({"workload": args.workload, "elements": mb.nelems, "rhs": mb.problem.nrhs,
                    "steps": mb.problem.nsteps, "max_rel_l2": max(l2), "median_rel_l2": float(np.median(l2)),
                    "max_peak_rel": max(pk), "per_rhs_rel_l2": [round(v, 10) for v in l2],
                    "worst_rhs": int(np.argmax(l2))})
    if args.accuracy_steps > 0:
        m = workloads.build("valley", scale=args.scale, steps=args.accuracy_steps)
        seis, us = pair(m, {})
        out["valley_full_length"] = {
            "workload": "valley", "elements": m.nelems, "rhs": m.problem.nrhs, "steps": m.problem.nsteps,
            "max_rel_l2": float(per_receiver_rel(seis[1][0], seis[0][0]).max()),
            "max_peak_rel": float(peak_rel(seis[1][0], seis[0][0]).max()),
            "fp32_us_per_step": round(us[1], 2), "fp64_us_per_step": round(us[0], 2),
            "timing": "device time of the whole run (CUDA events on the context's stream), default shapes"}
    return out


def config4_leg(args, local):
    """The serving config as specified: Poisson arrivals at 20/s of
    problem.in texts (canyons and valleys of 1e4-3e6 elements, 1-16 angles,
    1000-20000 steps), meshed and served by the server.  At these sizes the
    offered load is many times one GPU's capacity, so latency is queueing;
    throughput is the work over the makespan.  The plain FP64 form is timed
    (10 steps after 3) on every `stride`-th request and the serial FP64 time
    of the whole stream is the sampled seconds per unit of work times the
    stream's work."""
    from exfem import decks
    from exfem.gpu import Solver
    from exfem.model import Model
    from exfem.serve import run_stream
    stream = decks.serving_stream(n=args.config4_requests, rate=20.0, seed=11, min_scale=0.2, max_scale=1.0,
                                  max_angles=16, step_range=(1000, 20000), canyon_nperlen=25.0, valley_chper=0.045)
    recs, summary, _ = run_stream(stream, server_kw={"max_active": 16, "chunk_steps": 256, "device": local},
                                  timeout=3000.0)
    ok = [r for r in recs.values() if r.get("status") == 0]
    sizes = sorted(r["nelems"] for r in ok)
    work = sum(r["nelems"] * r["nrhs"] * r["nsteps"] for r in ok)
    stride = max(1, len(stream) // 32)
    w64 = t64 = 0.0
    for _, d, n in stream[::stride]:
        m = Model(d, nsteps=n)
        with Solver(m, device=local) as s:
            s.init_explicit()
            s.run(3)
            s.sync()
            ms = C.c_double(0)
            if s.lib.exfem_gpu_run_timed(s.h, 10, C.byref(ms)) != 0:
                break
        w64 += m.nelems * m.problem.nrhs * n
        t64 += n * ms.value / 10.0 / 1000.0
    fp64 = w64 / t64 if t64 > 0 else None
    summary.update({"mode": "serving_config4", "work": work, "elements_min": sizes[0] if sizes else None,
                    "elements_p50": sizes[len(sizes) // 2] if sizes else None,
                    "elements_max": sizes[-1] if sizes else None,
                    "offered_load": 20.0 * work / max(len(ok), 1),
                    "fp64_throughput_sampled": fp64, "fp64_sample_requests": len(stream[::stride]),
                    "ratio_served_fp32_over_fp64": summary["throughput"] / fp64 if fp64 else None,
                    "note": "%d requests, Poisson 20/s, 1-16 angles, 1000-20000 steps, meshed by the server; "
                            "plain FP64 timed on every %d-th request" % (len(stream), stride)})
    return summary


def reference_model(workload, scale, steps):
    """The workload's mesh and problem as plain arrays: meshed by a child
    process (which maps the host library) and loaded here, so the process the
    reference arm times maps the oracle alone."""
    from oracle.model_arrays import ArrayModel
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "model.npz")
        code = ("import sys; sys.path[:0] = [%r, %r]; from exfem import workloads; "
                "from oracle import model_arrays; "
                "model_arrays.dump(workloads.build(%r, scale=%r, steps=%d), %r)"
                % (HERE, os.path.join(HERE, "damian.par_gb300"), workload, float(scale), int(steps), path))
        subprocess.run([sys.executable, "-c", code], check=True)
        return ArrayModel(path)


def run_reference(args, ws, rank, dist):
    if rank != 0:
        return
    m = reference_model(args.workload, args.scale, 20000)
    from oracle import oracle
    nt = os.cpu_count() or 1
    probe = oracle.run(m, nsteps=2, nthreads=nt, want_u=False)["seconds"] / 2.0
    budget = 150.0 / max(args.steps + args.warmup, 1)      # whole run within a few minutes
    sample = int(max(1, min(m.problem.nsteps, budget / max(probe, 1e-6))))
    secs = []
    for i in range(args.warmup + args.steps):
        r = oracle.run(m, nsteps=sample, nthreads=nt, want_u=False)
        if i >= args.warmup:
            secs.append(r["seconds"])
    t = float(np.mean(secs))
    val = m.nelems * sample / t
    out = {"metric": "elem-steps/s", "value": val, "unit": "elem-steps*rhs/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 * t / sample, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.workload, "scale": args.scale, "elements": m.nelems, "rhs_timed": 1,
                      "sample_steps": sample},
           "impl": "reference",
           "cpu_baseline": {"value": val, "unit": "elem-steps*rhs/s", "cores": nt, "kind": "port",
                            "sample": "%d time steps of rhs 0 per bench step" % sample},
           "e2e": {"value": val, "unit": "elem-steps*rhs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_ours(args, ws, rank, local, dist, torch):
    from exfem import workloads
    from exfem.abi import ExfemError
    from exfem.gpu import Solver

    form = FORMS[args.form]
    fp64 = form == 0
    total = args.warmup + args.steps
    if args.burst_request >= 0:
        # one request of the saturated serving burst, timed alone
        from exfem.model import Model
        m = Model(burst_stream(args.serve_burst)[args.burst_request][1], nsteps=max(total, 8))
        args.workload = "burst request %d of %d" % (args.burst_request, args.serve_burst)
        args.no_extras = True
    else:
        m = workloads.build(args.workload, scale=args.scale, steps=max(total, 8))
    R = m.problem.nrhs
    tuned = {}
    if args.block or args.rpt or args.variant >= 0:
        tuned = {k: v for k, v in (("block_threads", args.block), ("rhs_per_thread", args.rpt)) if v}
        if args.variant >= 0:
            tuned["variant"] = args.variant
    elif not fp64 and not args.no_extras:
        from exfem import autotune
        mt = workloads.build(args.workload, scale=args.scale, steps=24)
        choice = autotune.tune(mt, steps=10, warmup=3, device=local)
        tuned = {"variant": choice["variant"], "block_threads": choice["block_threads"],
                 "rhs_per_thread": choice["rhs_per_thread"]}
        del mt
    s = Solver(m, precision=form, device=local, **tuned)
    s.init_explicit()
    s.run(args.warmup)
    s.sync()
    barrier(dist)
    clk = ClockSampler(local).start() if rank == 0 else None
    l0 = s.launches
    ms = C.c_double(0)
    rc = s.lib.exfem_gpu_run_timed(s.h, int(args.steps), C.byref(ms))
    if rc != 0:
        raise ExfemError(rc, s.lib.exfem_gpu_last_error(s.h).decode())
    s.sync()
    launches = s.launches - l0
    clocks = clk.stop() if clk else None
    barrier(dist)
    t_ms = allreduce_max(dist, torch, ms.value)
    s.close()
    value = ws * m.nelems * R * args.steps / (t_ms / 1000.0)
    if args.no_extras:
        if rank == 0:
            print(json.dumps({"metric": "elem-steps/s", "value": value, "unit": "elem-steps*rhs/s", "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
                              "config": {"workload": args.workload, "form": args.form, "scale": args.scale,
                                         "elements": m.nelems, "rhs": R}, "tuned": tuned or None,
                              "gpu_launches": launches, "clocks": clocks, "mode": "timed loop only"}))
        return

    # per-kernel CUDA-event times on a fresh context (no graph, same stream)
    prof_steps = max(4, min(64, args.steps))
    mp = workloads.build(args.workload, scale=args.scale, steps=prof_steps + 2)
    sp = Solver(mp, precision=form, device=local, **tuned)
    sp.init_explicit()
    sp.run(2)
    ms_arr = (C.c_double * 16)()
    nm_arr = (C.c_char_p * 16)()
    nk = sp.lib.exfem_gpu_profile_kernels(sp.h, prof_steps, ms_arr, nm_arr, 16)
    kern = {nm_arr[i].decode(): ms_arr[i] for i in range(max(nk, 0))}
    sp.close()
    dom = max(kern, key=lambda k: kern[k]) if kern else None
    peak, peak_kind = measured_peaks()
    roof = None
    if dom:
        b = kernel_bytes(dom, m, R, fp64)
        achieved = b / (kern[dom] / 1000.0) / 1e9 if b else None
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "traffic": ncu_traffic(dom, args.workload), "algorithmic_bytes": b,
                "kernel_ms": kern[dom], "kernels_ms": kern}

    # end to end through the C ABI with host buffers: create (uploads) + init +
    # run + seismogram read-back
    e2e_steps = args.steps
    me = workloads.build(args.workload, scale=args.scale, steps=e2e_steps)
    t_req = []
    for _ in range(3):   # three requests; the median is reported
        t0 = time.perf_counter()
        se = Solver(me, precision=form, device=local, **tuned)
        se.init_explicit(want_mfull=False)   # the request's result is its seismograms
        se.run(e2e_steps)
        seis = se.seismograms()
        h2d, d2h = se.copy_bytes()
        se.close()
        t_req.append(time.perf_counter() - t0)
    t_e2e = sorted(t_req)[1]
    e2e = {"value": ws * me.nelems * R * e2e_steps / t_e2e, "unit": "elem-steps*rhs/s",
           "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
           "h2d_bytes_per_request": h2d, "d2h_bytes_per_request": d2h, "input_bytes": input_bytes(me),
           "seismogram_bytes": int(seis.nbytes), "request_s": [round(t, 4) for t in t_req],
           "note": "a request of %d time steps: create (host plan + uploads) + init_explicit + the steps + "
                   "seismograms, median of 3; byte counts are the context's own host<->device copies, per "
                   "request and divided by its time steps" % e2e_steps}

    # the plain FP64 form on the same workload, for the FP32 / FP64 ratio
    fp64_ref = None
    if not fp64 and args.fp64_steps > 0:
        mf = workloads.build(args.workload, scale=args.scale, steps=args.fp64_steps + 3)
        sf = Solver(mf, device=local)
        sf.init_explicit()
        sf.run(3)
        sf.sync()
        msf = C.c_double(0)
        rc = sf.lib.exfem_gpu_run_timed(sf.h, int(args.fp64_steps), C.byref(msf))
        sf.close()
        if rc == 0:
            v64 = ws * mf.nelems * R * args.fp64_steps / (msf.value / 1000.0)
            fp64_ref = {"value": v64, "ms_per_step": msf.value / args.fp64_steps, "steps": args.fp64_steps,
                        "ratio_fp32_over_fp64": value / v64}
        del mf

    serving = serving_leg(args, local) if args.serve_requests > 0 else None
    accuracy = (accuracy_leg(args, local, tuned)
                if (not fp64 and (args.accuracy_steps > 0 or args.accuracy_batched_steps > 0) and rank == 0)
                else None)
    if serving is not None and args.serve_burst > 0:
        serving["saturated"] = saturated_serving_leg(args, local)
    if serving is not None and args.config4_requests > 0:
        serving["config4"] = config4_leg(args, local)

    if rank != 0:
        return
    cpu = cpu_baseline(m) if ws == 1 else None
    out = {"metric": "elem-steps/s", "value": value, "unit": "elem-steps*rhs/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if fp64 else "f32+kahan", "data": "synthetic (seeded deck)",
           "config": {"workload": args.workload, "form": args.form, "scale": args.scale, "elements": m.nelems,
                      "nodes": m.nnodes, "rhs": R, "hanging": m.problem.nhanging,
                      "l2": "no flush: a bench step is one time step; the state of this workload is %.1f MB"
                            % ((2 * m.nnodes * R * (8 if fp64 else 4) * (2 if fp64 else 4)) / 1e6),
                      "parallelism": "replicas" if ws > 1 else "single"},
           "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
           "accuracy": accuracy,
           "tuned": tuned or None, "plain_fp64": fp64_ref, "serving": serving}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD[0])
    ap.add_argument("--form", default=DEFAULT_WORKLOAD[1], choices=sorted(FORMS))
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--no-extras", action="store_true",
                    help="timed loop only (no autotune, kernel profile, e2e, CPU or FP64 legs): for ncu captures")
    ap.add_argument("--block", type=int, default=0, help="force the step kernel's block size")
    ap.add_argument("--rpt", type=int, default=0, help="force right-hand sides per thread")
    ap.add_argument("--variant", type=int, default=-1, help="force the kernel variant (FP32: 0 direct gather, 1 shared-memory tiles, 2 bulk-copy "
                         "pipeline, 3 tensor-core step, 4 persistent direct gather, 5 list-form direct gather; "
                         "FP64: 0 reference order, 1 closed form)")
    ap.add_argument("--serve-requests", type=int, default=32, help="requests in the serving sample (0: skip)")
    ap.add_argument("--serve-burst", type=int, default=16, help="requests in the saturated serving sample (0: skip)")
    ap.add_argument("--burst-request", type=int, default=-1,
                    help="time request I of the saturated serving burst alone (timed loop only)")
    ap.add_argument("--fp64-steps", type=int, default=10, help="steps of the plain FP64 form timed for comparison")
    ap.add_argument("--accuracy-steps", type=int, default=20000,
                    help="steps of the FP32-vs-FP64 seismogram comparison on the one-wave valley (0: skip)")
    ap.add_argument("--accuracy-batched-steps", type=int, default=2000,
                    help="steps of the FP32-vs-FP64 comparison of every RHS of the timed workload (0: skip)")
    ap.add_argument("--serve-config4", action="store_true",
                    help="only the serving config as specified (512 requests, minutes of GPU time); prints its own line")
    ap.add_argument("--config4-requests", type=int, default=512,
                    help="requests of the serving config run inside the default line (serving.config4; 0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local, dist, torch = dist_setup()
    if args.serve_config4:
        if rank == 0:
            print(json.dumps(config4_leg(args, local)))
    elif args.impl == "reference":
        run_reference(args, ws, rank, dist)
    else:
        run_ours(args, ws, rank, local, dist, torch)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
