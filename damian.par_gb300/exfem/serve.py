"""Python view of the serving C ABI (include/exfem_srv.h): continuous
batching of many site-response solves on one GPU.

    from exfem.serve import Server
    with Server(hbm_budget=8 << 30) as srv:
        rid = srv.submit(model, nsteps)
        for res in srv.wait_all():
            seis = srv.fetch(res)

run_stream() replays a timed request stream (Poisson arrivals) against a
server and reports p50/p99 latency and throughput.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from .abi import SRV_SYMBOLS, ExfemError, SrvOpts, SrvResult, bind
from .gpu import default_opts, gpu_lib

_srv_lib = None


def srv_lib():
    global _srv_lib
    if _srv_lib is None:
        _srv_lib = bind(gpu_lib(), SRV_SYMBOLS)
    return _srv_lib


class Server:
    def __init__(self, hbm_budget=0, max_active=16, chunk_steps=256, preparers=4, max_bypass=8, **solver_opts):
        L = srv_lib()
        o = SrvOpts()
        L.exfem_srv_default_opts(C.byref(o))
        o.hbm_budget = int(hbm_budget)
        o.max_active = int(max_active)
        o.chunk_steps = int(chunk_steps)
        o.preparers = int(preparers)
        o.max_bypass = int(max_bypass)
        so = default_opts(**{"precision": 1, "drm_inline": 1, **solver_opts})
        o.solver = so
        h = C.c_void_p()
        rc = L.exfem_srv_open(C.byref(o), C.byref(h))
        if rc != 0:
            raise ExfemError(rc, "exfem_srv_open failed")
        self.h = h
        self.L = L
        self.models = {}
        self.results = {}

    def submit(self, model, nsteps=None):
        nsteps = model.problem.nsteps if nsteps is None else int(nsteps)
        rid = C.c_longlong()
        rc = self.L.exfem_srv_submit(self.h, C.byref(model.mesh), C.byref(model.problem), nsteps, C.byref(rid))
        if rc != 0:
            raise ExfemError(rc, self.L.exfem_srv_last_error(self.h).decode())
        self.models[rid.value] = model
        return rid.value

    def submit_deck(self, deck, nsteps=None):
        """Queue problem.in text; the server meshes it on a worker thread."""
        rid = C.c_longlong()
        rc = self.L.exfem_srv_submit_deck(self.h, deck.encode(), 0 if nsteps is None else int(nsteps), C.byref(rid))
        if rc != 0:
            raise ExfemError(rc, self.L.exfem_srv_last_error(self.h).decode())
        return rid.value

    def poll(self, wait_ms=0, cap=64):
        buf = (SrvResult * cap)()
        n = self.L.exfem_srv_poll(self.h, buf, cap, int(wait_ms))
        out = []
        for i in range(max(n, 0)):
            r = buf[i]
            d = {f: getattr(r, f) for f, _ in SrvResult._fields_}
            self.results[d["id"]] = d
            out.append(d)
        return out

    def fetch(self, rid):
        d = self.results[rid]
        shape = (d["nrhs"], d["nsave"], d["nrecv"], 2)
        out = np.zeros(shape)
        rc = self.L.exfem_srv_fetch(self.h, rid, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
        self.models.pop(rid, None)
        if rc != 0:
            raise ExfemError(rc, self.L.exfem_srv_last_error(self.h).decode())
        return out

    def stats(self):
        w, p, a, pk = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        f, b = C.c_longlong(), C.c_size_t()
        self.L.exfem_srv_stats(self.h, C.byref(w), C.byref(p), C.byref(a), C.byref(f), C.byref(b), C.byref(pk))
        return {"waiting": w.value, "preparing": p.value, "active": a.value, "finished": f.value,
                "bytes": b.value, "peak_active": pk.value}

    def wait_all(self, n, timeout=600.0):
        got = []
        t_end = time.time() + timeout
        while len(got) < n and time.time() < t_end:
            got += self.poll(wait_ms=100)
        return got

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.exfem_srv_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_stream(requests, server_kw=None, keep_seis=False, timeout=3600.0):
    """Replay [(arrival_s, model or deck text, nsteps), ...] in real time
    against a new server (deck text is meshed by the server, inside the
    latency).  Returns per-request records and a summary (p50/p99 latency,
    throughput in elem-steps*rhs/s over the makespan)."""
    server_kw = server_kw or {}
    recs = {}
    with Server(**server_kw) as srv:
        t0 = time.perf_counter()
        pending = sorted(requests, key=lambda r: r[0])
        i = 0
        done = 0
        seis = {}
        while done < len(pending):
            now = time.perf_counter() - t0
            while i < len(pending) and pending[i][0] <= now:
                arr, model, nsteps = pending[i]
                if isinstance(model, str):
                    rid = srv.submit_deck(model, nsteps)
                else:
                    rid = srv.submit(model, nsteps)
                recs[rid] = {"arrival": arr, "submitted": time.perf_counter() - t0, "nsteps": nsteps}
                i += 1
            wait = 0 if i < len(pending) else 50
            if i < len(pending):
                wait = int(max(0.0, min(50.0, (pending[i][0] - now) * 1000.0)))
            for d in srv.poll(wait_ms=wait):
                r = recs[d["id"]]
                r["finished"] = time.perf_counter() - t0
                r["status"] = d["status"]
                r["t_admit"], r["t_ready"], r["t_done"] = d["t_admit"], d["t_ready"], d["t_done"]
                r["t_meshed"], r["t_submit"] = d["t_meshed"], d["t_submit"]   # server clock
                r["nelems"], r["nrhs"], r["nsteps"] = d["nelems"], d["nrhs"], d["nsteps"]
                r["latency"] = r["finished"] - r["arrival"]
                if d["status"] == 0:
                    s = srv.fetch(d["id"])
                    if keep_seis:
                        seis[d["id"]] = s
                done += 1
            if time.perf_counter() - t0 > timeout:
                break
        stats = srv.stats()
    ok = [r for r in recs.values() if r.get("status") == 0]
    lat = np.array([r["latency"] for r in ok]) if ok else np.zeros(1)
    work = sum(r["nelems"] * r["nrhs"] * r["nsteps"] for r in ok)
    first = min(r["arrival"] for r in recs.values())
    last = max(r.get("finished", 0.0) for r in recs.values())
    summary = {"requests": len(recs), "ok": len(ok), "p50_s": float(np.percentile(lat, 50)),
               "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
               "makespan_s": last - first, "throughput": work / max(last - first, 1e-9),
               "unit": "elem-steps*rhs/s", "peak_active": stats["peak_active"]}
    return recs, summary, seis
