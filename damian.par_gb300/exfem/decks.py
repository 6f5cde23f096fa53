"""Seeded synthetic problem decks for the five workloads of this path.

Each function returns the text of a problem.in deck (io.cpp:113-228 format,
plus the RECEIVERS/RHS/REFINE/HETEROGENEITY extension sections that
include/exfem_host.h documents).  ``scale`` shrinks the domain while keeping
the element size, materials and wave content, so the same physics runs at
sizes a CPU oracle finishes in seconds.

Workloads (sizes at scale=1):
  homogeneous_rectangle  4000x2000 m, 256x128 Q4 (15.625 m), SV 0 deg, fc 2 Hz, 4000 steps
  canyon                 6000x3000 m half-space, r = 500 m canyon, two rim levels,
                         P/SV at 0-60 deg (SV kept sub-critical), fc 3 Hz, 8000 steps
  valley                 12000x4000 m, semi-elliptical valley a=1500 b=400, four
                         quadtree levels, +-10% log-normal heterogeneity, SV fc 5 Hz
  valley_batched         the valley mesh with 64 right-hand sides
  serving_stream         seeded canyon/valley requests with Poisson arrivals
  point_source           POINTN/POINTD Ricker source (model.f90:1051-1078) on the
                         rectangle or the refined canyon
"""
from __future__ import annotations

import math

import numpy as np

HEADER = "PROBLEM FILE EXFEM\n"
ROCK_HALFSPACE = "p 2000 s 1000 2000"


def _deck(width, height, time, inttime, chper, nperlen, sperlen, materials, prob, pparams,
          geom="NONE", gparams=(), receivers=None, rhs=None, refine=None, heterogeneity=None):
    lines = [HEADER.rstrip("\n"), "DOMAIN:", "%r %r" % (float(width), float(height)),
             "TIME:", "%r %r" % (float(time), float(inttime)),
             "CH PERIOD:", "%r" % float(chper),
             "CONTROL:", "%r %r" % (float(nperlen), float(sperlen)),
             "MATERIALS:", str(len(materials)), *materials,
             "PROBLEM:", prob, " ".join([str(len(pparams))] + ["%r" % float(v) for v in pparams]),
             "GEOMETRY:", geom, " ".join([str(len(gparams))] + ["%r" % float(v) for v in gparams])]
    if receivers is not None:
        lines += ["RECEIVERS:", "%r %r %r" % tuple(float(v) for v in receivers)]
    if rhs:
        lines += ["RHS:", str(len(rhs))]
        for kind, angle, amp, freq, t0 in rhs:
            lines.append("%s %r %r %r %r" % (kind, float(angle), float(amp), float(freq), float(t0)))
    if refine is not None:
        lines += ["REFINE:", "%d %r" % (int(refine[0]), float(refine[1]))]
    if heterogeneity is not None:
        lines += ["HETEROGENEITY:", "%r %d" % (float(heterogeneity[0]), int(heterogeneity[1]))]
    return "\n".join(lines) + "\n"


def rest_delay(kind, angle, freq, box_w, box_h, x0_rel, vp, vs, margin=1.2):
    """Smallest time-to-origin that keeps the incident pulse out of the DRM box
    at t = 0 (the model starts from rest): the earliest arrival over the box
    corners, t0 + v1 with v1 = (x sin - z cos)/v of the incident ray
    (pwaves.f90:153, 189), plus `margin`/fc for the wavelet's half-width."""
    if kind == "WAVEP":
        v, sa, ca = vp, math.sin(angle), math.cos(angle)
    else:
        v, sa, ca = vs, math.sin(angle), math.cos(angle)
    worst = 0.0
    for x in (x0_rel - box_w / 2.0, x0_rel + box_w / 2.0):
        for z in (0.0, box_h):
            worst = max(worst, -(x * sa - z * ca) / v)
    return worst + margin / freq


def homogeneous_rectangle(scale=1.0, steps=4000, angle=0.0, kind="WAVESV", freq=2.0, save_every=1, t0=1.0):
    """Plain FP64 workload: 256x128 square Q4 at 15.625 m, dt = 0.5 CFL.

    The deck gives h = chper*vs/nperlen = 0.15625*1000/10 = 15.625 m and
    dt = h/(vp*sperlen) = 3.90625e-3 s (formulation.f90:20-25).  The DRM box is
    3000 m wide and 375 m deep so that the 1 s delay keeps the pulse outside
    the box at t = 0."""
    h = 15.625
    ncol = max(8, int(round(256 * scale)))
    nrow = max(4, int(round(128 * scale)))
    width, height = ncol * h, nrow * h
    dt = h / (2000.0 * 2.0)
    box_w, box_h = 0.75 * width, min(375.0, 0.75 * height)
    x0 = 0.5 * width
    pparams = [box_w, box_h, x0, 0.0, 1, t0, angle, 1.0, freq]
    recv_dist = width / 64.0
    return _deck(width, height, steps * dt, save_every * dt, 0.15625, 10, 2, [ROCK_HALFSPACE],
                 kind, pparams, receivers=(0.0, width - recv_dist, recv_dist))


def canyon(scale=1.0, steps=8000, radius=500.0, nperlen=25.0, waves=None, refine_levels=2,
           refine_band=60.0, freq=3.0, save_every=4):
    """Semicircular canyon cut into a half-space; two extra quadtree levels
    around the rim (REFINE:).  h = 0.25*1000/nperlen (10 m at nperlen 25).
    SV stays below the critical angle asin(vs/vp) = 30 deg (pwaves.f90:76-89)."""
    width, height = 6000.0 * scale, 3000.0 * scale
    radius = radius * scale
    h = 0.25 * 1000.0 / nperlen
    hmin = h / (2 ** refine_levels)
    dt = hmin / (2000.0 * 2.0)
    if waves is None:
        waves = [("WAVEP", 0.0), ("WAVEP", 30.0), ("WAVEP", 60.0),
                 ("WAVESV", 0.0), ("WAVESV", 15.0), ("WAVESV", 25.0)]
    box_w = max(2000.0 * scale, 2.0 * radius + 8 * h)
    box_h = max(1000.0 * scale, radius + 4 * h)
    rhs = [(k, math.radians(a), 1.0, freq, rest_delay(k, math.radians(a), freq, box_w, box_h, 0.0, 2000.0, 1000.0))
           for k, a in waves]
    pparams = [box_w, box_h, width / 2, 0.0, 1, rhs[0][4], rhs[0][1], 1.0, freq]
    ncol = 64
    dist = width / ncol
    # dt <= h/(vp*2) for any refinement: the save interval uses that bound
    return _deck(width, height, steps * (h / 4000.0) * 1.0000001, save_every * (h / 4000.0), 0.25, nperlen, 2,
                 [ROCK_HALFSPACE], rhs[0][0], pparams, geom="CANYON",
                 gparams=(width / 2, 0.0, radius), receivers=(0.0, width - dist, dist), rhs=rhs,
                 refine=(refine_levels, refine_band * max(scale, 0.25)))


def point_source(scale=1.0, steps=4000, kind="POINTN", geom="NONE", amp=None, sigma=0.01, start=0.4,
                 dist=None, point=None, save_every=4, refine_levels=2):
    """A point source (POINTN force or POINTD displacement) on the y dof of
    every node within `dist` of `point` (setup_point_source,
    model.f90:1051-1078); pparams = (amp, sigma, start, dist, x, y).

    geom "NONE": the homogeneous rectangle's mesh (15.625 m), source at the
    middle of the surface.  geom "CANYON": the canyon with two REFINE levels
    around the rim, source on the surface at the rim, where refined and
    hanging nodes lie within `dist`.  No DRM layer, no free field."""
    if geom == "NONE":
        h = 15.625
        ncol = max(8, int(round(256 * scale)))
        nrow = max(4, int(round(128 * scale)))
        width, height = ncol * h, nrow * h
        hmin, chper, nperlen, extra = h, 0.15625, 10, {}
        point = point or (0.5 * width, 0.0)
        dist = dist or 1.5 * h
    else:
        width, height = 6000.0 * scale, 3000.0 * scale
        radius = 500.0 * scale
        h = 10.0
        hmin, chper, nperlen = h / 2 ** refine_levels, 0.25, 25
        extra = dict(geom="CANYON", gparams=(width / 2, 0.0, radius),
                     refine=(refine_levels, 60.0 * max(scale, 0.25)))
        point = point or (width / 2 + radius + 0.5 * h, 0.0)
        dist = dist or 3.0 * h
    if amp is None:
        amp = 1.0e6 if kind == "POINTN" else 1.0e-3
    dt_bound = hmin / 4000.0   # dt = hmin/(vp*2) with vp 2000
    ncol_r = 64
    rd = width / ncol_r
    return _deck(width, height, steps * dt_bound * 1.0000001, save_every * dt_bound, chper, nperlen, 2,
                 [ROCK_HALFSPACE], kind, [amp, sigma, start, dist, point[0], point[1]],
                 receivers=(0.0, width - rd, rd), **extra)


VALLEY_MATERIALS = ["p 3000 s 1500 2400", "p 700 s 300 1800"]


def valley(scale=1.0, steps=20000, chper=0.056, rhs=None, seed=2024, sigma=0.1, freq=5.0,
           save_every=10, half_width=1500.0, depth=400.0):
    """Semi-elliptical sedimentary valley over bedrock (EVALLY geometry).

    With CONTROL 10 2 the rock length is chper*1500/10 and the infill
    (vs 300 m/s) needs three halvings: four quadtree levels.  The DRM box
    holds the valley with a margin; rhs entries are (kind, angle, amp, freq)
    and get their delay from the box (rest_delay)."""
    width, height = 12000.0 * scale, 4000.0 * scale
    a, b = half_width * scale, depth * scale
    h_rock = chper * 1500.0 / 10.0
    box_w = min(width - 8 * h_rock, 2.0 * a + max(1000.0 * scale, 8 * h_rock))
    box_h = min(height - 8 * h_rock, b + max(400.0 * scale, 8 * h_rock))
    if rhs is None:
        rhs = [("WAVESV", 0.0, 1.0, freq)]
    rhs = [(k, ang, amp, fc, rest_delay(k, ang, fc, box_w, box_h, 0.0, 3000.0, 1500.0)) for k, ang, amp, fc in rhs]
    # upper bound of the stable step (any element: h <= h_rock, vp >= 0.7*700)
    dt_up = h_rock / (0.7 * 700.0 * 2.0)
    pparams = [box_w, box_h, width / 2, 0.0, 1, rhs[0][4], rhs[0][1], 1.0, rhs[0][3]]
    ncol = 64
    dist = width / ncol
    return _deck(width, height, steps * dt_up, save_every * dt_up, chper, 10, 2, VALLEY_MATERIALS,
                 rhs[0][0], pparams, geom="EVALLY", gparams=(width / 2, 0.0, a, b),
                 receivers=(0.0, width - dist, dist), rhs=rhs,
                 heterogeneity=(sigma, seed) if sigma > 0 else None)


def batched_rhs():
    """64 right-hand sides: 16 angles x {P, SV} x fc {2, 5} Hz.  P spans
    0-70 deg; SV spans 0-28 deg (SV at or past asin(vs/vp) = 30 deg is
    post-critical, pwaves.f90:76-89)."""
    out = []
    for freq in (2.0, 5.0):
        for i in range(16):
            out.append(("WAVEP", math.radians(70.0 * i / 15.0), 1.0, freq))
        for i in range(16):
            out.append(("WAVESV", math.radians(28.0 * i / 15.0), 1.0, freq))
    return out


def valley_batched(scale=1.0, steps=20000, **kw):
    return valley(scale=scale, steps=steps, rhs=batched_rhs(), **kw)


def serving_stream(n=512, rate=20.0, seed=7, min_scale=0.1, max_scale=1.0, max_angles=16,
                   step_range=(1000, 20000), canyon_nperlen=10.0, valley_chper=0.25):
    """Seeded request stream: (arrival_time, deck_text, nsteps) tuples.

    Each request is a canyon (radius 200-800 m) or a semi-elliptical valley
    (half-width 500-2500 m, depth 100-600 m) in a half-space, with 1-16
    incidence angles of one wave kind and Poisson arrivals at `rate` per second.
    `scale` (uniform in [min_scale, max_scale]) sets the domain size; the
    feature is clamped to fit its domain.  Mesh size grows with scale**2 and
    with 1/chper**2 (valleys) or nperlen**2 (canyons)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate)
        s = float(rng.uniform(min_scale, max_scale))
        nang = int(rng.integers(1, max_angles + 1))
        steps = int(rng.integers(step_range[0], step_range[1] + 1))
        kind = "WAVESV" if rng.random() < 0.5 else "WAVEP"
        lim = 28.0 if kind == "WAVESV" else 70.0
        angles = sorted(float(a) for a in rng.uniform(0.0, lim, nang))
        if rng.random() < 0.5:
            r = min(float(rng.uniform(200, 800)), 0.3 * 3000.0 * s)
            deck = canyon(scale=s, steps=steps, radius=r / s, waves=[(kind, a) for a in angles],
                          refine_levels=1, nperlen=canyon_nperlen, save_every=4)
        else:
            a = min(float(rng.uniform(500, 2500)), 0.3 * 12000.0 * s)
            d = min(float(rng.uniform(100, 600)), 0.2 * 4000.0 * s)
            rhs = [(kind, math.radians(x), 1.0, 5.0) for x in angles]
            deck = valley(scale=s, steps=steps, chper=valley_chper, rhs=rhs, seed=int(rng.integers(1 << 30)),
                          half_width=a / s, depth=d / s, sigma=0.1, save_every=4)
        out.append((t, deck, steps))
    return out
