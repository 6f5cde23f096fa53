"""numpy emulation of the FP64 step kernels over the library's own plan.

Used by the CPU suite to check the plan (numbering, gather lists, hanging
weights, DRM slots, receiver weights) and the device arithmetic (compiled for
the host by tests/native/probe.cu) against the oracle without a GPU.
"""
from __future__ import annotations

import numpy as np

import native_probe as npb


def q4_ku(k, ux, uy):
    """Vectorised twin of q4_ku (exfem_device.cuh) for checks."""
    A, B, Cc, D = k[:, 0], k[:, 1], k[:, 2], k[:, 3]
    px, qx = ux[:, 2] - ux[:, 0], ux[:, 1] - ux[:, 3]
    c1x, c2x, c3x = px + qx, px - qx, (ux[:, 0] + ux[:, 2]) - (ux[:, 1] + ux[:, 3])
    py, qy = uy[:, 2] - uy[:, 0], uy[:, 1] - uy[:, 3]
    c1y, c2y, c3y = py + qy, py - qy, (uy[:, 0] + uy[:, 2]) - (uy[:, 1] + uy[:, 3])
    F1 = A * c1x + B * c2y
    F2 = A * c2y + B * c1x
    S = Cc * (c2x + c1y)
    Gx, Gy = D * c3x, D * c3y
    ax, bx = F1 + S, F1 - S
    ay, by = S + F2, S - F2
    fx = np.stack([Gx - ax, bx - Gx, ax + Gx, -(bx + Gx)], axis=1)
    fy = np.stack([Gy - ay, by - Gy, ay + Gy, -(by + Gy)], axis=1)
    return fx, fy


def emulate_fp64(model, nsteps, rhs=0, reorder=True):
    P = npb.PlanView(model, reorder=reorder)
    sc = P.scalars
    na, nh = int(sc[0]), int(sc[1])
    a1, a2, a3, dt = sc[2], sc[3], sc[4], sc[5]
    io = int(sc[7])
    nn = model.nnodes
    econn = P.econn.reshape(-1, 4)
    ne = econn.shape[0]
    ecoef = P.ecoef.reshape(-1, 4)
    emass = P.emass
    edamp = P.edamp
    edampv = P.edampv.reshape(-1, 8)
    damped = np.nonzero(edamp >= 0)[0]
    nodes = model.nodes()[P.ref_of_node]
    worigin = np.array(model.problem.worigin[:])
    s_elem, s_kind = P.s_elem, P.s_kind
    ns = s_elem.size
    tptr, tlist = P.tptr, P.tlist
    dptr, dlist = P.dptr, P.dlist
    t_node = np.repeat(np.arange(na), np.diff(tptr))
    t_w = np.where(tlist & 1, 0.5, 1.0)
    t_e = (tlist >> 1) >> 2
    t_c = (tlist >> 1) & 3
    d_node = np.repeat(np.arange(na), np.diff(dptr))
    d_w = np.where(dlist & 1, 0.5, 1.0)
    d_s = (dlist >> 1) >> 2
    d_c = (dlist >> 1) & 3
    inv_m = P.inv_mfull.reshape(-1, 2)
    hang = P.hang.reshape(-1, 3)
    rnode = P.rnode.reshape(-1, 4)
    rw = P.rw.reshape(-1, 4)
    rsoil, rxy = P.rsoil, P.rxy.reshape(-1, 2)
    nrecv = rsoil.size
    nsave = nsteps // io + 1
    seis = np.zeros((nsave, nrecv, 2))
    L = npb.lib()

    def sample(slot, u):
        time = dt * slot * io
        f = np.einsum("rk,rkc->rc", rw, u[rnode])   # hanging corners hold their averages
        for i in np.nonzero(rsoil)[0]:
            w = P.wave(rhs, time, rxy[i, 0] - worigin[0], rxy[i, 1] - worigin[1])
            f[i] += w[0:2]
        seis[slot] = f

    u = np.zeros((nn, 2))
    um = np.zeros((nn, 2))
    sample(0, u)
    for step in range(1, nsteps + 1):
        t = step * dt
        fdrm = np.zeros((max(ns, 1), 8))
        for s in range(ns):
            ie = s_elem[s]
            u0 = np.zeros(8)
            a0 = np.zeros(8)
            for k in range(4):
                x = econn[ie, k]
                w = P.wave(rhs, t, nodes[x, 0] - worigin[0], nodes[x, 1] - worigin[1])
                u0[2 * k:2 * k + 2] = w[0:2]
                a0[2 * k:2 * k + 2] = w[4:6]
            p = np.zeros(8)
            kc = np.ascontiguousarray(ecoef[ie])
            L.probe_drm_forces(npb.dp(kc), float(emass[ie]), int(s_kind[s]), npb.dp(u0), npb.dp(a0), npb.dp(p))
            fdrm[s] = p
        ux, uy = u[econn, 0], u[econn, 1]
        vx, vy = um[econn, 0], um[econn, 1]
        fx, fy = q4_ku(ecoef, ux, uy)
        lr = np.zeros((ne, 8))
        lr[:, 0::2] = (a3 * ux - a1 * vx) * emass[:, None]
        lr[:, 1::2] = (a3 * uy - a1 * vy) * emass[:, None]
        dv = edampv[edamp[damped]]
        lr[damped, 0::2] += a2 * dv[:, 0::2] * vx[damped]
        lr[damped, 1::2] += a2 * dv[:, 1::2] * vy[damped]
        lr[:, 0::2] -= fx
        lr[:, 1::2] -= fy
        r = np.zeros((na, 2))
        if dlist.size:
            np.add.at(r, d_node, d_w[:, None] * np.stack([fdrm[d_s, 2 * d_c], fdrm[d_s, 2 * d_c + 1]], axis=1))
        np.add.at(r, t_node, t_w[:, None] * np.stack([lr[t_e, 2 * t_c], lr[t_e, 2 * t_c + 1]], axis=1))
        unew = np.zeros((nn, 2))
        unew[:na] = r * inv_m
        if nh:
            unew[hang[:, 0]] = (unew[hang[:, 1]] + unew[hang[:, 2]]) / 2.0
        um, u = u, unew
        if step % io == 0:
            sample(step // io, u)
    u_ref = np.zeros((nn, 2))
    u_ref[P.ref_of_node] = u
    return {"seis": seis, "u": u_ref.ravel(), "mfull": P.mfull_ref}


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((b + np.uint32(0x7FFF) + ((b >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)).astype(np.uint32)
    return r.view(np.float32)


def emulate_fp32(model, nsteps, rhs=0, comp="bf16"):
    """float32 twin of k_drm32/k_step32/k_hang32: delta = (f - K u - 2 a2 C D
    + anchor terms) / m_full, D+ = D + delta and u+ = u + D+, both Kahan
    compensated, the compensations stored as `comp` ("bf16" or "f32")."""
    P = npb.PlanView(model)
    sc = P.scalars
    na, nh = int(sc[0]), int(sc[1])
    a1, a2, dt = sc[2], sc[3], sc[5]
    io = int(sc[7])
    nn = model.nnodes
    f32 = np.float32
    rnd = bf16 if comp == "bf16" else (lambda v: np.asarray(v, f32))
    econn = P.econn.reshape(-1, 4)
    ecoef = P.ecoef.reshape(-1, 4)
    k32 = np.asarray(P.ecoef32).reshape(-1, 4)   # the kernels' FP32 coefficients
    emass = P.emass
    nodes = model.nodes()[P.ref_of_node]
    worigin = np.array(model.problem.worigin[:])
    s_elem, s_kind = P.s_elem, P.s_kind
    ns = s_elem.size
    tptr, tlist, dptr, dlist = P.tptr, P.tlist, P.dptr, P.dlist
    t_node = np.repeat(np.arange(na), np.diff(tptr))
    t_w = np.where(tlist & 1, 0.5, 1.0).astype(f32)
    t_e, t_c = (tlist >> 1) >> 2, (tlist >> 1) & 3
    d_node = np.repeat(np.arange(na), np.diff(dptr))
    d_w = np.where(dlist & 1, 0.5, 1.0).astype(f32)
    d_s, d_c = (dlist >> 1) >> 2, (dlist >> 1) & 3
    inv_m = P.inv_mfull.reshape(-1, 2).astype(f32)
    nmass, ndamp = P.nmass, P.ndamp.reshape(-1, 2)
    E = (-2.0 * a2 * ndamp).astype(f32)
    D = (a1 * nmass[:, None] + a2 * ndamp).astype(f32)
    hang = P.hang.reshape(-1, 3)
    lptr, llist = P.lptr, P.llist.reshape(-1, 2)
    l_node = np.repeat(np.arange(na), np.diff(lptr))
    rnode, rw = P.rnode.reshape(-1, 4), P.rw.reshape(-1, 4)
    rsoil, rxy = P.rsoil, P.rxy.reshape(-1, 2)
    seis = np.zeros((nsteps // io + 1, rsoil.size, 2))
    L = npb.lib()
    uh, uc, dh, dc = (np.zeros((nn, 2), f32) for _ in range(4))

    def sample(slot):
        time = dt * slot * io
        u = uh.astype(np.float64) - uc.astype(np.float64)
        if nh:
            u[hang[:, 0]] = (u[hang[:, 1]] + u[hang[:, 2]]) / 2
        f = np.einsum("rk,rkc->rc", rw, u[rnode])
        for i in np.nonzero(rsoil)[0]:
            f[i] += P.wave(rhs, time, rxy[i, 0] - worigin[0], rxy[i, 1] - worigin[1])[0:2]
        seis[slot] = f

    sample(0)
    for step in range(1, nsteps + 1):
        t = step * dt
        fdrm = np.zeros((max(ns, 1), 8), f32)
        for s in range(ns):
            ie = s_elem[s]
            u0, a0 = np.zeros(8), np.zeros(8)
            for k in range(4):
                x = econn[ie, k]
                w = P.wave(rhs, t, nodes[x, 0] - worigin[0], nodes[x, 1] - worigin[1])
                u0[2 * k:2 * k + 2] = w[0:2]
                a0[2 * k:2 * k + 2] = w[4:6]
            p = np.zeros(8)
            kc = np.ascontiguousarray(ecoef[ie])
            L.probe_drm_forces(npb.dp(kc), float(emass[ie]), int(s_kind[s]), npb.dp(u0), npb.dp(a0), npb.dp(p))
            fdrm[s] = p.astype(f32)
        fx, fy = q4_ku(k32, uh[econn, 0], uh[econn, 1])
        acc = np.zeros((na, 2), f32)
        if dlist.size:
            np.add.at(acc, d_node, d_w[:, None] * np.stack([fdrm[d_s, 2 * d_c], fdrm[d_s, 2 * d_c + 1]], axis=1))
        np.add.at(acc, t_node, -t_w[:, None] * np.stack([fx[t_e, t_c], fy[t_e, t_c]], axis=1))
        acc += E[:na] * dh[:na]
        if llist.size:
            h = llist[:, 0]
            term = f32(0.5) * (E[h] * dh[h] + D[h] * ((uh[h] - uh[l_node]) + (dh[h] - dh[l_node])))
            np.add.at(acc, l_node, term.astype(f32))
        delta = (acc * inv_m).astype(f32)
        # D+ = D + delta (Kahan, compensation rounded to `comp`)
        y = (delta - dc[:na]).astype(f32)
        tt = (dh[:na] + y).astype(f32)
        dc[:na] = rnd(((tt - dh[:na]).astype(f32) - y).astype(f32))
        dh[:na] = tt
        # u+ = u + D+ (Kahan)
        y = (tt - uc[:na]).astype(f32)
        tu = (uh[:na] + y).astype(f32)
        uc[:na] = rnd(((tu - uh[:na]).astype(f32) - y).astype(f32))
        uh[:na] = tu
        if nh:
            a_, b_ = hang[:, 1], hang[:, 2]
            for arr in (uh, uc, dh, dc):
                arr[hang[:, 0]] = f32(0.5) * (arr[a_] + arr[b_])
            uc[hang[:, 0]] = rnd(uc[hang[:, 0]])
            dc[hang[:, 0]] = rnd(dc[hang[:, 0]])
        if step % io == 0:
            sample(step // io)
    return {"seis": seis}
