"""ORACLE -- test infrastructure, not product code.

FP64 reference for the discrete adjoint: the RK4 trajectory (massive all-pairs gravity,
tracers under the star term with radiation pressure, PR and stellar-wind drag, the
optional Lorentz force and the bodies' gravity -- src/gpu_functions.cu:71-943) and the
bilinear-splat image of the flux (src/gpu_functions.cu:1049-1078), written with torch
float64 operations on the CPU.  torch.autograd differentiates it, which gives an
independent reference gradient for the hand-written adjoint kernels.  Small systems only.
"""
from __future__ import annotations

import math

import torch

LIGHT_AU = 63239.6717367
AU = 1.49598e11
CSPEED = 299792458.0
KBOLTZ = 1.3806503e-23
HPLANK = 6.626068e-34
PI = 3.14159265358979323846
NR = 100


def star_term(d, r, m0, bet, betsw, SWQ, vsw, lorentz=None):
    """lorentz: None, or (cL, Wz) with cL = q Bstar Rstar^3 / m per tracer (nd, 1): the force
    cL (ry - Wz dx, -(rx + Wz dy), 0) / R^3 of src/gpu_functions.cu:706-713."""
    RR = (d * d).sum(-1, keepdim=True)
    R3 = RR * torch.sqrt(RR)
    Fg = (1.0 - bet - betsw) * m0 / R3
    if SWQ == 1:
        Fb1 = m0 / RR * (bet / LIGHT_AU + betsw / vsw)
    else:
        Fb1 = bet * m0 / LIGHT_AU / RR
    Fb2 = (d * r).sum(-1, keepdim=True) / RR
    a = -Fg * d - Fb1 * (Fb2 * d + r)
    if lorentz is not None:
        cL, Wz = lorentz
        flx = cL / R3 * (r[:, 1:2] - Wz * d[:, 0:1])
        fly = -cL / R3 * (r[:, 0:1] + Wz * d[:, 1:2])
        a = a + torch.cat([flx, fly, torch.zeros_like(flx)], dim=1)
    return a


def massive_acc(P, m):
    d = P[None, :, :] - P[:, None, :]                      # d[j, k] = P_k - P_j
    RR = (d * d).sum(-1)
    eye = torch.eye(len(m), dtype=torch.bool)
    RR = torch.where(eye, torch.ones_like(RR), RR)
    f = torch.where(eye, torch.zeros_like(RR), m[None, :] / (RR * torch.sqrt(RR)))
    return (f[:, :, None] * d).sum(1)


def dust_acc(x, r, P, m, bet, betsw, SWQ, vsw, lorentz=None):
    a = star_term(x - P[0], r, m[0], bet, betsw, SWQ, vsw, lorentz)
    for j in range(1, len(m)):
        d = P[j] - x
        RR = (d * d).sum(-1, keepdim=True)
        a = a + m[j] / (RR * torch.sqrt(RR)) * d
    return a


def trajectory(massive, dust, bet, betsw, dt, n_steps, SWQ, vsw, lorentz=None):
    """massive (ng, 7), dust (nd, 6) -> dust state after n_steps (nd, 6).  lorentz: see
    star_term (cL per tracer, shape (nd,))."""
    if lorentz is not None:
        lorentz = (lorentz[0][:, None], lorentz[1])
    xm, vm, m = massive[:, 0:3], massive[:, 3:6], massive[:, 6]
    xd, vd = dust[:, 0:3], dust[:, 3:6]
    bet = bet[:, None]
    betsw = betsw[:, None]
    h2, d6 = dt * 0.5, dt / 6.0
    for _ in range(n_steps):
        P1 = xm
        A1 = massive_acc(P1, m)
        R2 = vm + A1 * h2
        P2 = xm + vm * h2
        A2 = massive_acc(P2, m)
        R3 = vm + A2 * h2
        P3 = xm + R2 * h2
        A3 = massive_acc(P3, m)
        R4 = vm + A3 * dt
        P4 = xm + R3 * dt
        A4 = massive_acc(P4, m)
        a1 = dust_acc(xd, vd, P1, m, bet, betsw, SWQ, vsw, lorentz)
        r2 = vd + a1 * h2
        a2 = dust_acc(xd + vd * h2, r2, P2, m, bet, betsw, SWQ, vsw, lorentz)
        r3 = vd + a2 * h2
        a3 = dust_acc(xd + r2 * h2, r3, P3, m, bet, betsw, SWQ, vsw, lorentz)
        r4 = vd + a3 * dt
        a4 = dust_acc(xd + r3 * dt, r4, P4, m, bet, betsw, SWQ, vsw, lorentz)
        xd = xd + d6 * (vd + 2.0 * (r2 + r3) + r4)
        vd = vd + d6 * (a1 + 2.0 * (a2 + a3) + a4)
        xm = xm + d6 * (vm + 2.0 * R2 + 2.0 * R3 + R4)
        vm = vm + d6 * (A1 + 2.0 * A2 + 2.0 * A3 + A4)
    return torch.cat([xd, vd], dim=1)


def splat_image(pos, N, ids, optics, size, view, wj):
    """Bilinear-splat image (n_img, xsize, ysize) of the flux of every tracer."""
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    rot, inc, PA, dist = view["longitude"], view["inc"], view["PA"], view["dist"]
    xs, ys = view["xsize"], view["ysize"]
    psca = view["fov"] / max(xs, ys)
    cr, sr, ci, si, cp, sp = math.cos(rot), math.sin(rot), math.cos(inc), math.sin(inc), math.cos(PA), math.sin(PA)
    R = torch.sqrt(x * x + y * y + z * z)
    x1, y1 = x * cr - y * sr, x * sr + y * cr
    ly0, lz0 = -dist * math.sin(inc), dist * math.cos(inc)
    L = torch.sqrt(x1 * x1 + (ly0 - y1) ** 2 + (lz0 - z) ** 2)
    c = (x1 * x1 + y1 * y1 + z * z - y1 * ly0 - z * lz0) / (R * L)
    nth = optics["Qpfunc"].shape[1]
    c = torch.clamp(c, min=-1.0, max=1.0 - 2.0 / nth)
    y2 = y1 * ci + z * si
    X, Y = x1 * cp - y2 * sp, x1 * sp + y2 * cp
    u = X / psca + 0.5 * xs - 0.5
    w = Y / psca + 0.5 * ys - 0.5
    i0, j0 = torch.floor(u).detach(), torch.floor(w).detach()
    fu, fw = u - i0, w - j0
    Rmin, Rmax = optics["Rmin"], optics["Rmax"]
    Td = torch.as_tensor(optics["Td"], dtype=torch.float64)
    lT = torch.log(Td)
    fR = math.log(Rmax / Rmin) / (NR - 1.0)
    lr = torch.log(R / Rmin)
    k = torch.clamp((lr / fR).detach().floor().long() + 1, 1, NR - 1)
    # (integer tensor) * (python float) would promote to float32: convert first
    frac = (lr - (k - 1).double() * fR) / fR
    idl = ids.long()
    T = torch.exp(lT[idl, k - 1] + (lT[idl, k] - lT[idl, k - 1]) * frac)
    T = torch.where(R <= Rmin, Td[idl, 0], torch.where(R >= Rmax, Td[idl, NR - 1], T))
    lQ = torch.log(torch.as_tensor(optics["Qpfunc"], dtype=torch.float64))
    cm = torch.floor(0.5 * (c.detach() + 1.0) * (nth - 1)).long()
    cosm = cm.double() * 2.0 / (nth - 1) - 1.0
    cosp = (cm + 1).double() * 2.0 / (nth - 1) - 1.0
    wt = (c - cosm) / (cosp - cosm)
    s = torch.as_tensor(size, dtype=torch.float64)[idl]
    Qabs = torch.as_tensor(optics["Qabs"], dtype=torch.float64)
    Qsca = torch.as_tensor(optics["Qsca"], dtype=torch.float64)
    wv = torch.as_tensor(optics["w"], dtype=torch.float64)
    influx = torch.as_tensor(optics["in"], dtype=torch.float64)
    lit = (R > Rmin) & (ids >= 0) & (N != 0)
    img = torch.zeros((len(wj), xs, ys), dtype=torch.float64)
    for kk, j in enumerate(wj):
        wvl = wv[j]
        xq = HPLANK * CSPEED / (wvl * KBOLTZ * T)
        I = torch.where(xq < 700.0, (2 * HPLANK * CSPEED * CSPEED) / (wvl ** 5 * (torch.exp(torch.clamp(xq, max=700.0)) - 1.0)) * PI,
                        torch.zeros_like(xq))
        P = torch.exp(lQ[idl, cm, j] + (lQ[idl, cm + 1, j] - lQ[idl, cm, j]) * wt)
        Fscat = influx[j] * PI * s * s * Qsca[idl, j] * P / R / R / AU / AU
        Fther = I * s * s * Qabs[idl, j] / dist / dist
        F = N * (Fther + Fscat) * 1e26 * wvl * wvl / CSPEED
        F = torch.where(lit, F, torch.zeros_like(F))
        flat = img[kk].reshape(-1)
        for a in (0, 1):
            for b in (0, 1):
                px, py = (i0 + a).long(), (j0 + b).long()
                inside = (px >= 0) & (px < xs) & (py >= 0) & (py < ys)
                wgt = (fu if a else 1.0 - fu) * (fw if b else 1.0 - fw)
                idx = torch.where(inside, px * ys + py, torch.zeros_like(px))
                flat = flat.index_add(0, idx, torch.where(inside, F * wgt, torch.zeros_like(F)))
        img = torch.cat([img[:kk], flat.reshape(1, xs, ys), img[kk + 1:]], dim=0)
    return img
