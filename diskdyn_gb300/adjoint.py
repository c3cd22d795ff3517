"""Gradients of an image loss through the RK4 trajectory: a torch.autograd.Function over
the discrete-adjoint kernels of libddx.so (ddx_adjoint_forward / ddx_adjoint_backward).

    img = trajectory_image(engine, massive, dust, N, ids, dt, n_steps, ckpt, phys, view, wj)
    loss = ((img - target) ** 2).sum(); loss.backward()

`massive` is (n_grav, 7) = x, y, z, vx, vy, vz, m*4pi^2 (star first) and `dust` is
(n_dust, 6); both FP64 CUDA tensors, so gradients reach anything they were built from --
for instance planet orbital elements through `planet_state` (the reference's `coe2rv`,
src/functions.cu:6-46, and `recalc_COM`, src/read_in.cu:344-375, written in torch).
The image is the flux of ddx_image deposited with bilinear weights (continuous in the
positions); the backward is checkpoint-and-recompute every `ckpt` steps.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import abi, synth
from .engine import DeviceState, _stream_handle, make_phys, make_view


class _TrajectoryImage(torch.autograd.Function):
    @staticmethod
    def forward(ctx, massive, dust, eng, N, ids, dt, n_steps, ckpt, phys, view, wj, mass):
        ng, nd = massive.shape[0], dust.shape[0]
        dev = massive.device
        zeros = torch.zeros(nd, dtype=torch.float64, device=dev) if mass is None else mass.to(torch.float64)
        st = DeviceState(
            x=torch.cat([massive[:, 0], dust[:, 0]]).contiguous(),
            y=torch.cat([massive[:, 1], dust[:, 1]]).contiguous(),
            z=torch.cat([massive[:, 2], dust[:, 2]]).contiguous(),
            vx=torch.cat([massive[:, 3], dust[:, 3]]).contiguous(),
            vy=torch.cat([massive[:, 4], dust[:, 4]]).contiguous(),
            vz=torch.cat([massive[:, 5], dust[:, 5]]).contiguous(),
            m=torch.cat([massive[:, 6], zeros]).contiguous(),
            N=torch.cat([torch.ones(ng, dtype=torch.float64, device=dev), N]).contiguous(),
            id=torch.cat([torch.full((ng,), -1, dtype=torch.int32, device=dev), ids]).contiguous())
        wj_a = np.ascontiguousarray(wj, np.int32)
        img = torch.empty((len(wj_a), view.xsize, view.ysize), dtype=torch.float64, device=dev)
        abi.check(eng.lib.ddx_adjoint_forward(eng.ctx, C.byref(st._abi), ng, nd, float(dt), int(n_steps),
                                              int(ckpt), C.byref(phys), C.byref(view),
                                              wj_a.ctypes.data_as(C.c_void_p), len(wj_a),
                                              C.c_void_p(img.data_ptr()), C.c_void_p(_stream_handle(None))),
                  "ddx_adjoint_forward")
        ctx.eng, ctx.ng, ctx.nd = eng, ng, nd
        ctx.keep = st          # the state buffers must outlive the asynchronous forward
        return img

    @staticmethod
    def backward(ctx, gimg):
        eng, ng, nd = ctx.eng, ctx.ng, ctx.nd
        g = gimg.contiguous()
        gs = torch.empty((6, ng + nd), dtype=torch.float64, device=g.device)
        gm = torch.empty(ng, dtype=torch.float64, device=g.device)
        abi.check(eng.lib.ddx_adjoint_backward(eng.ctx, C.c_void_p(g.data_ptr()), C.c_void_p(gs.data_ptr()),
                                               C.c_void_p(gm.data_ptr()), C.c_void_p(_stream_handle(None))),
                  "ddx_adjoint_backward")
        g_massive = torch.cat([gs[:, :ng].T, gm[:, None]], dim=1)
        g_dust = gs[:, ng:].T
        return g_massive, g_dust, None, None, None, None, None, None, None, None, None, None


def trajectory_image(eng, massive, dust, N, ids, dt, n_steps, ckpt, phys, view, wj, mass=None):
    """Differentiable image of the state after n_steps (see module docstring).  mass: the
    grains' masses (n_dust,), which the Lorentz force divides by (phys.FLQ = 1); without them
    the grains count as massless and feel no Lorentz force."""
    return _TrajectoryImage.apply(massive, dust, eng, N, ids, dt, n_steps, ckpt, phys, view, wj, mass)


def coe2rv_t(M, m, a, e, i, w, o, nu, beta=0.0):
    """src/functions.cu:6-46 in torch (differentiable in every argument)."""
    p = a * (1.0 - e * e)
    mu = (M + m) * (1.0 - beta)
    cn, sn = torch.cos(nu), torch.sin(nu)
    xe = p * cn / (1.0 + e * cn)
    ye = p * sn / (1.0 + e * cn)
    vxe = -torch.sqrt(mu / p) * sn
    vye = torch.sqrt(mu / p) * (e + cn)
    co, so, cw, sw, ci, si = torch.cos(o), torch.sin(o), torch.cos(w), torch.sin(w), torch.cos(i), torch.sin(i)
    r11, r12 = co * cw - so * sw * ci, -co * sw - so * cw * ci
    r21, r22 = so * cw + co * sw * ci, -so * sw + co * cw * ci
    r31, r32 = sw * si, cw * si
    return (xe * r11 + ye * r12, xe * r21 + ye * r22, xe * r31 + ye * r32,
            vxe * r11 + vye * r12, vxe * r21 + vye * r22, vxe * r31 + vye * r32)


def planet_state(Mstar, pm, pa, pe, pi, pw, po, pnu):
    """(n_planets + 1, 7) massive state of a star and planets given in orbital elements
    (masses already x 4pi^2), moved to the centre-of-mass frame like recalc_COM
    (src/read_in.cu:344-375).  Differentiable in every element."""
    x, y, z, vx, vy, vz = coe2rv_t(Mstar, pm, pa, pe, pi, pw, po, pnu)
    zero = torch.zeros(1, dtype=pm.dtype, device=pm.device)
    m = torch.cat([Mstar.reshape(1), pm])
    X = torch.cat([zero, x]); Y = torch.cat([zero, y]); Z = torch.cat([zero, z])
    Mt = m.sum()
    X = X - (m * X).sum() / Mt
    Y = Y - (m * Y).sum() / Mt
    Z = Z - (m * Z).sum() / Mt
    VX = torch.cat([-(pm * vx).sum().reshape(1) / m[0], vx])
    VY = torch.cat([-(pm * vy).sum().reshape(1) / m[0], vy])
    VZ = torch.cat([-(pm * vz).sum().reshape(1) / m[0], vz])
    return torch.stack([X, Y, Z, VX, VY, VZ, m], dim=1)


def adjoint_system(n_dust=262144, xsize=512, ysize=512, n_steps=2000, seed=synth.SEED, n_plsml=0):
    """The image-loss workload: the dusty-ring star (1.5 Msun, L = 8.7 Lsun) with its two
    planets (1e-3 Msun at 20 AU, 3e-4 Msun at 60 AU), n_plsml gravitating planetesimals of
    the ring and n_dust grains of the ring with radiation pressure, PR and stellar-wind
    drag.  Optics:
    HG tables on the grains' size bins, grey grains at T = 278.3 L^(1/4) (r/AU)^(-1/2) K;
    a 512 x 512 image, 300 AU across, at 30 deg inclination, at 1.25 um (scattered light)
    and 100 um (thermal)."""
    s = synth.dusty_ring(n_dust=n_dust, n_plsml=n_plsml, seed=seed, n_steps=n_steps)
    synth.ring_imaging(s, xsize, ysize)
    s.name = "adjoint_ring"
    return s


def planet_elements(sysm):
    """Orbital elements of the planets of `dusty_ring` (index 1, 2 of the massive set),
    as synth.dusty_ring drew them: circular, coplanar, true anomalies from its stream."""
    g = synth.rng(sysm.meta["seed"], 11)
    nu = g.uniform(0.0, 2 * math.pi, 2)
    return {"m": np.array([1e-3, 3e-4]) * synth.GRAV, "a": np.array([20.0, 60.0]), "e": np.zeros(2),
            "i": np.zeros(2), "w": np.zeros(2), "o": np.zeros(2), "nu": nu,
            "Mstar": sysm.meta["Mstar"] * synth.GRAV}
