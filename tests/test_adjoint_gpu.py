"""Discrete adjoint of the trajectory + image on the GPU against (1) an FP64 reference
gradient from torch.autograd over the same model on the CPU, (2) central finite
differences of the loss in planet mass, a, e, i, and (3) its own checkpoint interval."""
import math

import numpy as np
import pytest
import torch

import oracle.torch_ref as tr
from diskdyn_gb300 import abi, adjoint as adj
from diskdyn_gb300.engine import Engine, make_phys, make_view

pytestmark = pytest.mark.gpu


def setup(n_dust, n_steps, xsize=64, ysize=64):
    s = adj.adjoint_system(n_dust=n_dust, xsize=xsize, ysize=ysize, n_steps=n_steps, seed=77)
    eng = Engine(0)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    return s, eng


def elements(s, device):
    el = adj.planet_elements(s)
    t = {k: torch.tensor(np.asarray(v, dtype=np.float64), device=device) for k, v in el.items()}
    for k in ("m", "a", "e", "i"):
        t[k].requires_grad_(True)
    return t


def massive_from(t):
    return adj.planet_state(t["Mstar"], t["m"], t["a"], t["e"], t["i"], t["w"], t["o"], t["nu"])


def dust_from(s, device):
    ng = s.n_grav
    d = np.stack([s.state[k][ng:] for k in ("x", "y", "z", "vx", "vy", "vz")], axis=1)
    return torch.tensor(d, dtype=torch.float64, device=device)


def gpu_loss(s, eng, t, dust, target, n_steps, ckpt):
    ng = s.n_grav
    N = torch.tensor(s.state["N"][ng:], dtype=torch.float64, device="cuda")
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int32, device="cuda")
    img = adj.trajectory_image(eng, massive_from(t), dust, N, ids, s.dt, n_steps, ckpt,
                               make_phys(**s.phys), make_view(**s.view), s.image_wj)
    return ((img - target) ** 2).sum(), img


def test_adjoint_matches_torch_autograd_reference():
    n_steps = 24
    s, eng = setup(n_dust=192, n_steps=n_steps)
    ng = s.n_grav
    # GPU adjoint
    tg = elements(s, "cuda")
    dg = dust_from(s, "cuda").requires_grad_(True)
    with torch.no_grad():
        _, img0 = gpu_loss(s, eng, tg, dg, 0.0, n_steps, 5)
    target = 0.5 * img0.detach()
    Lg, _ = gpu_loss(s, eng, tg, dg, target, n_steps, 5)
    Lg.backward()
    # torch autograd on the CPU, FP64
    tc = elements(s, "cpu")
    dc = dust_from(s, "cpu").requires_grad_(True)
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int64)
    beta = torch.tensor(s.size_table["beta"].astype(np.float64))[ids]
    betasw = torch.tensor(s.size_table["betasw"].astype(np.float64))[ids]
    final = tr.trajectory(massive_from(tc), dc, beta, betasw, s.dt, n_steps, s.phys["SWQ"], s.phys["vsw_AUyr"])
    N = torch.tensor(s.state["N"][ng:], dtype=torch.float64)
    imgc = tr.splat_image(final[:, :3], N, ids, s.optics, s.optics["size"], s.view, s.image_wj)
    Lc = ((imgc - target.cpu()) ** 2).sum()
    Lc.backward()
    assert abs(Lg.item() - Lc.item()) <= 1e-9 * abs(Lc.item())
    np.testing.assert_allclose(dg.grad.cpu().numpy(), dc.grad.numpy(), rtol=1e-7,
                               atol=1e-9 * np.abs(dc.grad.numpy()).max())
    for k in ("m", "a", "e", "i"):
        np.testing.assert_allclose(tg[k].grad.cpu().numpy(), tc[k].grad.numpy(), rtol=1e-7,
                                   atol=1e-9 * np.abs(tc[k].grad.numpy()).max(), err_msg=k)
    eng.close()


def test_gradient_independent_of_checkpoint_interval():
    n_steps = 30
    s, eng = setup(n_dust=2048, n_steps=n_steps)
    grads = []
    for ckpt in (1, 7, 30):
        t = elements(s, "cuda")
        d = dust_from(s, "cuda").requires_grad_(True)
        L, _ = gpu_loss(s, eng, t, d, 0.0, n_steps, ckpt)
        L.backward()
        grads.append((d.grad.clone(), t["m"].grad.clone(), t["a"].grad.clone()))
    # the recompute reproduces the forward exactly and every reduction has a fixed order;
    # only the forward image's atomic sums vary between runs, at the last ulp
    for g in grads[1:]:
        for a, b in zip(grads[0], g):
            np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-10,
                                       atol=1e-12 * a.abs().max().item())
    eng.close()


def test_adjoint_matches_central_finite_differences():
    n_steps = 120
    s, eng = setup(n_dust=4096, n_steps=n_steps, xsize=128, ysize=128)
    t = elements(s, "cuda")
    d = dust_from(s, "cuda")
    with torch.no_grad():
        t_target = elements(s, "cuda")
        t_target["m"][0] *= 1.2
        t_target["a"][0] += 2.0
        _, target = gpu_loss(s, eng, t_target, d, 0.0, n_steps, 40)
    L, _ = gpu_loss(s, eng, t, d, target, n_steps, 40)
    L.backward()
    for key, idx in (("m", 0), ("a", 0), ("m", 1), ("e", 0), ("i", 1)):
        base = t[key].detach()[idx].item()
        h = 1e-6 * abs(base) if base != 0.0 else 1e-6
        vals = []
        for sgn in (1.0, -1.0):
            tp = {k: v.detach().clone() for k, v in t.items()}
            tp[key][idx] = base + sgn * h
            with torch.no_grad():
                Lp, _ = gpu_loss(s, eng, tp, d, target, n_steps, 40)
            vals.append(Lp.item())
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = t[key].grad[idx].item()
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-12 * abs(L.item()), (key, idx, ad, fd)
    eng.close()


def test_splat_image_carries_the_flux_of_ddx_image():
    s, eng = setup(n_dust=4096, n_steps=1, xsize=256, ysize=256)
    s.view["fov"] = 400.0   # every tracer well inside the frame
    ng = s.n_grav
    t = elements(s, "cuda")
    d = dust_from(s, "cuda")
    with torch.no_grad():
        _, img = gpu_loss(s, eng, t, d, 0.0, 1, 1)
        from diskdyn_gb300.engine import DeviceState
        # the binned image of the same (one-step-evolved) state through ddx_step + ddx_image
        st = DeviceState.from_numpy(s.state)
        st.x[:ng] = massive_from(t)[:, 0]; st.y[:ng] = massive_from(t)[:, 1]; st.z[:ng] = massive_from(t)[:, 2]
        st.vx[:ng] = massive_from(t)[:, 3]; st.vy[:ng] = massive_from(t)[:, 4]; st.vz[:ng] = massive_from(t)[:, 5]
        st.m[:ng] = massive_from(t)[:, 6]
        eng.step(st, ng, s.dt, make_phys(**s.phys), abi.DDX_PREC_FP64)
        binned = eng.image(st, ng, make_view(**s.view), s.image_wj)
    for k in range(len(s.image_wj)):
        assert abs(img[k].sum().item() - binned[k].sum().item()) <= 1e-9 * binned[k].sum().item()
    eng.close()


def test_adjoint_rejects_massive_sets_beyond_its_limit():
    s, eng = setup(n_dust=64, n_steps=2)
    d = dust_from(s, "cuda")
    ng = s.n_grav
    N = torch.ones(64, dtype=torch.float64, device="cuda")
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int32, device="cuda")
    big = torch.zeros((131073, 7), dtype=torch.float64, device="cuda")
    big[:, 6] = 1.0
    big[:, 0] = torch.arange(131073, dtype=torch.float64, device="cuda")
    with pytest.raises(abi.DDXError) as ei:
        adj.trajectory_image(eng, big, d, N, ids, s.dt, 2, 1, make_phys(**s.phys), make_view(**s.view), s.image_wj)
    assert ei.value.status == 5
    eng.close()


def test_adjoint_with_planetesimals_and_lorentz_matches_torch_autograd():
    """A massive set of the star, two planets and 256 gravitating planetesimals (the
    launch-per-pass path), charged grains under the Lorentz force: the gradients of the loss
    in the planets' elements, in every planetesimal's state and mass and in every grain's
    state agree with torch autograd of the same FP64 model on the CPU.  The charges give the
    smallest grains (m ~ 3e-43) a Lorentz acceleration of about a tenth of the star's pull at
    100 AU (cL = q Bstar Rstar^3 / m ~ 0.15)."""
    n_steps, ckpt = 10, 4
    s = adj.adjoint_system(n_dust=128, xsize=64, ysize=64, n_steps=n_steps, seed=77, n_plsml=256)
    s.phys = dict(s.phys, FLQ=1, Bstar=5e-20, Wz=14.6)
    s.size_table = dict(s.size_table, q=np.linspace(1e-18, 2e-18, len(s.size_table["q"])).astype(np.float32))
    eng = Engine(0)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    ng = s.n_grav
    pl = np.stack([s.state[k][3:ng] for k in ("x", "y", "z", "vx", "vy", "vz", "m")], axis=1)

    def massive(t, plt):
        return torch.cat([massive_from(t), plt], dim=0)

    tg = elements(s, "cuda")
    pg = torch.tensor(pl, dtype=torch.float64, device="cuda").requires_grad_(True)
    dg = dust_from(s, "cuda").requires_grad_(True)
    N = torch.tensor(s.state["N"][ng:], dtype=torch.float64, device="cuda")
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int32, device="cuda")
    mass = torch.tensor(s.state["m"][ng:], dtype=torch.float64, device="cuda")

    def gpu_image(t, plt, d):
        return adj.trajectory_image(eng, massive(t, plt), d, N, ids, s.dt, n_steps, ckpt, make_phys(**s.phys),
                                    make_view(**s.view), s.image_wj, mass=mass)

    with torch.no_grad():
        target = 0.5 * gpu_image(tg, pg, dg).detach()
    Lg = ((gpu_image(tg, pg, dg) - target) ** 2).sum()
    Lg.backward()
    tc = elements(s, "cpu")
    pc = torch.tensor(pl, dtype=torch.float64).requires_grad_(True)
    dc = dust_from(s, "cpu").requires_grad_(True)
    idc = torch.tensor(s.state["id"][ng:], dtype=torch.int64)
    beta = torch.tensor(s.size_table["beta"].astype(np.float64))[idc]
    betasw = torch.tensor(s.size_table["betasw"].astype(np.float64))[idc]
    q = torch.tensor(s.size_table["q"].astype(np.float64))[idc]
    cL = q * s.phys["Bstar"] * s.phys["Rstar"] ** 3 / torch.tensor(s.state["m"][ng:])
    final = tr.trajectory(massive(tc, pc), dc, beta, betasw, s.dt, n_steps, s.phys["SWQ"], s.phys["vsw_AUyr"],
                          lorentz=(cL, s.phys["Wz"]))
    imgc = tr.splat_image(final[:, :3], N.cpu(), idc, s.optics, s.optics["size"], s.view, s.image_wj)
    Lc = ((imgc - target.cpu()) ** 2).sum()
    Lc.backward()
    assert abs(Lg.item() - Lc.item()) <= 1e-9 * abs(Lc.item())
    np.testing.assert_allclose(dg.grad.cpu().numpy(), dc.grad.numpy(), rtol=1e-7,
                               atol=1e-9 * np.abs(dc.grad.numpy()).max())
    np.testing.assert_allclose(pg.grad.cpu().numpy(), pc.grad.numpy(), rtol=1e-7,
                               atol=1e-9 * np.abs(pc.grad.numpy()).max())
    for k in ("m", "a", "e", "i"):
        np.testing.assert_allclose(tg[k].grad.cpu().numpy(), tc[k].grad.numpy(), rtol=1e-7,
                                   atol=1e-9 * np.abs(tc[k].grad.numpy()).max(), err_msg=k)
    eng.close()


def test_tracers_far_off_the_frame_add_nothing_and_carry_no_gradient():
    """Grains thrown far out (1e7 to 1e22 AU, beyond int pixel range) and a NaN grain: the
    differentiable image equals the image without them, their gradient is zero, and the
    binned ddx_image ignores them too."""
    n_steps = 2
    s, eng = setup(n_dust=256, n_steps=n_steps)
    ng = s.n_grav
    far = [1e7, -3e9, 2e12, -5e15, 7e18, -1e22]
    for k, r in enumerate(far):
        s.state["x"][ng + k] = r
        s.state["y"][ng + k] = -0.7 * r
    s.state["z"][ng + len(far)] = np.nan
    n_bad = len(far) + 1
    t = elements(s, "cuda")
    d = dust_from(s, "cuda").requires_grad_(True)
    L, img = gpu_loss(s, eng, t, d, 0.0, n_steps, 1)
    L.backward()
    assert torch.isfinite(img).all()
    assert (d.grad[:n_bad] == 0).all() and torch.isfinite(d.grad).all()
    # the same image with those grains removed (N = 0)
    N_off = torch.tensor(s.state["N"][ng:], dtype=torch.float64, device="cuda")
    N_off[:n_bad] = 0.0
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int32, device="cuda")
    with torch.no_grad():
        img_off = adj.trajectory_image(eng, massive_from(t), d.detach(), N_off, ids, s.dt, n_steps, 1,
                                       make_phys(**s.phys), make_view(**s.view), s.image_wj)
    np.testing.assert_allclose(img.detach().cpu().numpy(), img_off.cpu().numpy(), rtol=1e-12,
                               atol=1e-14 * img_off.abs().max().item())
    # the binned image of the initial state skips them as well
    from diskdyn_gb300.engine import DeviceState
    Ns = dict(s.state)
    Ns["N"] = s.state["N"].copy()
    Ns["N"][ng:ng + n_bad] = 0.0
    for prec, rtol in ((abi.DDX_PREC_FP64, 1e-12), (abi.DDX_PREC_MIXED, 1e-6)):
        binned = eng.image(DeviceState.from_numpy(s.state), ng, make_view(**s.view), s.image_wj, precision=prec)
        binned_off = eng.image(DeviceState.from_numpy(Ns), ng, make_view(**s.view), s.image_wj, precision=prec)
        np.testing.assert_allclose(binned.cpu().numpy(), binned_off.cpu().numpy(), rtol=rtol,
                                   atol=rtol * binned_off.abs().max().item())
    eng.close()
