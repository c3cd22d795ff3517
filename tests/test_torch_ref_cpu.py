"""The torch FP64 reference of the adjoint tests (oracle/torch_ref.py) against the C
oracle, which the GPU tests pin to the reference's own kernels: same trajectory, same
total flux.  This ties the autograd reference gradient to the reference's physics."""
import numpy as np
import torch

import oracle.cpu as oc
import oracle.torch_ref as tr
from diskdyn_gb300 import adjoint as adj


def small():
    return adj.adjoint_system(n_dust=96, xsize=64, ysize=64, n_steps=8, seed=31)


def test_torch_trajectory_matches_c_oracle():
    s = small()
    ng = s.n_grav
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int64)
    beta = torch.tensor(s.size_table["beta"].astype(np.float64))[ids]
    betasw = torch.tensor(s.size_table["betasw"].astype(np.float64))[ids]
    massive = torch.tensor(np.stack([s.state[k][:ng] for k in ("x", "y", "z", "vx", "vy", "vz", "m")], 1))
    dust = torch.tensor(np.stack([s.state[k][ng:] for k in ("x", "y", "z", "vx", "vy", "vz")], 1))
    with torch.no_grad():
        out = tr.trajectory(massive, dust, beta, betasw, s.dt, 8, s.phys["SWQ"], s.phys["vsw_AUyr"]).numpy()
    ref = oc.step(s.state, ng, s.dt, s.size_table, s.phys, 8)
    for c, k in enumerate(("x", "y", "z", "vx", "vy", "vz")):
        np.testing.assert_allclose(out[:, c], ref[k][ng:], rtol=1e-12, atol=1e-12)


def test_torch_splat_flux_matches_c_oracle_image_flux():
    s = small()
    s.view["fov"] = 400.0                      # every tracer inside the frame
    ng = s.n_grav
    pos = torch.tensor(np.stack([s.state[k][ng:] for k in ("x", "y", "z")], 1))
    N = torch.tensor(s.state["N"][ng:])
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int64)
    img = tr.splat_image(pos, N, ids, s.optics, s.optics["size"], s.view, s.image_wj)
    Fo, _ = oc.image(s.state, ng, s.optics, s.size_table["size"], s.view, s.image_wj)
    for k in range(len(s.image_wj)):
        assert abs(img[k].sum().item() / Fo[k].sum() - 1.0) < 1e-13


def lorentz_system():
    """The image-loss ring with 40 gravitating planetesimals, charged grains and a stellar
    field (the Lorentz force on)."""
    s = adj.adjoint_system(n_dust=96, xsize=64, ysize=64, n_steps=6, seed=31, n_plsml=40)
    s.phys = dict(s.phys, FLQ=1, Bstar=5e-20, Wz=14.6)
    s.size_table = dict(s.size_table, q=np.linspace(1e-3, 2e-3, len(s.size_table["q"])).astype(np.float32))
    return s


def lorentz_constants(s):
    """cL = q Bstar Rstar^3 / m per tracer, the Lorentz force's coefficient."""
    ng = s.n_grav
    ids = s.state["id"][ng:]
    q = s.size_table["q"].astype(np.float64)[ids]
    return torch.tensor(q * s.phys["Bstar"] * s.phys["Rstar"] ** 3 / s.state["m"][ng:])


def test_torch_trajectory_with_planetesimals_and_lorentz_matches_c_oracle():
    s = lorentz_system()
    ng = s.n_grav
    ids = torch.tensor(s.state["id"][ng:], dtype=torch.int64)
    beta = torch.tensor(s.size_table["beta"].astype(np.float64))[ids]
    betasw = torch.tensor(s.size_table["betasw"].astype(np.float64))[ids]
    massive = torch.tensor(np.stack([s.state[k][:ng] for k in ("x", "y", "z", "vx", "vy", "vz", "m")], 1))
    dust = torch.tensor(np.stack([s.state[k][ng:] for k in ("x", "y", "z", "vx", "vy", "vz")], 1))
    with torch.no_grad():
        out = tr.trajectory(massive, dust, beta, betasw, s.dt, 6, s.phys["SWQ"], s.phys["vsw_AUyr"],
                            lorentz=(lorentz_constants(s), s.phys["Wz"])).numpy()
        plain = tr.trajectory(massive, dust, beta, betasw, s.dt, 6, s.phys["SWQ"], s.phys["vsw_AUyr"]).numpy()
    ref = oc.step(s.state, ng, s.dt, s.size_table, s.phys, 6)
    for c, k in enumerate(("x", "y", "z", "vx", "vy", "vz")):
        np.testing.assert_allclose(out[:, c], ref[k][ng:], rtol=1e-12, atol=1e-12)
    assert np.abs(plain[:, 3] - out[:, 3]).max() > 1e-9   # the force matters on this system
