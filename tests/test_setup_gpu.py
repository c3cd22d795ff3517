"""ddx_setup_device: the initial system drawn on the GPU.

Counts, order, grain masses, size bins and grain numbers are those of ddx_setup_host (which
is the reference's set-up to the bit, tests/test_setup_cpu.py); the gravitating masses come
from the same chain evaluated without cancellation, within 1e-5 of the reference's (whose own
rounding of that chain is of that order).  The orbits come from the
counter-based generator: compared body for body with the oracle's restatement of it, to
rounding (the CUDA math library's log, pow, sin and cos instead of libm, and contracted
products): 1e-12 of each body's radius or speed."""
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import abi, formats

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "setup"


def system(case, scale=1):
    d = np.load(GOLD / f"{case}.npz")
    d = {k: d[k] for k in d.files}
    p = formats.read_param_struct(GOLD / f"{case}.param")
    for j in range(p.n_disks):
        p.disks[j].Nsmall *= scale
    for j in range(p.n_blobs):
        p.blobs[j].Nsmall *= scale
    formats.param_grid(p, float(d["dmin"]), float(d["dmax"]))
    return d, p


def to_host(st):
    return {f: getattr(st, f).cpu().numpy() for f in ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")}


@pytest.mark.parametrize("case,scale", [("disks_blobs", 1), ("rejections", 1), ("disks_blobs", 30)])
def test_setup_device_matches_oracle(engine, case, scale):
    d, p = system(case, scale)
    dmin, dmax = float(d["dmin"]), float(d["dmax"])
    host, run = formats.setup_host(p, dmin, dmax, d["beta"])
    st, run_g = engine.setup_device(p, dmin, dmax, d["beta"], seed=2024)
    g = to_host(st)
    assert (run_g.n_all, run_g.n_mass, run_g.n_dust) == (run.n_all, run.n_mass, run.n_dust)
    for k in ("N", "id"):
        np.testing.assert_array_equal(g[k], host[k], err_msg=k)
    # gravitating masses: the getbod chain in double, formed without cancellation (1e-16 of
    # a high-precision evaluation), against the reference's chain, whose next limit mmin
    # carries double rounding into a difference of two nearly equal powers: 7.8e-7 for
    # this file's blob
    grains = host["id"] >= 0
    np.testing.assert_array_equal(g["m"][grains], host["m"][grains])
    np.testing.assert_allclose(g["m"][~grains], host["m"][~grains], rtol=1e-5, atol=0)
    npl = p.n_planets
    for k in ("x", "y", "z", "vx", "vy", "vz"):                  # star and planets: copied
        np.testing.assert_array_equal(g[k][:npl], host[k][:npl])
    kind, idx = oc.setup_populations(p, dmin, dmax)
    ids = host["id"][npl:]
    beta = np.where(ids >= 0, d["beta"][np.maximum(ids, 0)].astype(np.float64), 0.0)
    beta[beta >= 0.5] = 0.0
    ref, bad = oc.setup_philox(p, kind, idx, host["m"][npl:], beta, 2024, npl)
    assert bad == 0
    gp = np.stack([g[k][npl:] for k in ("x", "y", "z")], 1)
    gv = np.stack([g[k][npl:] for k in ("vx", "vy", "vz")], 1)
    finite = np.isfinite(ref).all(1)
    assert (np.isfinite(np.hstack([gp, gv])).all(1) == finite).all()
    r = np.linalg.norm(ref[finite, :3], axis=1, keepdims=True)
    v = np.linalg.norm(ref[finite, 3:], axis=1, keepdims=True)
    assert (np.abs(gp[finite] - ref[finite, :3]) <= 1e-12 * r).all()
    assert (np.abs(gv[finite] - ref[finite, 3:]) <= 1e-12 * v).all()
    np.testing.assert_array_equal(np.isnan(gp[:, 0]), np.isnan(ref[:, 0]))


def test_setup_device_is_reproducible(engine):
    d, p = system("disks_blobs", 5)
    a, _ = engine.setup_device(p, float(d["dmin"]), float(d["dmax"]), d["beta"], seed=99)
    b, _ = engine.setup_device(p, float(d["dmin"]), float(d["dmax"]), d["beta"], seed=99)
    c, _ = engine.setup_device(p, float(d["dmin"]), float(d["dmax"]), d["beta"], seed=100)
    assert all(bool((getattr(a, f) == getattr(b, f)).all()) for f in ("x", "vx", "vz"))
    assert not bool((a.vx[p.n_planets:] == c.vx[p.n_planets:]).any())


def test_setup_device_rejects_small_capacity(engine):
    import ctypes as C
    import torch
    d, p = system("disks_blobs")
    run = formats.setup_count(p, float(d["dmin"]), float(d["dmax"]))
    n = run.n_all - 1
    ts = {f: torch.zeros(n, dtype=torch.int32 if f == "id" else torch.float64, device="cuda") for f in
          ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")}
    from diskdyn_gb300.engine import DeviceState
    st = DeviceState(**ts)
    beta = np.ascontiguousarray(d["beta"], np.float32)
    r = engine.lib.ddx_setup_device(engine.ctx, C.byref(p), float(d["dmin"]), float(d["dmax"]),
                                    C.c_void_p(beta.ctypes.data), 1, C.byref(st._abi), n, C.byref(run), None)
    assert r == abi.DDX_OK + 5
