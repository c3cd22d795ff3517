"""The oracle against golden vectors from the reference's own kernels (tests/golden/,
made by tests/golden/make_golden.py on a GB300 with the reference's unmodified
src/gpu_functions.cu).  Steps: positions to 1e-11 relative and identical removal flags
(the oracle computes in libm and without FMA contraction, the reference kernel with the
CUDA math library and nvcc's contraction); images and SED: 1e-11 relative per pixel and
per wavelength."""
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc

GOLD = Path(__file__).resolve().parent / "golden"
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")


def unpack(z, prefix):
    return {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}


def load(name):
    p = GOLD / f"{name}.npz"
    if not p.exists():
        pytest.fail(f"missing golden fixture {p.name}; regenerate with tests/golden/make_golden.py")
    return np.load(p)


@pytest.mark.parametrize("name", ["step_ring", "step_star_lorentz", "step_solar"])
def test_oracle_step_matches_reference_kernel_golden(name):
    z = load(name)
    state = unpack(z, "in_")
    tab = unpack(z, "tab_")
    phys = {k: float(v) for k, v in unpack(z, "phys_").items()}
    ref = unpack(z, "out_")
    n_grav, n_steps = int(z["n_grav"]), int(z["n_steps"])
    o = oc.step(state, n_grav, float(z["dt"]), tab, phys, n_steps, ref_mode=True)
    np.testing.assert_array_equal(o["N"] != 0, ref["N"] != 0)
    alive = ref["N"] != 0
    p_o = np.stack([o[k] for k in ("x", "y", "z")])
    p_r = np.stack([ref[k] for k in ("x", "y", "z")])
    err = np.linalg.norm(p_o - p_r, axis=0) / np.maximum(np.linalg.norm(p_r, axis=0), 1e-300)
    assert err[alive].max() < 1e-11, err[alive].max()
    v_o = np.stack([o[k] for k in ("vx", "vy", "vz")])
    v_r = np.stack([ref[k] for k in ("vx", "vy", "vz")])
    verr = np.linalg.norm(v_o - v_r, axis=0) / np.maximum(np.linalg.norm(v_r, axis=0), 1e-300)
    assert verr[alive].max() < 1e-10, verr[alive].max()


def test_oracle_image_and_sed_match_reference_kernel_golden():
    z = load("flux_small")
    state = unpack(z, "in_")
    opt = unpack(z, "opt_")
    opt["Rmin"], opt["Rmax"] = float(opt["Rmin"]), float(opt["Rmax"])
    view = {k: float(v) for k, v in unpack(z, "view_").items()}
    view["xsize"], view["ysize"] = int(view["xsize"]), int(view["ysize"])
    n_grav = int(z["n_grav"])
    F, _ = oc.image(state, n_grav, opt, opt["size"], view, [int(w) for w in z["wj"]])
    Fr = z["out_image"]
    assert np.array_equal(F != 0, Fr != 0)
    np.testing.assert_allclose(F, Fr, rtol=1e-11, atol=0)
    S = oc.sed(state, n_grav, opt, opt["size"], view, ref_mode=True)
    np.testing.assert_allclose(S, z["out_sed"], rtol=1e-11)
