"""Near sources in the mixed step: a planetesimal nearer to a body than eta times the body's
largest |coordinate| takes the FP64 pair force (ddx_set_near_radius), so close encounters
do not amplify the FP32 rounding of that pull.

Planted close pairs (grains 0.05 to 0.3 AU from a planetesimal, planetesimals 0.05 AU from
each other: inside the default radius anywhere in the ring, and still resolved by the step)
make that pull's FP32 rounding the largest error of the pair.  With the default radius their
positions after 5 steps stay within 1e-12 (relative) of the FP64 step's, the level of the
other grains; with the radius set to 0 (every planetesimal in FP32) they are orders of
magnitude further off.  The spatially ordered step (1,100 planetesimals) and the index-order
step (256) are both covered, and so is the massive set's sliced pass.
"""
import numpy as np
import pytest
import torch

from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_phys

pytestmark = pytest.mark.gpu


def rel_err(a, b, sl):
    pa = np.stack([a[f][sl] for f in ("x", "y", "z")])
    pb = np.stack([b[f][sl] for f in ("x", "y", "z")])
    return np.linalg.norm(pa - pb, axis=0) / np.linalg.norm(pb, axis=0)


def planted(n_plsml, n_dust=4096, n_grain_pairs=64, n_body_pairs=16, seed=41):
    """A dusty ring in which the first n_grain_pairs grains sit 0.05..0.3 AU from a
    planetesimal with its velocity (plus 1e-3 AU/yr), and the first n_body_pairs
    planetesimals of the second half sit 0.05 AU from one of the first half."""
    s = synth.dusty_ring(n_dust=n_dust, n_plsml=n_plsml, seed=seed, n_steps=5)
    st = {k: v.copy() for k, v in s.state.items()}
    g = np.random.default_rng(seed)
    ng = s.n_grav
    half = (ng - 3) // 2
    for k in range(n_body_pairs):
        i, j = 3 + k, 3 + half + k
        for a, f in enumerate("xyz"):
            st[f][j] = st[f][i] + (0.05 if a == 0 else 0.0)
            st["v" + f][j] = st["v" + f][i]
    src = g.choice(np.arange(3, ng), n_grain_pairs, replace=False)
    d = g.normal(size=(n_grain_pairs, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= 10 ** g.uniform(np.log10(0.05), np.log10(0.3), (n_grain_pairs, 1))
    for k, j in enumerate(src):
        t = ng + k
        for a, f in enumerate("xyz"):
            st[f][t] = st[f][j] + d[k, a]
            st["v" + f][t] = st["v" + f][j] + 1e-3 * d[k, a] / np.linalg.norm(d[k])
    body_rows = np.concatenate([np.arange(3, 3 + n_body_pairs), np.arange(3 + half, 3 + half + n_body_pairs)])
    return synth.System(s.name, ng, st, s.dt, 5, s.phys, s.size_table), body_rows


def run(engine, s, prec, eta=None, n_steps=5):
    engine.set_size_table(**s.size_table)
    engine.set_near_radius(-1.0 if eta is None else eta)
    st = DeviceState.from_numpy(s.state)
    engine.evolve(st, s.n_grav, s.dt, n_steps, make_phys(**s.phys), prec, abi.DDX_MODE_FIXED)
    torch.cuda.synchronize()
    engine.set_near_radius(-1.0)      # back to the defaults
    return st.to_numpy()


@pytest.mark.parametrize("n_plsml", [256, 1100])
def test_near_sources_take_the_fp64_pull(engine, n_plsml):
    s, body_rows = planted(n_plsml)
    ng = s.n_grav
    f = run(engine, s, abi.DDX_PREC_FP64)
    m = run(engine, s, abi.DDX_PREC_MIXED)
    m0 = run(engine, s, abi.DDX_PREC_MIXED, eta=0.0)
    np.testing.assert_array_equal(f["N"] != 0, m["N"] != 0)
    grains = slice(ng, ng + 64)
    e_near, e_off = rel_err(m, f, grains), rel_err(m0, f, grains)
    live = f["N"][grains] != 0
    assert e_near[live].max() < 1e-12, e_near[live].max()
    assert np.median(e_off[live]) > 100 * max(np.median(e_near[live]), 1e-16)
    eb_near = rel_err(m, f, body_rows)
    eb_off = rel_err(m0, f, body_rows)
    assert eb_near.max() < 1e-12, eb_near.max()
    assert eb_off.max() > 100 * eb_near.max()
    # the other grains and bodies: the usual mixed error
    rest = rel_err(m, f, slice(ng + 64, None))[f["N"][ng + 64:] != 0]
    assert np.quantile(rest, 0.99) < 1e-12
    assert rel_err(m, f, slice(0, ng)).max() < 1e-12


def test_near_radius_zero_is_the_plain_fp32_step(engine):
    """eta = 0 takes no FP64 pull; results do not depend on the radius when nothing is near."""
    s = synth.dusty_ring(n_dust=2048, n_plsml=1100, seed=9, n_steps=2)
    a = run(engine, s, abi.DDX_PREC_MIXED, eta=0.0, n_steps=2)
    b = run(engine, s, abi.DDX_PREC_MIXED, eta=1e-9, n_steps=2)   # a radius of ~1e-7 AU: nothing near
    for k in ("x", "y", "z", "vx", "vy", "vz", "N"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_near_radius_argument_checks(engine):
    lib = engine.lib
    import ctypes as C
    assert lib.ddx_set_near_radius(engine.ctx, C.c_double(0.3)) == abi.DDX_ERR_ARG
    assert lib.ddx_set_near_radius(engine.ctx, C.c_double(float("nan"))) == abi.DDX_ERR_ARG
    assert lib.ddx_set_near_radius(engine.ctx, C.c_double(0.25)) == abi.DDX_OK
    assert lib.ddx_set_near_radius(engine.ctx, C.c_double(-1.0)) == abi.DDX_OK   # the defaults again
