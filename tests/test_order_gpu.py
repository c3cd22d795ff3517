"""The spatial order of the mixed step (ddx_order.cu): the step visits the tracers and reads
the planetesimals in cell order, and a tracer far from a span of 32 planetesimals takes
their separation from the high parts alone.  That choice depends on the tracer and the
sources only, so a tracer's result does not depend on where it sits in the state, nor on
the order inside a cell, which comes from atomics.  Checked bit for bit on a ring where far
spans occur (1,024 planetesimals, tracers all around the ring)."""
import numpy as np
import pytest
import torch

from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_phys

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N")


def ring(n_plsml=1024):
    return synth.dusty_ring(n_dust=20000, n_plsml=n_plsml, seed=31, n_steps=20)


def permuted(state, n_grav, perm):
    out = {}
    for k, v in state.items():
        v = np.asarray(v)
        out[k] = np.concatenate([v[:n_grav], v[n_grav:][perm]])
    return out


@pytest.mark.parametrize("n_plsml", [1024, 9000])   # the planetesimals ordered in one block / by radix sort
def test_mixed_step_does_not_depend_on_tracer_order(engine, n_plsml):
    s = ring(n_plsml)
    engine.set_size_table(**s.size_table)
    n_dust = len(s.state["x"]) - s.n_grav
    perm = np.random.default_rng(7).permutation(n_dust)
    a = DeviceState.from_numpy(s.state)
    b = DeviceState.from_numpy(permuted(s.state, s.n_grav, perm))
    phys = make_phys(**s.phys)
    for _ in range(3):
        engine.step(a, s.n_grav, s.dt, phys, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
        engine.step(b, s.n_grav, s.dt, phys, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
    torch.cuda.synchronize()
    inv = torch.as_tensor(np.argsort(perm), device="cuda")
    for f in FIELDS:
        u, v = getattr(a, f), getattr(b, f)
        assert torch.equal(u[:s.n_grav], v[:s.n_grav]), f
        assert torch.equal(u[s.n_grav:], v[s.n_grav:][inv]), f


@pytest.mark.parametrize("n_plsml", [1024, 9000])
def test_mixed_step_repeats_bit_for_bit(engine, n_plsml):
    s = ring(n_plsml)
    engine.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    runs = []
    for _ in range(2):
        st = DeviceState.from_numpy(s.state)
        for _ in range(3):
            engine.step(st, s.n_grav, s.dt, phys, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
        torch.cuda.synchronize()
        runs.append(st)
    for f in FIELDS:
        assert torch.equal(getattr(runs[0], f), getattr(runs[1], f)), f


def test_far_spans_keep_the_mixed_error(engine):
    """The planetesimals moved in to 12-14 AU (radii and speeds scaled as circular orbits)
    while the grains stay at 120-140 AU: every span is far from every grain (at least
    106 AU against half the largest coordinate, about 70 AU), so all their
    pulls take the high-part separation.  Against FP64 over 20 steps the mixed run stays
    within the bounds of the near-span test (median 1e-13, p99 1e-12)."""
    s = synth.dusty_ring(n_dust=16384, n_plsml=1024, seed=5, n_steps=20)
    st = {k: np.array(v, copy=True) for k, v in s.state.items()}
    q = slice(3, s.n_grav)                        # planetesimals (star and two planets first)
    for f in ("x", "y", "z"):
        st[f][q] *= 0.1
    for f in ("vx", "vy", "vz"):
        st[f][q] *= 0.1 ** -0.5
    engine.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    out = {}
    for prec in (abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED):
        d = DeviceState.from_numpy(st)
        engine.evolve(d, s.n_grav, s.dt, 20, phys, prec, abi.DDX_MODE_FIXED)
        torch.cuda.synchronize()
        out[prec] = d.to_numpy()
    f, m = out[abi.DDX_PREC_FP64], out[abi.DDX_PREC_MIXED]
    g = slice(s.n_grav, None)
    alive = (f["N"][g] != 0) & (m["N"][g] != 0)
    pf = np.stack([f[k][g] for k in ("x", "y", "z")])
    pm = np.stack([m[k][g] for k in ("x", "y", "z")])
    e = (np.linalg.norm(pm - pf, axis=0) / np.linalg.norm(pf, axis=0))[alive]
    assert alive.mean() > 0.99
    assert np.median(e) < 1e-13
    assert np.quantile(e, 0.99) < 1e-12


@pytest.mark.parametrize("n_dust", [3000, 100])   # 100 grains: blocks of 64 threads
def test_ordered_step_with_removed_non_finite_and_distant_tracers(engine, n_dust):
    """The ordered step (1,100 planetesimals) with removed tracers (N = 0), a NaN and an
    infinite coordinate, and a tracer at 1e30 AU: the boxes and the far tests take them
    like any other, and the mixed step removes the same tracers as FP64 and keeps the rest
    within the mixed tolerance."""
    s = synth.dusty_ring(n_dust=n_dust, n_plsml=1100, seed=17, n_steps=20)
    st = {k: np.array(v, copy=True) for k, v in s.state.items()}
    g = s.n_grav
    st["N"][g::7] = 0.0
    st["x"][g + 5] = np.nan
    st["y"][g + 9] = np.inf
    st["z"][g + 13] = 1e30
    engine.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    out = {}
    for prec in (abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED):
        d = DeviceState.from_numpy(st)
        engine.step(d, g, s.dt, phys, prec, abi.DDX_MODE_FIXED)
        torch.cuda.synchronize()
        out[prec] = d.to_numpy()
    f, m = out[abi.DDX_PREC_FP64], out[abi.DDX_PREC_MIXED]
    np.testing.assert_array_equal(m["N"] == 0, f["N"] == 0)
    assert f["N"][g + 5] == 0 and f["N"][g + 9] == 0
    ok = (f["N"][g:] != 0) & np.isfinite(f["x"][g:])
    pf = np.stack([f[k][g:][ok] for k in ("x", "y", "z")])
    pm = np.stack([m[k][g:][ok] for k in ("x", "y", "z")])
    e = np.linalg.norm(pm - pf, axis=0) / np.linalg.norm(pf, axis=0)
    assert e.max() < 1e-12


@pytest.mark.parametrize("n_plsml", [1100, 9000])
def test_grains_step_alike_alone_and_among_many(engine, n_plsml):
    """A tracer's result depends only on its own state and the massive set, not on the other
    grains (which set the spatial visiting order, the blocks' span choices and the block
    size): the first 20,000 grains of a 400,000-grain system step to the same bits as those
    20,000 grains alone."""
    s = synth.dusty_ring(n_dust=400_000, n_plsml=n_plsml, seed=23, n_steps=2)
    ng = s.n_grav
    sub = {k: np.asarray(v)[:ng + 20000].copy() for k, v in s.state.items()}
    engine.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    big, small = DeviceState.from_numpy(s.state), DeviceState.from_numpy(sub)
    for _ in range(2):
        engine.step(big, ng, s.dt, phys, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
        engine.step(small, ng, s.dt, phys, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
    torch.cuda.synchronize()
    for f in FIELDS:
        assert torch.equal(getattr(big, f)[:ng + 20000], getattr(small, f)), f
