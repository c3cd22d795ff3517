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


def ring():
    return synth.dusty_ring(n_dust=20000, n_plsml=1024, seed=31, n_steps=20)


def permuted(state, n_grav, perm):
    out = {}
    for k, v in state.items():
        v = np.asarray(v)
        out[k] = np.concatenate([v[:n_grav], v[n_grav:][perm]])
    return out


def test_mixed_step_does_not_depend_on_tracer_order(engine):
    s = ring()
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


def test_mixed_step_repeats_bit_for_bit(engine):
    s = ring()
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
