"""DDX_PREC_COMPENSATED: the massive set in FP64 and the planetesimals' pull on each tracer
in float-float (pairs of FP32 numbers through error-free transformations) for the spans
within the compensated radius, FP32 beyond, FP64 for sources within the near radius.

The target it is built for: over 1,000 steps of the dusty ring (all 4,099 massive bodies,
a 16,384-grain shard) every grain and every massive body ends within 1e-9 (relative) of
the FP64 step's position.  The plain mixed step stays near 3e-11 at the median but ends up
1e-8 and more off for a few grains: this chaotic system amplifies the FP32 rounding of the
pulls by three to four orders of magnitude, and float-float removes most of it.  The worst
grain of a shard still varies from draw to draw (on one of four shards measured it ends
2.3e-9 away); the test holds the bench's shard to the target and every shard's 99th
percentile far below it.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_phys

pytestmark = pytest.mark.gpu


def run(engine, s, n_steps, prec, comp_eta=None):
    engine.set_size_table(**s.size_table)
    engine.set_near_radius(-1.0)
    if comp_eta is not None:
        engine.set_compensated_radius(comp_eta)
    st = DeviceState.from_numpy(s.state)
    engine.evolve(st, s.n_grav, s.dt, n_steps, make_phys(**s.phys), prec, abi.DDX_MODE_FIXED)
    torch.cuda.synchronize()
    engine.set_compensated_radius(0.5)
    return st


def rel(a, b, sl):
    d = torch.sqrt((a.x - b.x) ** 2 + (a.y - b.y) ** 2 + (a.z - b.z) ** 2)
    r = torch.sqrt(b.x ** 2 + b.y ** 2 + b.z ** 2)
    return (d / r)[sl].double().cpu().numpy()


@pytest.mark.parametrize("n_plsml", [256, 1100])
def test_compensated_twenty_steps_at_the_fp64_level(engine, n_plsml):
    s = synth.dusty_ring(n_dust=8192, n_plsml=n_plsml, seed=13, n_steps=20)
    f = run(engine, s, 20, abi.DDX_PREC_FP64)
    c = run(engine, s, 20, abi.DDX_PREC_COMPENSATED)
    m = run(engine, s, 20, abi.DDX_PREC_MIXED)
    ng = s.n_grav
    assert torch.equal(f.N != 0, c.N != 0)
    live = (f.N[ng:] != 0).cpu().numpy()
    ec, em = rel(c, f, slice(ng, None))[live], rel(m, f, slice(ng, None))[live]
    assert ec.max() < 1e-12 and np.median(ec) < 1e-14
    assert np.median(em) > 4 * max(np.median(ec), 1e-17)
    assert rel(c, f, slice(0, ng)).max() < 1e-13          # the massive set is FP64 here


def test_compensated_thousand_steps_within_1e9_of_fp64(engine):
    s = synth.dusty_ring(n_dust=16384, n_plsml=4096, seed=synth.SEED + 17, n_steps=1000)
    f = run(engine, s, 1000, abi.DDX_PREC_FP64)
    c = run(engine, s, 1000, abi.DDX_PREC_COMPENSATED)
    ng = s.n_grav
    assert torch.equal(f.N != 0, c.N != 0)
    live = (f.N[ng:] != 0).cpu().numpy()
    ed = rel(c, f, slice(ng, None))[live]
    em = rel(c, f, slice(1, ng))
    print(f"compensated vs FP64, 1,000 steps: dust median {np.median(ed):.3e} max {ed.max():.3e}; "
          f"massive max {em.max():.3e}")
    assert ed.max() <= 1e-9 and em.max() <= 1e-9
    assert np.quantile(ed, 0.99) <= 3e-11


def test_compensated_thousand_steps_other_shard_p99(engine):
    """Another draw of the shard: the worst grain may pass closer to a planetesimal than any
    on the bench's shard, but 99 % of the grains stay two orders of magnitude under 1e-9."""
    s = synth.dusty_ring(n_dust=16384, n_plsml=4096, seed=synth.SEED + 18, n_steps=1000)
    f = run(engine, s, 1000, abi.DDX_PREC_FP64)
    c = run(engine, s, 1000, abi.DDX_PREC_COMPENSATED)
    ng = s.n_grav
    assert torch.equal(f.N != 0, c.N != 0)
    live = (f.N[ng:] != 0).cpu().numpy()
    ed = rel(c, f, slice(ng, None))[live]
    assert np.quantile(ed, 0.99) <= 3e-11 and np.median(ed) <= 5e-12
    assert ed.max() <= 1e-8 and rel(c, f, slice(1, ng)).max() <= 1e-9


def test_compensated_radius_infinite_and_argument_checks(engine):
    """Every span float-float (radius +inf) agrees with the default radius to the FP64 level;
    a negative or NaN radius is refused."""
    s = synth.dusty_ring(n_dust=4096, n_plsml=1100, seed=5, n_steps=5)
    a = run(engine, s, 5, abi.DDX_PREC_COMPENSATED)
    b = run(engine, s, 5, abi.DDX_PREC_COMPENSATED, comp_eta=float("inf"))
    ng = s.n_grav
    live = (a.N[ng:] != 0).cpu().numpy()
    assert rel(a, b, slice(ng, None))[live].max() < 1e-13
    lib = engine.lib
    assert lib.ddx_set_compensated_radius(engine.ctx, C.c_double(-1.0)) == abi.DDX_ERR_ARG
    assert lib.ddx_set_compensated_radius(engine.ctx, C.c_double(float("nan"))) == abi.DDX_ERR_ARG
    assert lib.ddx_set_compensated_radius(engine.ctx, C.c_double(0.5)) == abi.DDX_OK


def test_compensated_removes_coincident_and_nonfinite_tracers_like_fp64(engine):
    s = synth.dusty_ring(n_dust=2048, n_plsml=300, seed=3, n_steps=2)
    st = {k: v.copy() for k, v in s.state.items()}
    ng = s.n_grav
    for f in ("x", "y", "z"):
        st[f][ng + 0] = st[f][10]                 # on top of a planetesimal
    st["x"][ng + 1] = np.nan
    st["y"][ng + 2] = np.inf
    s2 = synth.System(s.name, ng, st, s.dt, 2, s.phys, s.size_table)
    f = run(engine, s2, 2, abi.DDX_PREC_FP64)
    c = run(engine, s2, 2, abi.DDX_PREC_COMPENSATED)
    assert torch.equal(f.N != 0, c.N != 0)
    assert not bool((c.N[ng:ng + 3] != 0).any())
