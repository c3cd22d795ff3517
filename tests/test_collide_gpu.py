"""Spatial-hash collision pairs on the GPU against CPU brute force (ground truth) and a
CPU cell list, bit for bit: same pairs, same (i, j) order."""
import math

import numpy as np
import pytest
import torch

import oracle.cpu as oc
from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState

pytestmark = pytest.mark.gpu


def gpu_pairs(engine, state, i0, i1, h, cap=None):
    st = DeviceState.from_numpy(state)
    p = engine.collide(st, i0, i1, h, cap)
    torch.cuda.synchronize()
    return p.cpu().numpy(), engine.last_pair_count


def test_pairs_match_brute_force_ring(engine):
    s = synth.dusty_ring(n_dust=20000, n_plsml=64, seed=9)
    n = len(s.state["x"])
    for h in (0.05, 0.5, 2.0):
        g, tot = gpu_pairs(engine, s.state, s.n_grav, n, h)
        o = oc.collide(s.state, s.n_grav, n, h, "brute")
        assert tot == len(o)
        np.testing.assert_array_equal(g, o)
    # a buffer too small keeps the first cap pairs of the ordered list
    for cap in (1, tot // 3, tot - 1):
        part, tot2 = gpu_pairs(engine, s.state, s.n_grav, n, 2.0, cap)
        assert tot2 == tot
        np.testing.assert_array_equal(part, o[:cap])


def test_pairs_match_cell_list_full_size(engine):
    s = synth.dusty_ring(n_dust=1048576, n_plsml=4096, seed=2)
    n = len(s.state["x"])
    g, tot = gpu_pairs(engine, s.state, s.n_grav, n, 0.1)
    o = oc.collide(s.state, s.n_grav, n, 0.1, "grid")
    assert tot == len(o) > 1000
    np.testing.assert_array_equal(g, o)


def cluster_state(n, seed=4):
    g = synth.rng(seed)
    st = {k: g.normal(0.0, 1e-3, n) + 50.0 for k in ("x", "y", "z")}
    st.update({k: np.zeros(n) for k in ("vx", "vy", "vz", "m")})
    st["N"] = np.ones(n)
    st["id"] = np.full(n, -1, np.int32)
    return st


def test_dense_cluster_dead_tracers_and_capacity(engine):
    st = cluster_state(3000)
    st["N"][::7] = 0.0                       # removed tracers take no part
    g, tot = gpu_pairs(engine, st, 0, 3000, 2e-3)
    o = oc.collide(st, 0, 3000, 2e-3, "brute")
    assert tot == len(o) > 100000
    np.testing.assert_array_equal(g, o)
    # buffers too small: the cut falls inside tracers' segments of tens of partners (found
    # by a second walk), which keep their smallest j
    for cap in (1000, 77777):
        part, tot2 = gpu_pairs(engine, st, 0, 3000, 2e-3, cap=cap)
        assert tot2 == tot
        np.testing.assert_array_equal(part, o[:cap])


def test_boundary_distances_and_cell_edges(engine):
    # pairs at exactly h (excluded), one ulp inside (included), straddling cell edges
    h = 0.25
    xs = [10.0, 10.0 + h, 20.0, np.nextafter(20.0 + h, 0.0), 30.0 - 1e-13, 30.0 + h - 2e-13,
          h * 4 - 1e-15, h * 5 - 1e-15]
    n = len(xs)
    st = {"x": np.array(xs), "y": np.zeros(n), "z": np.zeros(n), "vx": np.zeros(n), "vy": np.zeros(n),
          "vz": np.zeros(n), "m": np.zeros(n), "N": np.ones(n), "id": np.full(n, -1, np.int32)}
    g, tot = gpu_pairs(engine, st, 0, n, h)
    o = oc.collide(st, 0, n, h, "brute")
    np.testing.assert_array_equal(g, o)
    assert [0, 1] not in o.tolist() and [2, 3] in o.tolist()


def margin_state(base, h, n, seed):
    """n tracers within +-1.2 h of (base, base, base) on each axis, plus pairs placed at one
    FP64 step inside and outside h along a diagonal."""
    g = synth.rng(seed)
    pts = base + g.uniform(-1.2 * h, 1.2 * h, (n, 3))
    d = np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    extra = []
    for k in range(8):
        a = base + g.uniform(-h, h, 3)
        for f in (1.0 - 2.0 ** -50, 1.0, 1.0 + 2.0 ** -50):
            extra += [a, a + d * h * f]
    pts = np.vstack([pts, np.array(extra)])
    m = len(pts)
    st = {"x": pts[:, 0].copy(), "y": pts[:, 1].copy(), "z": pts[:, 2].copy(), "vx": np.zeros(m), "vy": np.zeros(m),
          "vz": np.zeros(m), "m": np.zeros(m), "N": np.ones(m), "id": np.full(m, -1, np.int32)}
    return st, m


@pytest.mark.parametrize("base,h", [(130.0, 0.1), (1.0, 0.3), (1.0e5, 0.25), (3.0e3, 1e-4), (-2.5e4, 0.5),
                                    (7.0e15, 1e3), (0.0, 1e-13)])
def test_float_rejection_keeps_every_pair(engine, base, h):
    """The FP32 rejection in front of the FP64 test drops no pair: separations within one FP64
    step of h where its margin is small against h (the ring's scale), at coordinates where a
    float's step (2^-23 of the coordinate) is near or above h, beyond the range where the
    rejection is used (1e15), and at an h below it (1e-12)."""
    st, m = margin_state(base, h, 400, 11)
    g, tot = gpu_pairs(engine, st, 0, m, h)
    o = oc.collide(st, 0, m, h, "brute")
    assert tot == len(o) > 0
    np.testing.assert_array_equal(g, o)


def test_empty_and_single_ranges(engine):
    s = synth.solar_like(n_dust=16)
    n = len(s.state["x"])
    for i0, i1 in ((n, n), (n - 1, n), (3, 3)):
        g, tot = gpu_pairs(engine, s.state, i0, i1, 1.0)
        assert tot == 0 and len(g) == 0
    with pytest.raises(abi.DDXError):
        gpu_pairs(engine, s.state, 0, n, -1.0)
    with pytest.raises(abi.DDXError):
        gpu_pairs(engine, s.state, 5, 2, 1.0)


def test_non_finite_positions_take_no_pairs(engine):
    """Tracers with NaN or infinite coordinates get a cell like any other (the conversion
    saturates, or gives 0 for NaN), never pass the distance test, and leave the other
    pairs as brute force finds them."""
    st = cluster_state(2000, seed=8)
    st["x"][10] = np.nan
    st["y"][20] = np.inf
    st["z"][30] = -np.inf
    st["x"][40] = 1e300
    g, tot = gpu_pairs(engine, st, 0, 2000, 2e-3)
    o = oc.collide(st, 0, 2000, 2e-3, "brute")
    assert tot == len(o) > 1000
    np.testing.assert_array_equal(g, o)
    assert not np.isin(o, [10, 20, 30, 40]).any()
