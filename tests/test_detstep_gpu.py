"""ddx_det_step (Grid::det_step, src/grid.cu:312-342) on the GPU state against the oracle's
restatement of the reference's host loop: identical to the bit."""
import math

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import synth
from diskdyn_gb300.engine import DeviceState

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["solar_like", "dusty_ring"])
def test_det_step_bit_identical_to_reference_loop(engine, name):
    s = synth.solar_like(n_dust=64) if name == "solar_like" else synth.dusty_ring(n_dust=64, n_plsml=4096)
    st = DeviceState.from_numpy(s.state)
    for n_step in (1, 100, 300):
        assert engine.det_step(st, s.n_grav, n_step) == oc.det_step(s.state, s.n_grav, n_step)
    disks, blobs = [80.0, 30.0], [(40.0, 0.3, 2.0)]
    assert engine.det_step(st, s.n_grav, 300, disks, blobs) == oc.det_step(s.state, s.n_grav, 300, disks, blobs)


def test_det_step_degenerate_ring_takes_every_body():
    """3,000 equal bodies on one circle: every key ties with the minimum, more than the
    candidate buffer holds, so the scan hands every body to the host."""
    from diskdyn_gb300.engine import Engine
    n = 3001
    phi = np.linspace(0.0, 2 * math.pi, n - 1, endpoint=False)
    st = {"x": np.concatenate([[0.0], 50.0 * np.cos(phi)]), "y": np.concatenate([[0.0], 50.0 * np.sin(phi)]),
          "z": np.zeros(n), "vx": np.zeros(n), "vy": np.zeros(n), "vz": np.zeros(n),
          "m": np.concatenate([[synth.GRAV], np.full(n - 1, 1e-9 * synth.GRAV)]),
          "N": np.ones(n), "id": np.full(n, -1, np.int32)}
    eng = Engine(0)
    try:
        d = DeviceState.from_numpy(st)
        assert eng.det_step(d, n, 300) == oc.det_step(st, n, 300)
        assert eng.det_step(d, 1, 300, [5.0]) == oc.det_step(st, 1, 300, [5.0])
        assert eng.det_step(d, 1, 300) == 1e137
    finally:
        eng.close()
