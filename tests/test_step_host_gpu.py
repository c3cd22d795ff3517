"""ddx_step_host: one step of a system in host memory, the dust streamed through the GPU in
up to three chunks with the copies on their own streams.  Each tracer's step does
not depend on the others, so the result must equal ddx_step on the device bit for bit,
whatever the chunking.  The reference mode and the spatially ordered mixed step (1,024
planetesimals or more) run unchunked; FP64, and mixed with the 64 planetesimals here, run
500,000 grains in three chunks of unequal size."""
import numpy as np
import pytest
import torch

from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, Engine, make_phys

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")


def pinned(arrays):
    return {f: torch.from_numpy(np.ascontiguousarray(arrays[f])).pin_memory() for f in FIELDS}


@pytest.mark.parametrize("prec,mode", [(abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED),
                                       (abi.DDX_PREC_FP64, abi.DDX_MODE_FIXED),
                                       (abi.DDX_PREC_MIXED, abi.DDX_MODE_REFERENCE)])
def test_host_step_equals_device_step(prec, mode):
    n_dust = 500000     # fixed mode: three chunks of unequal size
    s = synth.dusty_ring(n_dust=n_dust, n_plsml=64, seed=12)
    eng = Engine(0)
    eng.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    ref = DeviceState.from_numpy(s.state)
    eng.step(ref, s.n_grav, s.dt, phys, prec, mode)
    want = ref.to_numpy()
    host_in = pinned(s.state)
    host_out = {f: torch.empty_like(t).pin_memory() for f, t in host_in.items()}
    host_out["m"].copy_(host_in["m"])
    host_out["id"].copy_(host_in["id"])
    dev = DeviceState.from_numpy({f: np.zeros_like(s.state[f]) for f in FIELDS})
    eng.step_host(dev, host_in, host_out, s.n_grav, s.dt, phys, prec, mode)
    for f in FIELDS:
        np.testing.assert_array_equal(host_out[f].numpy(), want[f], err_msg=f)
    # in place: the same host arrays in and out, a second step against the device's second step
    eng.step_host(dev, host_out, host_out, s.n_grav, s.dt, phys, prec, mode)
    eng.step(ref, s.n_grav, s.dt, phys, prec, mode)
    want = ref.to_numpy()
    for f in FIELDS:
        np.testing.assert_array_equal(host_out[f].numpy(), want[f], err_msg=f)


def test_host_step_rejects_short_host_arrays():
    import ctypes as C
    from diskdyn_gb300.formats import HostState
    s = synth.dusty_ring(n_dust=1000, n_plsml=8, seed=3)
    eng = Engine(0)
    eng.set_size_table(**s.size_table)
    dev = DeviceState.from_numpy(s.state)
    h = pinned(s.state)
    hs = HostState(*[h[f].data_ptr() for f in FIELDS], len(s.state["x"]) - 1)
    r = eng.lib.ddx_step_host(eng.ctx, C.byref(hs), C.byref(hs), C.byref(dev._abi), s.n_grav, s.n_dust, s.dt,
                              C.byref(make_phys(**s.phys)), abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED, None)
    assert r == 1
