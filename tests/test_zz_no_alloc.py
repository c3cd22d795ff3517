"""ddx_step_noalloc: the RK4 step for callers that cannot allocate device memory.

Those callers -- a host inside a framework whose pool allocator owns the device memory,
or a loop that must keep a fixed device footprint -- get a step whose scratch is a fixed
file-scope device array instead of cudaMalloc'd context buffers.  The test calls it
through the C ABI twice in a row (the second call reuses the array the first one left
behind) and checks every result against ddx_step on the same input: bit for bit in FP64,
where both run the same kernels.  In mixed precision, from 1,024 planetesimals on, the
context's step visits the tracers and the sources in a spatial order and takes far sources
with the high-part separation, which the fixed array has no room to order for; the test
then allows 1e-12 of the largest position or velocity component after two steps and the
same removed tracers.  It passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_phys

pytestmark = pytest.mark.gpu


def noalloc_step(lib, st, sysm, tab, prec, mode):
    phys = make_phys(**sysm.phys)
    r = lib.ddx_step_noalloc(0, C.byref(st._abi), sysm.n_grav, st.n_all - sysm.n_grav, C.c_double(sysm.dt),
                             C.byref(phys), len(tab["beta"]), C.c_void_p(tab["beta"].data_ptr()),
                             C.c_void_p(tab["betasw"].data_ptr()), C.c_void_p(tab["q"].data_ptr()),
                             prec, mode, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    abi.check(r, "ddx_step_noalloc")


@pytest.mark.parametrize("prec", [abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED])
@pytest.mark.parametrize("mode", [abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE])
def test_noalloc_step_matches_ddx_step_twice(built_lib, prec, mode):
    from diskdyn_gb300.engine import Engine
    lib = abi.load()
    eng = Engine(0)
    sysm = synth.dusty_ring(n_dust=4096, n_plsml=1100, seed=21, n_steps=2)   # ddx_step orders in space
    eng.set_size_table(**sysm.size_table)
    tab = {k: torch.tensor(np.asarray(sysm.size_table[k], np.float32), device="cuda")
           for k in ("beta", "betasw", "q")}
    a = DeviceState.from_numpy(sysm.state)
    b = DeviceState.from_numpy(sysm.state)
    for _ in range(2):
        eng.step(a, sysm.n_grav, sysm.dt, make_phys(**sysm.phys), prec, mode)
        noalloc_step(lib, b, sysm, tab, prec, mode)
        torch.cuda.synchronize()
        for f in ("x", "y", "z", "vx", "vy", "vz", "N"):
            if prec == abi.DDX_PREC_FP64 or f == "N":
                assert torch.equal(getattr(a, f), getattr(b, f)), f
            else:
                group = ("x", "y", "z") if f in ("x", "y", "z") else ("vx", "vy", "vz")
                scale = max(float(getattr(a, g).abs().max()) for g in group)
                u, v = getattr(a, f), getattr(b, f)
                assert float((u - v).abs().max()) <= 1e-12 * scale, f
    eng.close()


def test_noalloc_reports_a_wait_that_ran_out(built_lib):
    """A mixed call whose bounded wait runs out (the test hook leaves one tile's copy
    unissued and bounds the waits by 20 ms) leaves every tracer unchanged and is reported
    once by ddx_noalloc_sync_status; the next call steps normally and reports nothing."""
    lib = abi.load()
    sysm = synth.dusty_ring(n_dust=2048, n_plsml=256, seed=7, n_steps=2)
    tab = {k: torch.tensor(np.asarray(sysm.size_table[k], np.float32), device="cuda")
           for k in ("beta", "betasw", "q")}
    st = DeviceState.from_numpy(sysm.state)
    h = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    lib.ddx_noalloc_sync_status(0, h)                      # nothing pending from earlier calls
    ng = sysm.n_grav
    before = st.to_numpy()
    abi.check(lib.ddx_debug_noalloc_lose_tile_copy(0, 1, 20_000_000), "inject")
    noalloc_step(lib, st, sysm, tab, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
    assert lib.ddx_noalloc_sync_status(0, h) == abi.DDX_ERR_TIMEOUT
    after = st.to_numpy()
    for f in ("x", "y", "z", "vx", "vy", "vz", "N"):
        assert np.array_equal(after[f][ng:], before[f][ng:]), f
    assert lib.ddx_noalloc_sync_status(0, h) == abi.DDX_OK   # the report was cleared
    noalloc_step(lib, st, sysm, tab, abi.DDX_PREC_MIXED, abi.DDX_MODE_FIXED)
    assert lib.ddx_noalloc_sync_status(0, h) == abi.DDX_OK
    assert not np.array_equal(st.to_numpy()["x"][ng:], before["x"][ng:])


def test_noalloc_rejects_sizes_beyond_its_limit(built_lib):
    lib = abi.load()
    sysm = synth.solar_like(n_dust=8)
    st = DeviceState.from_numpy(sysm.state)
    phys = make_phys(**sysm.phys)
    tab = torch.zeros(4, dtype=torch.float32, device="cuda")
    p = C.c_void_p(tab.data_ptr())
    too_many = abi.load().ddx_step_noalloc(0, C.byref(st._abi), 8193, 0, C.c_double(0.1), C.byref(phys),
                                            4, p, p, p, 0, 0, None)
    assert too_many == 5
    assert lib.ddx_step_noalloc(0, C.byref(st._abi), sysm.n_grav, 8, C.c_double(0.1), C.byref(phys),
                                2701, p, p, p, 0, 0, None) == 5
    assert lib.ddx_step_noalloc(0, C.byref(st._abi), 0, 8, C.c_double(0.1), C.byref(phys),
                                4, p, p, p, 0, 0, None) == 1
