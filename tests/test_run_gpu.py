"""ddx_run: Grid::evolve's loop with its output cadence in one call.

Checked against the same run done call by call (ddx_step with the step sizes of
ddx_schedule, which tests/test_run_cpu.py pins to the reference's clock, then ddx_sed,
ddx_image and a state copy at each output): the states and SEDs are identical (the step and
the SED are deterministic); the images' pixel sums are atomics whose order varies, so they
agree to 1e-12 (FP64 sums) or 1e-5 (the mixed images' FP32 sums)."""
from pathlib import Path

import numpy as np
import pytest

from diskdyn_gb300 import abi, formats, run, synth
from diskdyn_gb300.engine import DeviceState, Engine, make_phys, make_view

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")


def setup(n_dust=3000, xsize=48, ysize=40):
    s = synth.dusty_ring(n_dust=n_dust, n_plsml=24, seed=31, n_steps=300)
    synth.ring_imaging(s, xsize, ysize)
    eng = Engine(0)
    eng.set_size_table(**s.size_table)
    o = s.optics
    eng.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])
    return s, eng


def manual(s, eng, cad, dt, prec):
    """The run done call by call: a list of (kind, time, payload)."""
    st = DeviceState.from_numpy(s.state)
    ng = s.n_grav
    phys, view, wj = make_phys(**s.phys), make_view(**s.view), s.image_wj
    out = []

    def emit(kind, t):
        if kind == "images":
            out.append((abi.DDX_OUT_IMAGES, t, eng.image(st, ng, view, wj, precision=prec).cpu().numpy().ravel()))
        elif kind == "sed":
            out.append((abi.DDX_OUT_SED, t, eng.sed(st, ng, view, precision=prec).cpu().numpy()))
        else:
            out.append((abi.DDX_OUT_STATE, t, {f: getattr(st, f).cpu().numpy() for f in FIELDS}))

    t = cad.get("time", 0.0)
    if cad.get("initial_outputs"):
        for k in ("images", "sed", "state"):
            emit(k, t)
    h, m = run.schedule(cad, dt)
    for k in range(len(h)):
        eng.step(st, ng, float(h[k]), phys, prec)
        t += h[k]
        for bit, kind in ((abi.DDX_OUT_SED, "sed"), (abi.DDX_OUT_IMAGES, "images"), (abi.DDX_OUT_STATE, "state")):
            if m[k] & (1 << bit):
                emit(kind, t)
    return out


@pytest.mark.parametrize("prec", [abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED])
def test_run_equals_the_call_by_call_run(prec):
    s, eng = setup()
    dt = s.dt
    cad = dict(t_write=7 * dt, t_fits=3.3 * dt, t_sed=2.1 * dt, t_end=20.5 * dt, initial_outputs=1)
    got = []
    st = DeviceState.from_numpy(s.state)
    clock = eng.run(st, s.n_grav, dt, make_phys(**s.phys), make_view(**s.view), s.image_wj, cad, got.append,
                    precision=prec)
    ref = manual(s, eng, cad, dt, prec)
    assert [(o["kind"], o["time"]) for o in got] == [(k, t) for k, t, _ in ref]
    for o, (kind, t, payload) in zip(got, ref):
        if kind == abi.DDX_OUT_STATE:
            for f in FIELDS:
                np.testing.assert_array_equal(o["state"][f], payload[f], err_msg=f)
            assert o["tlastd"] == t
        elif kind == abi.DDX_OUT_SED:
            np.testing.assert_array_equal(o["data"], payload)
        else:   # atomics in another order: FP64 sums (FP64 images), FP32 sums (mixed images)
            rtol = 1e-12 if prec == abi.DDX_PREC_FP64 else 1e-5
            np.testing.assert_allclose(o["data"], payload, rtol=rtol, atol=1e-300)
    assert clock["time"] == ref[-1][1]
    assert ref[-1][0] == abi.DDX_OUT_STATE                  # t_end: SED, images, then the state
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(st, f).cpu().numpy(), ref[-1][2][f], err_msg=f)


def test_run_stops_when_the_callback_asks():
    s, eng = setup(n_dust=1000)
    dt = s.dt
    cad = dict(t_write=100 * dt, t_fits=100 * dt, t_sed=2 * dt, t_end=50 * dt)
    got = []

    def on(o):
        got.append(o["time"])
        return len(got) >= 2

    st = DeviceState.from_numpy(s.state)
    clock = eng.run(st, s.n_grav, dt, make_phys(**s.phys), make_view(**s.view), s.image_wj, cad, on)
    assert len(got) >= 2 and clock["time"] < cad["t_end"]


def test_run_writes_the_reference_files(tmp_path):
    s, eng = setup(n_dust=1500)
    dt = s.dt
    p = formats.read_param_struct(Path(__file__).parent / "golden" / "setup" / "disks_blobs.param")
    formats.param_grid(p, 1e-7, 1e-4)                       # the data-file header's grid
    cad = dict(t_write=10 * dt, t_fits=5 * dt, t_sed=10 * dt, t_end=10 * dt, initial_outputs=1)
    view = make_view(**s.view)
    o = s.optics
    beta = np.asarray(s.size_table["beta"], np.float32)
    writer = run.file_writer(tmp_path, "ring", "2.0-gb300", p, o["w"], o["in"], s.image_wj, beta, view,
                             n_mass=s.n_grav - p.n_planets, n_dust=s.n_dust, Rmax=o["Rmax"])
    st = DeviceState.from_numpy(s.state)
    eng.run(st, s.n_grav, dt, make_phys(**s.phys), view, s.image_wj, cad, writer)
    names = {f.name for f in tmp_path.iterdir()}
    t1 = 10 * dt
    w = o["w"]
    for t in (0.0, t1):
        assert f"ring_{t:.2f}.dat" in names and f"ring_SED_{t:.2f}.dat" in names
        for k in s.image_wj:
            assert f"ring_{w[k] * 1e6:.2f}_{t:.3f}.fits" in names
    assert f"ring_{w[s.image_wj[0]] * 1e6:.2f}_{5 * dt:.3f}.fits" in names
    _, r, b = formats.read_dat(tmp_path / f"ring_{t1:.2f}.dat", "2.0-gb300", Rmax=o["Rmax"])
    np.testing.assert_allclose(b["x"], st.x.cpu().numpy(), rtol=1e-8, atol=1e-12)
