"""The run clock and output cadence of Grid::evolve on the host: ddx_schedule (the clock
ddx_run uses) against the oracle's restatement of the reference's loop, and the file
writer of the run outputs."""
import math
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import abi, formats, run

MASK = {"sed": 1 << abi.DDX_OUT_SED, "images": 1 << abi.DDX_OUT_IMAGES, "state": 1 << abi.DDX_OUT_STATE}

CADENCES = {
    "aligned": (dict(t_write=1.0, t_fits=0.5, t_sed=0.25, t_end=3.0), 0.05),
    "awkward": (dict(t_write=1.1, t_fits=0.7, t_sed=0.3, t_end=10.0), 0.0537),
    "outputs_finer_than_dt": (dict(t_write=0.07, t_fits=0.03, t_sed=0.011, t_end=1.0), 0.2),
    "restart_mid_interval": (dict(t_write=100.0, t_fits=10.0, t_sed=25.0, t_end=333.3, time=41.123456789,
                                  tlastd=0.0, tlastf=40.0, tlasts=25.0), 0.83),
    "long": (dict(t_write=1000.0, t_fits=100.0, t_sed=500.0, t_end=2000.0), 0.0913),
}


@pytest.mark.parametrize("name", list(CADENCES))
def test_schedule_is_the_reference_clock(built_lib, name):
    cad, dt = CADENCES[name]
    h, m = run.schedule(cad, dt)
    ref = oc.cadence(cad, dt)
    assert len(h) == len(ref)
    np.testing.assert_array_equal(h, [s for s, _ in ref])                     # step sizes to the bit
    np.testing.assert_array_equal(m, [sum(MASK[k] for k in due) for _, due in ref])
    assert m[-1] == sum(MASK.values())                                          # everything at t_end


def test_schedule_hits_output_times(built_lib):
    cad, dt = CADENCES["awkward"]
    h, m = run.schedule(cad, dt)
    t = np.cumsum(h)
    sed = t[(m & MASK["sed"]) != 0]
    assert len(sed) == math.ceil(cad["t_end"] / cad["t_sed"])
    np.testing.assert_allclose(np.diff(sed)[:-1], cad["t_sed"], rtol=1e-12)


def test_finished_run_takes_no_step(built_lib):
    """A run whose clock already reached t_end: the reference's do-while makes one step of
    size t_end - time (zero or negative) and writes its outputs; ddx_run makes none."""
    cad = dict(t_write=1.0, t_fits=1.0, t_sed=1.0, t_end=5.0, time=5.0, tlastd=5.0, tlastf=5.0, tlasts=5.0)
    h, _ = run.schedule(cad, 0.1)
    assert len(h) == 0
    ref = oc.cadence(cad, 0.1)
    assert len(ref) == 1 and ref[0][0] == 0.0


def test_file_writer_names_and_contents(built_lib, tmp_path):
    p = formats.read_param_struct(Path(__file__).parent / "golden" / "setup" / "disks_blobs.param")
    w = np.array([0.55e-6, 1.6e-6, 24e-6, 70e-6])
    influx = np.array([1e-9, 5e-10, 1e-12, 1e-14])
    view = abi.View(dist=3.0e17, fov=120.0, PA=0.0, inc=0.5, longitude=0.0, xsize=4, ysize=3)
    wj = [1, 2]
    n = 7
    writer = run.file_writer(tmp_path, "sys", "2.0-gb300", p, w, influx, wj, np.zeros(8, np.float32), view,
                             n_mass=2, n_dust=4, Rmax=100.0)
    writer({"kind": abi.DDX_OUT_IMAGES, "time": 12.5, "model_dt": 0.0, "tlastd": 0, "tlastf": 0, "tlasts": 0,
            "data": np.arange(2 * 12, dtype=np.float64)})
    writer({"kind": abi.DDX_OUT_SED, "time": 12.5, "model_dt": 0.0, "tlastd": 0, "tlastf": 0, "tlasts": 0,
            "data": np.array([0.0, 1e-3, 2e-3, 3e-3])})
    st = {k: np.linspace(1, 2, n) for k in ("x", "y", "z", "vx", "vy", "vz", "N", "m")}
    st["id"] = np.full(n, -1, np.int32)
    writer({"kind": abi.DDX_OUT_STATE, "time": 12.5, "model_dt": 0.0, "tlastd": 12.5, "tlastf": 12.5,
            "tlasts": 12.5, "state": st})
    names = sorted(Path(f).name for f in writer.written)
    assert names == sorted(["sys_1.60_12.500.fits", "sys_24.00_12.500.fits", "sys_SED_12.50.dat", "sys_12.50.dat"])
    q, r, b = formats.read_dat(tmp_path / "sys_12.50.dat", "2.0-gb300", Rmax=100.0)
    assert r.time == 12.5 and r.tlastd == 12.5 and r.n_all == n
    np.testing.assert_allclose(b["x"], st["x"], rtol=1e-8)
