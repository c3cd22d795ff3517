"""The ddyn_gb300 program against the same run made through the Python API: a parameter file
(disks, blobs and a planet), a Mie table and a spectrum, FP64 with the reference's generator,
run for 150 years with the file's output intervals.  The program calls the C ABI the way a
patched Grid would (src/ddyn.cu's main); the Python side makes the same calls through
ctypes.  Both write the reference's files: the data files and SEDs must be the same bytes,
the FITS images the same to the last bits of the FP64 pixel sums (whose atomic order
varies)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from diskdyn_gb300 import abi, build, formats, run as runmod, synth
from diskdyn_gb300.engine import DeviceState, Engine, make_phys, make_view

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden"
PARAM = GOLD / "setup" / "disks_blobs.param"
TABLE = GOLD / "optics" / "t1_table.dat"
SPEC = GOLD / "optics" / "s1_spec.dat"
T_END = 150.0


def python_run(out: Path):
    p = formats.read_param_struct(PARAM)
    p.t_end = T_END
    tab = formats.read_optical(TABLE)
    sw, sf = formats.read_spec(SPEC, p.rstar, p.dist)
    influx, wj = formats.stellar_grid(tab["w"], sw, sf, wavs=np.array(p.wavs[:p.nwavs]))
    formats.param_grid(p, tab["dmin"], tab["dmax"])
    eng = Engine(0)
    g = eng.dust_grid(tab["w"], influx, tab, n_grid=p.n_grid, amin=p.amin, amax=p.amax, dmax=tab["dmax"],
                      kqe=p.kqe, radQ=p.radQ, SWQ=p.SWQ, rho=p.rho, dist=p.dist, mstar=p.planets[0].m,
                      mloss=p.mloss, vsw=p.vsw)
    disks = [p.disks[k] for k in range(p.n_disks)]
    blobs = [p.blobs[k] for k in range(p.n_blobs)]
    planets = [p.planets[k] for k in range(1, p.n_planets)]
    rmax_in = max([d.Rout for d in disks] + [b.a * (1.0 + b.ecc) + b.sigma for b in blobs] +
                  [float(np.sqrt(q.x * q.x + q.y * q.y + q.z * q.z)) for q in planets] + [0.0])
    Td, Rmin, Rmax = eng.dust_temp(tab["w"], influx, g["Qabs"], p.dist, rmax_in)
    state, run = formats.setup_host(p, tab["dmin"], tab["dmax"], g["beta"])
    eng.set_size_table(size=g["s"], beta=g["beta"], betasw=g["betasw"], q=g["q"])
    eng.set_optics(tab["w"], influx, g["Qabs"], g["Qsca"], g["Qpfunc"], Td, Rmin, Rmax)
    st = DeviceState.from_numpy(state)
    n_grav = p.n_planets + run.n_mass
    dt = eng.det_step(st, n_grav, p.n_step, [d.Rin for d in disks], [(b.a, b.ecc, b.sigma) for b in blobs])
    phys = make_phys(radQ=p.radQ, SWQ=p.SWQ, FLQ=p.FLQ, Wz=p.Wz, Bstar=p.Bstar, Rstar=p.rstar, rho=p.rho,
                     vsw_AUyr=p.vsw * synth.YEAR / synth.AU, Rmin=Rmin, n_planets=p.n_planets)
    view = make_view(p.dist, p.fov, p.PA, p.inc, p.longitude, p.xsize, p.ysize)
    cad = dict(t_write=p.t_write, t_fits=p.t_fits, t_sed=p.t_sed, t_end=p.t_end, initial_outputs=1)
    writer = runmod.file_writer(out, p.name_stub.decode(), "2.0-gb300", p, tab["w"], influx, wj, g["beta"], view,
                                n_mass=run.n_mass, n_dust=run.n_dust, Rmax=Rmax)
    eng.run(st, n_grav, dt, phys, view, wj, cad, writer, precision=abi.DDX_PREC_FP64, mode=abi.DDX_MODE_FIXED)
    eng.close()


def fits_image(path: Path) -> np.ndarray:
    b = path.read_bytes()
    end = next(i for i in range(0, len(b), 80) if b[i:i + 3] == b"END" and b[i + 3:i + 80].strip() == b"")
    start = (end // 2880 + 1) * 2880
    return np.frombuffer(b[start:], dtype=">f8")


def test_driver_writes_the_files_of_the_python_api(tmp_path):
    exe = build.build_driver()
    a, b = tmp_path / "driver", tmp_path / "api"
    a.mkdir()
    b.mkdir()
    r = subprocess.run([str(exe), str(PARAM), "--table", str(TABLE), "--spec", str(SPEC), "--out", str(a),
                        "--t-end", str(T_END)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    python_run(b)
    names = sorted(f.name for f in a.iterdir())
    assert names == sorted(f.name for f in b.iterdir())
    kinds = {n.rsplit(".", 1)[1] for n in names}
    assert kinds == {"dat", "fits"} and sum(n.endswith(".fits") for n in names) >= 2 * 3
    assert any(n.endswith(f"_{T_END:.2f}.dat") and "_SED_" not in n for n in names)
    for n in names:
        if n.endswith(".dat"):
            assert (a / n).read_bytes() == (b / n).read_bytes(), n
        else:
            fa, fb = fits_image(a / n), fits_image(b / n)
            np.testing.assert_allclose(fa, fb, rtol=1e-12, atol=1e-300, err_msg=n)
            assert np.count_nonzero(fa) > 0
