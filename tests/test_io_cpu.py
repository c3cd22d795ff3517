"""Output and restart files in the reference's formats: the data file (writer, reader, and
the reference's own header reader read_in_model on our file), the SED file and the FITS
image.  The data-file layout is line-numbered (the reference reads its header by line
index), so a writer and a reader that agree with each other and with read_in_model keep
runs interchangeable."""
import json
import math
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from diskdyn_gb300 import formats

GOLD = Path(__file__).resolve().parent / "golden" / "params"
VERSION = "2.0-gb300"
GRAV, MSUN, AU, RSUN = 4.0 * math.pi * math.pi, 1.98892e30, 1.49598e11, 695700000.0


def system(seed=5):
    """A parsed parameter file with the optics-stage fields filled in, and a state of its
    planets, 5 more massive bodies and 200 grains on the mass grid."""
    p = formats.read_param_struct(GOLD / "planets_disks_blobs.param")
    p.amin, p.amax, p.n_grid = 1e-6, 1e-3, 64
    p.mmin = 4.0 / 3.0 * math.pi * p.rho * p.amin ** 3
    p.mmax = 4.0 / 3.0 * math.pi * p.rho * p.amax ** 3
    p.f = math.log(p.mmax / p.mmin) / (p.n_grid - 1.0)
    p.n_wav, p.n_theta, p.n_dust, p.seed = 200, 181, p.n_grid, 987654321
    for k in range(p.n_disks):
        p.disks[k].dmax, p.disks[k].dmmax, p.disks[k].C = 1e-3, 1.1e-5, 3.3e21 * (k + 1)
    for k in range(p.n_blobs):
        p.blobs[k].dmax, p.blobs[k].dmmax, p.blobs[k].C = 2e-3, 8.8e-5, 1.7e19 * (k + 1)
    g = np.random.default_rng(seed)
    ng_extra, nd = 5, 200
    npl = p.n_planets
    n = npl + ng_extra + nd
    a = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz", "N", "m")}
    a["id"] = np.full(n, -1, np.int32)
    for k in range(npl):
        b = p.planets[k]
        for f in ("x", "y", "z", "vx", "vy", "vz", "m"):
            a[f][k] = getattr(b, f)
    a["N"][:npl] = 1.0
    r = g.uniform(20.0, 90.0, n - npl)
    r[-3:] = (150.0, 220.0, 0.001)       # two beyond Rmax and one inside the star
    phi = g.uniform(0, 2 * np.pi, n - npl)
    a["x"][npl:], a["y"][npl:] = r * np.cos(phi), r * np.sin(phi)
    a["z"][npl:] = g.normal(0.0, 1.0, n - npl)
    a["z"][-1] = 0.0
    a["vx"][npl:], a["vy"][npl:] = -np.sin(phi) * 6.0, np.cos(phi) * 6.0
    a["vz"][npl:] = g.normal(0.0, 0.05, n - npl)
    a["m"][npl:npl + ng_extra] = g.uniform(1e-10, 1e-8, ng_extra) * GRAV
    a["N"][npl:npl + ng_extra] = 1.0
    ids = g.integers(0, p.n_grid, nd)
    a["id"][npl + ng_extra:] = ids
    a["m"][npl + ng_extra:] = p.mmin * np.exp(ids * p.f) * GRAV / MSUN
    a["N"][npl + ng_extra:] = 10 ** g.uniform(10, 20, nd)
    run = formats.DatRun(time=1234.5678912, dt=0.0537, tlastd=1200.0, tlastf=1230.5, tlasts=1234.0, Rmax=100.0, nR=100,
                         n_mass=ng_extra, n_dust=nd, n_all=n)
    beta = np.linspace(0.9, 0.001, p.n_grid).astype(np.float32)
    return p, run, a, beta


def test_data_file_round_trip(tmp_path):
    p, run, a, beta = system()
    f1, f2 = tmp_path / "m_1.dat", tmp_path / "m_2.dat"
    formats.write_dat(f1, VERSION, p, run, a, beta)
    q, r, b = formats.read_dat(f1, VERSION, Rmax=run.Rmax)
    # the file carries 9 significant digits of every state value
    for k in ("x", "y", "z", "vx", "vy", "vz", "m"):
        np.testing.assert_allclose(b[k], a[k], rtol=6e-9, atol=1e-300, err_msg=k)
    np.testing.assert_allclose(b["N"], a["N"], rtol=1e-12)
    np.testing.assert_array_equal(b["id"], a["id"])      # recomputed from the masses
    assert (r.n_mass, r.n_dust, r.n_all, r.nR) == (run.n_mass, run.n_dust, run.n_all, 100)
    assert r.time == float("%.8f" % run.time) and r.dt == float("%.8f" % run.dt)
    assert q.seed == p.seed and q.n_grid == p.n_grid and q.n_planets == p.n_planets
    assert q.name_stub == p.name_stub and q.comp == p.comp and q.specfile == p.specfile
    # writing what was read gives the same file, except the radius column, which is
    # derived from the 9-digit mass and may move in its last digit; a second round trip
    # reproduces the file exactly
    formats.write_dat(f2, VERSION, q, r, b, beta)
    l1, l2 = f1.read_text().splitlines(), f2.read_text().splitlines()
    assert len(l1) == len(l2)
    for x, y in zip(l1, l2):
        if x != y:
            tx, ty = x.split(), y.split()
            assert tx[:-3] == ty[:-3] and tx[-2:] == ty[-2:]
            assert float(tx[-3]) == pytest.approx(float(ty[-3]), rel=2e-8)
    q2, r2, b2 = formats.read_dat(f2, VERSION, Rmax=run.Rmax)
    f3 = tmp_path / "m_3.dat"
    formats.write_dat(f3, VERSION, q2, r2, b2, beta)
    assert f3.read_bytes() == f2.read_bytes()
    assert sum(ln.startswith("## ") for ln in l1) == 3      # beyond Rmax or inside the star


def test_data_file_rejects_other_version_or_radius_grid(tmp_path):
    p, run, a, beta = system()
    f = tmp_path / "m.dat"
    formats.write_dat(f, VERSION, p, run, a, beta)
    with pytest.raises(formats.ParamError) as e:
        formats.read_dat(f, "another-version")
    assert e.value.usage_code == 55
    with pytest.raises(formats.ParamError) as e:
        formats.read_dat(f, VERSION, nR=50)
    assert e.value.usage_code == 56


def reference_parser():
    import oracle.ref.build_param_ref as bp
    try:
        return bp.build()
    except RuntimeError:
        return None


def test_reference_reads_our_data_file_header_identically(tmp_path):
    from oracle.ref import paths
    paths.require(paths.SRC / "read_in.cu")
    exe = reference_parser()
    if exe is None:
        pytest.skip("the reference parser could not be built")
    p, run, a, beta = system()
    f = tmp_path / "m.dat"
    formats.write_dat(f, VERSION, p, run, a, beta)
    ref = json.loads(subprocess.run([str(exe), "-m", str(f), VERSION], capture_output=True, text=True,
                                    check=True).stdout)
    q, _, _ = formats.read_dat(f, VERSION)
    h = float.fromhex
    for k in ("t_gl", "t_write", "t_fits", "t_sed", "t_end", "teff", "rstar", "Bstar", "Wz", "mloss", "vsw",
              "dist", "fov", "PA", "inc", "longitude", "rho", "kqe", "amin", "amax", "mmin", "mmax", "f"):
        assert getattr(q, k) == h(ref[k]), k
    for k in ("verb", "gpuid", "gl", "n_step", "xsize", "ysize", "radQ", "SWQ", "FLQ", "n_grid", "n_wav",
              "n_theta", "n_dust"):
        assert getattr(q, k) == ref[k], k
    for k in ("sptype", "specfile", "comp", "name_stub"):
        assert getattr(q, k).decode() == ref[k], k
    assert [q.wavs[i] for i in range(q.nwavs)] == [h(v) for v in ref["wavs"]]
    for i, pl in enumerate(ref["planets"]):
        assert [getattr(q.planets[i], f) for f in ("x", "y", "z", "vx", "vy", "vz", "m")] == [h(v) for v in pl]
    for i, d in enumerate(ref["disks"]):
        for k, v in d.items():
            assert getattr(q.disks[i], k) == (v if k in ("Ngrav", "Nsmall") else h(v)), ("disk", k)
    for i, (dmax, dmmax, C) in enumerate(ref["disks_extra"]):
        assert (q.disks[i].dmax, q.disks[i].dmmax, q.disks[i].C) == (h(dmax), h(dmmax), h(C))
    for i, bl in enumerate(ref["blobs"]):
        for k, v in bl.items():
            assert getattr(q.blobs[i], k) == (v if k in ("Ngrav", "Nsmall", "collcloud") else h(v)), ("blob", k)


def test_sed_file(tmp_path):
    w = np.array([0.5e-6, 1.25e-6, 24e-6, 850e-6])
    influx = np.array([1.1e-9, 3.3e-10, 2.2e-14, 1.0e-19])
    exc = np.array([0.0, 1.5e-5, 2.25e-2, 3.0e-4])
    f = tmp_path / "s_SED_1.00.dat"
    formats.write_sed(f, VERSION, w, influx, exc)
    lines = f.read_text().splitlines()
    assert lines[0] == f"#Calculated with DiskDyn Version {VERSION}"
    assert lines[1] == "#Wav[mu]\tFlux_star[Jy]\tFlux_exc[Jy]"
    for j, ln in enumerate(lines[2:]):
        assert ln == "%.3f %.6e %.6e" % (w[j] * 1e6, influx[j] * 1e26 * w[j] * w[j] / 299792458.0, exc[j])


def read_fits(path):
    raw = Path(path).read_bytes()
    assert len(raw) % 2880 == 0
    cards, off = [], 0
    while True:
        c = raw[off:off + 80].decode("ascii")
        off += 80
        cards.append(c)
        if c.startswith("END"):
            break
    off = (off + 2879) // 2880 * 2880
    kv = {}
    for c in cards:
        if c[8:10] == "= ":
            v = c[10:].split(" / ")[0].strip()
            kv[c[:8].strip()] = v
    nx, ny = int(kv["NAXIS1"]), int(kv["NAXIS2"])
    data = np.frombuffer(raw[off:off + nx * ny * 8], dtype=">f8").reshape(ny, nx)
    return cards, kv, data


def test_fits_image(tmp_path):
    xs, ys = 7, 5
    F = np.arange(xs * ys, dtype=np.float64).reshape(xs, ys) * 1.5e-3 + 1e-6   # x-major, like ddx_image
    f = tmp_path / "s_1.25_10.000.fits"
    formats.write_fits(f, VERSION, F, 1.25e-6, 120.0, 10 * 3.08567758149137e16)
    cards, kv, data = read_fits(f)
    assert all(len(c) == 80 for c in cards)
    assert kv["SIMPLE"] == "T" and kv["BITPIX"] == "-64" and kv["NAXIS"] == "2"
    assert int(kv["NAXIS1"]) == xs and int(kv["NAXIS2"]) == ys
    np.testing.assert_array_equal(data, F.T)                    # image[y][x] = F[x][y]
    assert float(kv["WAVELENG"]) == pytest.approx(1.25, rel=1e-7)
    assert float(kv["FLUX"]) == pytest.approx(F.sum(), rel=1e-15)
    assert float(kv["PIXELSCA"]) == pytest.approx(120.0 / 10.0 / max(xs, ys), rel=1e-6)
    assert kv["VERSION"].strip("'").strip() == VERSION
    assert any(c.startswith("HISTORY Created with DiskDyn") for c in cards)
    assert kv["DATE"].startswith("'20")
