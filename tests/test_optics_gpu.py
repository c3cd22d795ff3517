"""Optics set-up on the GPU.

ddx_dust_temp (Grid::calculate_dust_temp, src/grid.cu:754-834) against the oracle's
restatement of the reference's host loop.  Tolerances: the Planck sums use the CUDA math
library's exp, log and pow instead of libm, so the tables agree to rounding: 1e-12 relative
for the temperatures, 1e-13 for the grid limits.

ddx_dust_grid (interpolate_dust_to_grid and calculate_beta, src/functions.cu:243-388)
against the reference's own output on the committed fixtures and against the oracle (pinned
to the reference bit for bit) on full-size tables; tolerances in assert_grid_close."""
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import abi, synth

pytestmark = pytest.mark.gpu


def nongrey(n_grid=24, n_wav=120):
    """Q_abs = 1 - exp(-2 pi s / lambda): grains absorb less at wavelengths beyond their size,
    so the bins have different equilibrium temperatures (and sublimation radii)."""
    opt = synth.hg_optics(n_grid=n_grid, n_theta=5, n_wav=n_wav, L=8.7, Teff=7500.0, Rstar=2.0 * synth.RSun)
    s, w = opt["size"], opt["w"]
    opt["Qabs"] = 1.0 - np.exp(-2 * np.pi * s[:, None] / w[None, :])
    return opt


@pytest.mark.parametrize("case", ["grey", "nongrey"])
def test_dust_temp_matches_oracle(engine, case):
    opt = synth.hg_optics(n_grid=16, n_wav=200) if case == "grey" else nongrey()
    dist = 10 * synth.PC
    for rmax in (50.0, 400.0):
        Td, rmin, rmax_out = engine.dust_temp(opt["w"], opt["in"], opt["Qabs"], dist, rmax)
        To, rmin_o, rmax_o = oc.dust_temp(opt["w"], opt["in"], opt["Qabs"], dist, rmax)
        assert rmax_out == rmax_o == 2 * rmax
        assert rmin == pytest.approx(rmin_o, rel=1e-13)
        assert np.isfinite(Td).all()
        np.testing.assert_allclose(Td, To, rtol=1e-12)


# -- size grid and beta tables (interpolate_dust_to_grid, calculate_beta) --------------------

GOLD = Path(__file__).resolve().parent / "golden" / "optics"
GRID_KEYS = ("n_grid", "amin", "amax", "dmax", "kqe", "radQ", "SWQ", "rho", "dist", "mstar", "mloss", "vsw")


def golden(case):
    d = np.load(GOLD / f"{case}.npz")
    d = {k: d[k] for k in d.files}
    table = {"s": d["file_s"], "Qabs": d["file_Qabs"], "Qsca": d["file_Qsca"], "Qpfunc": d["file_Qpfunc"]}
    g = {k: (int(d[k]) if k in ("n_grid", "radQ", "SWQ") else float(d[k])) for k in GRID_KEYS}
    return d, table, g


def assert_grid_close(out, ref):
    """The bin radii, q, beta_sw, Lum and the wind constant come from the host with the
    reference's rounding: identical.  The tables use the CUDA math library's log and exp
    (1 ulp) in the reference's operation order: 1e-13 relative.  beta is a float32 of a
    sum of those: within one float32 ulp."""
    for k in ("s", "q", "betasw"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    assert out["Lum"] == ref["Lum"] and out["betaswconst"] == ref["betaswconst"]
    for k in ("Qabs", "Qsca", "Qpfunc"):
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-13, atol=0, err_msg=k)
    ulp = np.spacing(np.abs(ref["beta"]).astype(np.float32))
    assert (np.abs(out["beta"].astype(np.float64) - ref["beta"]) <= ulp).all()


@pytest.mark.parametrize("case", ["typical", "narrow_spectrum", "many_bins"])
def test_dust_grid_matches_reference_fixture(engine, case):
    d, table, g = golden(case)
    out = engine.dust_grid(d["w"], d["in"], table, **g)
    assert_grid_close(out, d)


def test_dust_grid_full_size_tables_match_oracle(engine):
    """218 bins (1 to 1000 micron at a mass ratio of 1.1) on 200 wavelengths x 181 angles."""
    w, influx, table = synth.mie_table()
    g = dict(n_grid=218, amin=1.3e-7, amax=float(table["s"][-1]), dmax=float(table["s"][-1]), kqe=3e-3, radQ=1,
             SWQ=1, rho=3300.0, dist=7.7 * synth.PC, mstar=2.1 * 4 * np.pi ** 2, mloss=1e-13, vsw=5e5)
    out = engine.dust_grid(w, influx, table, **g)
    ref = oc.dust_grid(w, influx, table, **g)
    assert np.isfinite(out["Qpfunc"]).all() and (out["beta"] > 0).all()
    assert_grid_close(out, ref)


def test_dust_grid_bin_on_first_table_size(engine):
    d, table, g = golden("typical")
    g["amin"] = float(d["file_s"][0])
    out = engine.dust_grid(d["w"], d["in"], table, **g)
    ref = oc.dust_grid(d["w"], d["in"], table, **g)
    assert_grid_close(out, ref)
    np.testing.assert_allclose(out["Qabs"][0], d["file_Qabs"][0], rtol=1e-14)


def test_dust_grid_rejects_last_bin_beyond_dmax(engine):
    d, table, g = golden("typical")
    g["dmax"] = g["amax"] * (1 - 1e-6)
    with pytest.raises(abi.DDXError) as e:
        engine.dust_grid(d["w"], d["in"], table, **g)
    assert e.value.status == 5
