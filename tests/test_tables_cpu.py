"""Optical-table and stellar-spectrum set-up on the host, pinned to the reference.

tests/golden/optics/ holds synthetic Mie table and spectrum files in the reference's formats
and what the reference's own add_optical_data, add_specfile, interpolate_stellar_to_grid,
interpolate_dust_to_grid and calculate_beta made of them (tests/golden/make_optics_golden.py).
The library's file readers and ddx_stellar_grid give the reference's values to the bit, and
so does the oracle's restatement of the size grid and beta tables, which the GPU tests then
use as the checker."""
import importlib.util
import shutil
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import abi, formats

GOLD = Path(__file__).resolve().parent / "golden" / "optics"
CASES = ("typical", "narrow_spectrum", "many_bins")
GRID_KEYS = ("n_grid", "amin", "amax", "dmax", "kqe", "radQ", "SWQ", "rho", "dist", "mstar", "mloss", "vsw")


def load(case):
    d = np.load(GOLD / f"{case}.npz")
    return {k: d[k] for k in d.files}


def file_table(d):
    return {"s": d["file_s"], "Qabs": d["file_Qabs"], "Qsca": d["file_Qsca"], "Qpfunc": d["file_Qpfunc"]}


def grid_args(d):
    return {k: (int(d[k]) if k in ("n_grid", "radQ", "SWQ") else float(d[k])) for k in GRID_KEYS}


@pytest.mark.parametrize("case", CASES)
def test_optical_file_read_bit_exact(built_lib, case):
    d = load(case)
    t = formats.read_optical(GOLD / f"{d['table']}_table.dat")
    np.testing.assert_array_equal(t["w"], d["w"])
    for k in ("s", "Qabs", "Qsca", "Qpfunc"):
        np.testing.assert_array_equal(t[k], d["file_" + k], err_msg=k)
    assert (t["dmin"], t["dmax"]) == (d["dmin"], d["dmax"])


@pytest.mark.parametrize("case", CASES)
def test_spectrum_read_bit_exact(built_lib, case):
    d = load(case)
    w, F = formats.read_spec(GOLD / f"{d['spec']}_spec.dat", float(d["rstar"]), float(d["dist"]))
    np.testing.assert_array_equal(w, d["spec_w"])
    np.testing.assert_array_equal(F, d["spec_F"])


@pytest.mark.parametrize("case", CASES)
def test_stellar_grid_bit_exact(built_lib, case):
    d = load(case)
    for fn in (formats.stellar_grid, oc.stellar_grid):
        influx, wj = fn(d["w"], d["spec_w"], d["spec_F"], d["wavs"])
        np.testing.assert_array_equal(influx, d["in"])
        np.testing.assert_array_equal(wj, d["wj"])


@pytest.mark.parametrize("case", CASES)
def test_oracle_dust_grid_bit_exact(case):
    d = load(case)
    o = oc.dust_grid(d["w"], d["in"], file_table(d), **grid_args(d))
    for k in ("s", "q", "Qabs", "Qsca", "Qpfunc", "beta", "betasw"):
        np.testing.assert_array_equal(o[k], d[k], err_msg=k)
    assert o["Lum"] == d["Lum"] and o["betaswconst"] == d["betaswconst"]


def test_fixture_cases_cover_the_edges():
    t, n, m = load("typical"), load("narrow_spectrum"), load("many_bins")
    assert t["s"][-1] == t["dmax"]                              # last bin snapped onto dmax
    assert m["s"][0] == m["file_s"][1]                          # a bin exactly on a table size
    assert n["wj"][0] == -1                                     # image wavelength = w[0]
    assert (n["in"] == 0).any() and n["w"][-1] > n["spec_w"][-1]   # zero flux, w^-4 tail
    assert (t["in"][:1] == 0).all()                             # below the spectrum / zero head


def test_image_wavelength_outside_table_rejected(built_lib):
    d = load("typical")
    with pytest.raises(abi.DDXError) as e:
        formats.stellar_grid(d["w"], d["spec_w"], d["spec_F"], [d["w"][-1] * 1.01])
    assert e.value.status == 5
    with pytest.raises(ValueError, match="43"):
        oc.stellar_grid(d["w"], d["spec_w"], d["spec_F"], [d["w"][0] * 0.99])


def test_table_wavelength_on_the_last_spectrum_point(built_lib):
    """The reference's walk would read past the spectrum here; both implementations stop on
    the last point and give its flux."""
    d = load("typical")
    w = np.array([d["spec_w"][-3], d["spec_w"][-1], d["spec_w"][-1] * 1.5])
    a, _ = formats.stellar_grid(w, d["spec_w"], d["spec_F"])
    b, _ = oc.stellar_grid(w, d["spec_w"], d["spec_F"])
    np.testing.assert_array_equal(a, b)
    assert a[1] == pytest.approx(d["spec_F"][-1], rel=1e-14)


def test_oracle_bin_on_the_first_table_size():
    """amin == s[0] (the optical file's smallest size, where the reference reads s[-1]):
    the first interval is used, which returns the first size's values."""
    d = load("typical")
    g = grid_args(d)
    g["amin"] = float(d["file_s"][0])
    o = oc.dust_grid(d["w"], d["in"], file_table(d), **g)
    np.testing.assert_allclose(o["Qabs"][0], d["file_Qabs"][0], rtol=1e-14)
    np.testing.assert_allclose(o["Qpfunc"][0], d["file_Qpfunc"][0], rtol=1e-14)


def test_oracle_last_bin_overshoot_rejected():
    d = load("typical")
    g = grid_args(d)
    g["dmax"] = g["amax"] * (1 - 1e-6)
    with pytest.raises(ValueError, match="54"):
        oc.dust_grid(d["w"], d["in"], file_table(d), **g)


def test_optical_header_only(built_lib):
    import ctypes as C
    t = abi.OpticalTable()
    lo, hi = C.c_double(), C.c_double()
    st = abi.load().ddx_optical_read(str(GOLD / "t2_table.dat").encode(), C.byref(t), None, C.byref(lo), C.byref(hi))
    assert st == 0 and (t.n_size, t.n_wav, t.n_theta) == (5, 20, 5)
    assert (lo.value, hi.value) == (float("5.000000e-01") * 1e-6, float("5.000000e+01") * 1e-6)


def _edit(tmp_path, fn):
    lines = (GOLD / "t2_table.dat").read_text().splitlines(keepends=True)
    p = tmp_path / "table.dat"
    p.write_text("".join(fn(lines)))
    return p


@pytest.mark.parametrize("kind", ["values_before_first_size", "extra_size", "missing_phase_row", "extra_wavelength"])
def test_malformed_optical_files_rejected(built_lib, tmp_path, kind):
    """Where the reference would write outside its arrays or leave them partly unset."""
    first_size = 2
    if kind == "values_before_first_size":
        p = _edit(tmp_path, lambda L: L[:first_size] + ["1.0 0.5 0.5\n"] + L[first_size:])
    elif kind == "extra_size":
        p = _edit(tmp_path, lambda L: L + L[first_size:first_size + 31])
    elif kind == "missing_phase_row":
        p = _edit(tmp_path, lambda L: L[:-1])
    else:
        p = _edit(tmp_path, lambda L: L[:first_size + 1] + ["1.0 0.5 0.5\n"] + L[first_size + 1:])
    with pytest.raises(abi.DDXError) as e:
        formats.read_optical(p)
    assert e.value.status == 1


def test_missing_files(built_lib, tmp_path):
    with pytest.raises(abi.DDXError) as e:
        formats.read_optical(tmp_path / "absent.dat")
    assert e.value.status == 8
    with pytest.raises(abi.DDXError) as e:
        formats.read_spec(tmp_path / "absent.dat", 1.0, 1.0)
    assert e.value.status == 8


def test_spectrum_reader_skips_comments_and_partial_lines(built_lib, tmp_path):
    p = tmp_path / "spec.dat"
    p.write_text("# header\n1e-7 2.0\n\nonly\nabc 3.0\n2e-7 x\n3e-7@4.0 trailing words\n")
    w, F = formats.read_spec(p, 1.0, 1.49598e11)        # scale (rstar AU / dist)^2 = 1
    np.testing.assert_array_equal(w, [1e-7, 3e-7])
    np.testing.assert_array_equal(F, [2.0, 4.0])


from oracle.ref.paths import SRC as _REF_SRC  # noqa: E402

REF_SRC = _REF_SRC / "read_in.cu"


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc absent")
@pytest.mark.parametrize("case", CASES)
def test_reference_reproduces_fixtures(tmp_path, case):
    from oracle.ref import paths
    paths.require(REF_SRC)
    spec = importlib.util.spec_from_file_location("mog", Path(__file__).parent / "golden" / "make_optics_golden.py")
    mog = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mog)
    from oracle.ref import build_param_ref
    exe = build_param_ref.build_optics()
    c = mog.CASES[case]
    got = mog.run_reference(exe, GOLD / f"{c['table']}_table.dat", GOLD / f"{c['spec']}_spec.dat", c,
                            tmp_path / "out.bin")
    d = load(case)
    for k, v in got.items():
        np.testing.assert_array_equal(v, d[k], err_msg=k)
