"""The ddyn_gb300 program (diskdyn_gb300/driver/ddyn_gb300.cpp) builds against libddx.so
and reads a parameter file, a Mie table and a spectrum without a GPU (--dry-run): the
counts it prints are those of the same files read through the Python API."""
import subprocess
from pathlib import Path

from diskdyn_gb300 import build, formats

GOLD = Path(__file__).parent / "golden"


def test_driver_dry_run_counts_match_the_api():
    exe = build.build_driver()
    param = GOLD / "setup" / "disks_blobs.param"
    table, spec = GOLD / "optics" / "t1_table.dat", GOLD / "optics" / "s1_spec.dat"
    r = subprocess.run([str(exe), str(param), "--table", str(table), "--spec", str(spec), "--dry-run"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    p = formats.read_param_struct(param)
    t = formats.read_optical(table)
    formats.param_grid(p, t["dmin"], t["dmax"])
    run = formats.setup_count(p, t["dmin"], t["dmax"])
    want = (f"system: {p.n_planets + run.n_mass} massive ({p.n_planets} star and planets), {run.n_dust} grain "
            f"tracers, {p.n_grid} size bins, {t['w'].size} wavelengths")
    assert r.stdout.strip() == want


def test_driver_rejects_bad_arguments_and_files(tmp_path):
    exe = build.build_driver()
    r = subprocess.run([str(exe), "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    bad = tmp_path / "bad.param"
    bad.write_text("# nothing else\n")
    r = subprocess.run([str(exe), str(bad), "--table", "x", "--spec", "y", "--dry-run"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode != 0 and "rejected" in r.stderr


def test_driver_dry_run_reads_the_reference_systems():
    """The reference's own test systems (tests/*.param of its checkout), each read by the
    program with a synthetic Mie table and spectrum in the reference's formats: the counts
    it prints are those of the same files read through the Python API."""
    from oracle.ref import paths
    paths.require(paths.TESTS, "the reference's test systems")
    exe = build.build_driver()
    table, spec = GOLD / "optics" / "t1_table.dat", GOLD / "optics" / "s1_spec.dat"
    t = formats.read_optical(table)
    systems = sorted(paths.TESTS.glob("*.param"))
    assert len(systems) >= 13
    for param in systems:
        r = subprocess.run([str(exe), str(param), "--table", str(table), "--spec", str(spec), "--dry-run"],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, (param.name, r.stderr)
        p = formats.read_param_struct(param)
        formats.param_grid(p, t["dmin"], t["dmax"])
        run = formats.setup_count(p, t["dmin"], t["dmax"])
        want = (f"system: {p.n_planets + run.n_mass} massive ({p.n_planets} star and planets), {run.n_dust} "
                f"grain tracers, {p.n_grid} size bins, {t['w'].size} wavelengths")
        assert r.stdout.strip() == want, param.name
