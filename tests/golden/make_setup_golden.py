"""Generates tests/golden/setup/: synthetic parameter files (in the reference's format) and,
for each, the initial system the reference's own start-of-run set-up builds from it with the
Mie table and spectrum of tests/golden/optics/: the optical size limits and disk and blob
constants (detminmax, confCdisks, confCblobs), the beta table, and every body of
Grid::setup's generation with ran3 seeded at -2 (oracle/_ref/setup_dump, built from the
reference sources by oracle/ref/build_param_ref.py).  Needs the reference sources:

    python tests/golden/make_setup_golden.py
"""
from __future__ import annotations

import importlib.util
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
OUT = HERE / "setup"
OPTICS = HERE / "optics"

_spec = importlib.util.spec_from_file_location("mpg", HERE / "make_param_golden.py")
mpg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mpg)

# disk: Rin Rout dh/dr sigma_e amax[km] amin[um] eta_a Mtot[MEarth] gamma Ngrav Nsmall
# blob: a ecc inc w o nu amax[km] amin[um] eta_a Mtot Ngrav Nsmall cloud|collision sigma|vkepp
CASES = {
    # both disk and blob kinds, the three grain-number branches (eta 0, 1, other), a disk
    # reaching below the table's smallest size and one above its largest
    "disks_blobs": dict(
        planets=("3.0 12.0 0.1 5.0 80.0 200.0 1.0e-3",),
        disks=("38.0 43.0 0.05 0.2 10.0 1.0 3.65 2.0 0.0 20 400",
               "80.0 120.0 0.1 0.05 0.05 0.15 1.0 0.5 -1.5 10 300"),
        blobs=("30.0 0.3 5.0 45.0 30.0 90.0 1.0 2.0 3.65 0.1 5 200 cloud 2.0",
               "50.0 0.1 10.0 0.0 10.0 200.0 5.0 0.5 -2.0 0.01 3 150 Collision 5.0")),
    # draws the generators reject and repeat: eccentricities beyond 1 and blob radii below 0;
    # eta = 2 (the logarithmic constant branch)
    "rejections": dict(
        disks=("5.0 60.0 0.3 0.8 1.0 0.3 4.0 0.2 1.0 12 250",),
        blobs=("3.0 0.0 0.0 0.0 0.0 0.0 2.0 0.5 3.65 0.05 4 160 cloud 2.5",)),
}


def read_dump(raw: bytes) -> dict:
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=n, offset=off).copy()
        off += a.nbytes
        return a

    n_all, n_mass, n_dust, n_grid, n_disks, n_blobs = (int(v) for v in take("<i4", 6))
    d = {"n_all": n_all, "n_mass": n_mass, "n_dust": n_dust, "n_grid": n_grid}
    for k, v in zip(("amin", "amax", "mmin", "mmax", "f", "dmin", "dmax"), take("<f8", 7)):
        d[k] = v
    d["disks"] = take("<f8", 5 * n_disks).reshape(n_disks, 5)      # amin mmin dmax dmmax C
    d["blobs"] = take("<f8", 5 * n_blobs).reshape(n_blobs, 5)
    d["beta"] = take("<f4", n_grid)
    for k in ("x", "y", "z", "vx", "vy", "vz", "N", "m"):
        d[k] = take("<f8", n_all)
    d["id"] = take("<i4", n_all)
    assert off == len(raw)
    return d


def run_reference(exe, param: Path, out: Path) -> dict:
    subprocess.run([str(exe), str(param), str(OPTICS / "t1_table.dat"), str(OPTICS / "s1_spec.dat"), str(out)],
                   check=True, capture_output=True)
    return read_dump(out.read_bytes())


def main():
    from oracle.ref import build_param_ref
    exe = build_param_ref.build_setup()
    if exe is None:
        raise SystemExit("the reference sources are needed")
    OUT.mkdir(exist_ok=True)
    for name, kw in CASES.items():
        pf = OUT / f"{name}.param"
        pf.write_text(mpg.param(**kw))
        d = run_reference(exe, pf, OUT / f"{name}.bin")
        (OUT / f"{name}.bin").unlink()
        np.savez_compressed(OUT / f"{name}.npz", **d)
        print(name, "bodies", d["n_all"], "massive", d["n_mass"], "grains", d["n_dust"], "bins", d["n_grid"])


if __name__ == "__main__":
    main()
