"""Generates the golden fixtures of this directory from the reference's own kernels.

The reference ships no tests or golden vectors.  This script runs its unmodified kernels
(src/gpu_functions.cu, compiled for sm_103a into oracle/_ref/ and replayed through
oracle/ref/ref_runner.cpp with the reference host code's launch sequences) on small seeded
inputs and stores inputs and outputs together, so the CPU test suite can check the oracle
against the reference without a GPU (tests/test_golden_cpu.py).  Needs a GPU and the
built reference runner:

    python -c "import __graft_entry__ as g; g.build()"
    python tests/golden/make_golden.py [out_dir]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle.refk as refk  # noqa: E402
from diskdyn_gb300 import synth  # noqa: E402

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")
OUT_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N")


def pack(prefix: str, d: dict) -> dict:
    return {f"{prefix}{k}": np.asarray(v) for k, v in d.items()}


def step_case(name: str, s: synth.System, n_steps: int, out: Path) -> None:
    r = refk.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, n_steps)
    phys = {k: np.float64(v) for k, v in s.phys.items()}
    np.savez_compressed(out / f"{name}.npz", n_grav=s.n_grav, dt=s.dt, n_steps=n_steps,
                        **pack("in_", {k: s.state[k] for k in FIELDS}),
                        **pack("tab_", s.size_table), **pack("phys_", phys),
                        **pack("out_", {k: r[k] for k in OUT_FIELDS}))


def flux_case(out: Path) -> None:
    s = synth.solar_like(n_dust=2048, seed=synth.SEED + 3, with_ids=True, n_bins=8)
    s.state["N"][s.n_grav:] = 1e15
    opt = synth.hg_optics(n_grid=8, n_theta=31, n_wav=20)
    view = dict(dist=10 * synth.PC, fov=100.0, PA=0.3, inc=np.deg2rad(35.0), longitude=0.7, xsize=64, ysize=48)
    wj = [0, 7, 15]
    img = refk.image(s.state, s.n_grav, opt, opt["size"], view, wj)
    sed = refk.sed(s.state, s.n_grav, opt, opt["size"], view)
    np.savez_compressed(out / "flux_small.npz", n_grav=s.n_grav, wj=np.array(wj),
                        **pack("in_", {k: s.state[k] for k in FIELDS}),
                        **pack("opt_", {k: opt[k] for k in ("w", "in", "Qabs", "Qsca", "Qpfunc", "Td", "Rmin",
                                                           "Rmax", "size")}),
                        **pack("view_", {k: np.float64(v) for k, v in view.items()}),
                        out_image=img, out_sed=sed)


def main() -> None:
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent
    out.mkdir(parents=True, exist_ok=True)
    if not refk.available():
        raise SystemExit("the reference runner is not built (run __graft_entry__.build() on a GPU machine)")
    # dusty ring: star, two planets, 16 planetesimals, 512 grains with radiation pressure,
    # PR and stellar-wind drag; 5 steps
    step_case("step_ring", synth.dusty_ring(n_dust=512, n_plsml=16, seed=5, n_steps=5), 5, out)
    # star only with the Lorentz force on (no massive stage runs: src/grid.cu:698)
    s = synth.dusty_ring(n_dust=256, n_plsml=0, seed=6, n_steps=3)
    st = {k: np.concatenate([v[:1], v[s.n_grav:]]) for k, v in s.state.items()}
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        st[k][0] = 0.0
    tab = dict(s.size_table, q=np.linspace(1e-3, 2e-3, len(s.size_table["q"])).astype(np.float32))
    step_case("step_star_lorentz",
              synth.System("star_only", 1, st, s.dt, 3, dict(s.phys, FLQ=1, Bstar=5e-20, Wz=14.6, n_planets=1), tab),
              3, out)
    # solar-like: 8 planets, 256 massless tracers, 3 steps of 0.05 yr
    step_case("step_solar", synth.solar_like(n_dust=256, seed=synth.SEED + 1), 3, out)
    flux_case(out)
    for p in sorted(out.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
