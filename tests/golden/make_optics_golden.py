"""Generates tests/golden/optics/: synthetic Mie table files and stellar spectrum files in
the reference's formats (written here: the table layout of its table generator,
tools/runmie.c:196-213, and the two-column spectrum of its Kurucz files), and, for each
case, what the reference's own set-up makes of them: add_optical_data, add_specfile,
interpolate_dust_to_grid, interpolate_stellar_to_grid and calculate_beta, run by
oracle/_ref/optics_dump (built from the reference sources by oracle/ref/build_param_ref.py).
Needs the reference sources:

    python tests/golden/make_optics_golden.py
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent / "optics"

AU, RSUN, PC, GRAV = 1.49598e11, 695700000.0, 3.08567758149137e16, 4.0 * np.pi * np.pi


def table_text(n_dust, n_wav, n_theta, amin_um, amax_um, lmin_um, lmax_um, seed):
    """A Mie-like table: Q_abs and Q_sca smooth in the size parameter x = 2 pi s / lambda,
    a Henyey-Greenstein phase function with g rising with x; every value positive."""
    assert (n_theta * n_wav) % 10 == 0
    g = np.random.default_rng(seed)
    lam = np.exp(np.linspace(np.log(lmin_um), np.log(lmax_um), n_wav))
    mu = np.arange(n_theta) * 2.0 / (n_theta - 1) - 1.0
    out = ["#\tn_lnk\tnthetas\tndust\tamin\t\tamax\n", "#\t%d\t%d\t%d\t%.6e\t%.6e\n" % (n_wav, n_theta, n_dust, amin_um,
                                                                                      amax_um)]
    for z in range(n_dust):
        s = amin_um * np.exp(np.log(amax_um / amin_um) * z / (n_dust - 1.0))
        x = 2 * np.pi * s / lam
        qa = 1.1 * x / (1.0 + x) * (1.0 + 0.05 * g.standard_normal(n_wav) ** 2) + 1e-4
        qs = 2.0 * x ** 4 / (1.0 + x ** 4) + 1e-7
        gg = 0.8 * x / (1.0 + x)
        pf = qs[None, :] * (1 - gg ** 2)[None, :] / (1 + gg ** 2 - 2 * gg[None, :] * mu[:, None]) ** 1.5   # [theta][wav]
        out.append("#s %.6e\n" % s)
        out += ["%.6e %.6e %.6e\n" % (lam[i], qa[i], qs[i]) for i in range(n_wav)]
        flat = pf.reshape(-1)
        out += ["".join("%.6e " % v for v in flat[r * 10:(r + 1) * 10]) + "\n" for r in range(flat.size // 10)]
    return "".join(out)


def spec_text(n, wmin_m, wmax_m, T, zeros_head=0, zero_at=(), comment=True):
    """A blackbody spectrum, wavelength [m] and surface flux pi B_lambda [W m^-3], with
    optional zero fluxes."""
    w = np.exp(np.linspace(np.log(wmin_m), np.log(wmax_m), n))
    h, c, k = 6.626068e-34, 299792458.0, 1.3806503e-23
    F = np.pi * 2 * h * c * c / (w ** 5 * (np.exp(h * c / (w * k * T)) - 1.0))
    F[:zeros_head] = 0.0
    for k in zero_at:
        F[k] = 0.0
    lines = ["# synthetic spectrum\n"] if comment else []
    lines += ["%.5e %.5e\n" % (w[k], F[k]) for k in range(n)]
    return "".join(lines)


TABLES = {
    "t1": dict(n_dust=8, n_wav=30, n_theta=11, amin_um=0.1, amax_um=100.0, lmin_um=0.1, lmax_um=1000.0, seed=11),
    "t2": dict(n_dust=5, n_wav=20, n_theta=5, amin_um=0.5, amax_um=50.0, lmin_um=0.2, lmax_um=500.0, seed=12),
}
SPECS = {
    "s1": dict(n=150, wmin_m=9e-8, wmax_m=1.6e-4, T=8200.0, zeros_head=6),
    "s2": dict(n=60, wmin_m=3e-7, wmax_m=1.0e-4, T=5400.0, zero_at=(17,)),
}


def dmax_of(t):
    return float("%.6e" % TABLES[t]["amax_um"]) * 1e-6


def s_of(t, z):
    p = TABLES[t]
    return float("%.6e" % (p["amin_um"] * np.exp(np.log(p["amax_um"] / p["amin_um"]) * z / (p["n_dust"] - 1.0)))) * 1e-6


def w_of(t, i):
    p = TABLES[t]
    lam = np.exp(np.linspace(np.log(p["lmin_um"]), np.log(p["lmax_um"]), p["n_wav"]))
    return float("%.6e" % lam[i]) * 1e-6


COMMON = dict(kqe=1.7e-2, rho=2700.0, dist=10 * PC, rstar=1.8 * RSUN / AU, mstar=1.9 * GRAV, mloss=2.0e-14, vsw=4.0e5)
CASES = {
    # the usual set-up: amin above the first table size, amax the table's largest size
    # (the last bin is snapped onto it when it overshoots by rounding), both forces
    "typical": dict(table="t1", spec="s1", n_grid=20, radQ=1, SWQ=1, amin=1.2e-7, amax=dmax_of("t1"),
                    wavs=(1.6e-6, 24e-6, 70e-6), **COMMON),
    # a spectrum narrower than the table on both sides and with a zero inside; image
    # wavelengths at the table's ends (the first gives index -1, as in the reference)
    "narrow_spectrum": dict(table="t2", spec="s2", n_grid=7, radQ=1, SWQ=0, amin=0.8e-6, amax=30e-6,
                            wavs=(w_of("t2", 0), w_of("t2", 19), 10e-6), **COMMON),
    # many bins per table interval, the first bin on a table size, no radiation pressure
    "many_bins": dict(table="t1", spec="s1", n_grid=40, radQ=0, SWQ=1, amin=s_of("t1", 1), amax=s_of("t1", 6),
                      wavs=(0.55e-6,), **COMMON),
}


def read_dump(raw: bytes, n_grid: int, nwavs: int) -> dict:
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=n, offset=off).copy()
        off += a.nbytes
        return a

    nd, nw, nt, ns = (int(v) for v in take("<i4", 4))
    d = {"dmin": take("<f8", 1)[0], "dmax": take("<f8", 1)[0]}
    d["file_s"] = take("<f8", nd)
    d["w"] = take("<f8", nw)
    d["file_Qabs"] = take("<f8", nd * nw).reshape(nd, nw)
    d["file_Qsca"] = take("<f8", nd * nw).reshape(nd, nw)
    d["file_Qpfunc"] = take("<f8", nd * nt * nw).reshape(nd, nt, nw)
    d["spec_w"] = take("<f8", ns)
    d["spec_F"] = take("<f8", ns)
    d["in"] = take("<f8", nw)
    d["wj"] = take("<i4", nwavs)
    d["s"] = take("<f8", n_grid)
    d["q"] = take("<f4", n_grid)
    d["Qabs"] = take("<f8", n_grid * nw).reshape(n_grid, nw)
    d["Qsca"] = take("<f8", n_grid * nw).reshape(n_grid, nw)
    d["Qpfunc"] = take("<f8", n_grid * nt * nw).reshape(n_grid, nt, nw)
    d["beta"] = take("<f4", n_grid)
    d["betasw"] = take("<f4", n_grid)
    d["Lum"] = take("<f8", 1)[0]
    d["betaswconst"] = take("<f8", 1)[0]
    assert off == len(raw)
    return d


def run_reference(exe, table: Path, spec: Path, c: dict, out: Path) -> dict:
    args = [str(exe), str(table), str(spec), str(out), str(c["n_grid"]), str(c["radQ"]), str(c["SWQ"])]
    args += [float(c[k]).hex() for k in ("amin", "amax", "kqe", "rho", "dist", "rstar", "mstar", "mloss", "vsw")]
    args += [float(v).hex() for v in c["wavs"]]
    subprocess.run(args, check=True, capture_output=True)
    return read_dump(out.read_bytes(), c["n_grid"], len(c["wavs"]))


def main():
    from oracle.ref import build_param_ref
    exe = build_param_ref.build_optics()
    if exe is None:
        raise SystemExit("the reference sources are needed")
    OUT.mkdir(exist_ok=True)
    for name, p in TABLES.items():
        (OUT / f"{name}_table.dat").write_text(table_text(**p))
    for name, p in SPECS.items():
        (OUT / f"{name}_spec.dat").write_text(spec_text(**p))
    for name, c in CASES.items():
        d = run_reference(exe, OUT / f"{c['table']}_table.dat", OUT / f"{c['spec']}_spec.dat", c,
                          OUT / f"{name}.bin")
        (OUT / f"{name}.bin").unlink()
        params = {k: np.asarray(v) for k, v in c.items() if k not in ("table", "spec")}
        np.savez_compressed(OUT / f"{name}.npz", table=c["table"], spec=c["spec"], **params, **d)
        print(name, "beta", d["beta"][:3], "wj", d["wj"], "Lum", d["Lum"])


if __name__ == "__main__":
    main()
