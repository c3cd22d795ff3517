"""Generates tests/golden/params/: synthetic DiskDyn parameter files (written here, in the
reference's format) and, for each, what the reference's own parser makes of it
(oracle/_ref/param_dump, built from the reference sources by oracle/ref/build_param_ref.py;
doubles as hexadecimal strings).  For a file the reference rejects, the usage code of
its exit message (src/error.cu).  Needs the reference sources:

    python tests/golden/make_param_golden.py
"""
from __future__ import annotations

import json
import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent / "params"

HEADER = "# synthetic parameter file for the parser tests\n"


def param(star="1.0 G2V 5777 1.0 1.0 25.0 2.0e-14 400.0", geometry="10.0 120.0 15.0 60.0 30.0 256 200",
          waves="0.55 1.6 24.0 70.0", spec="Library", physics="yes yes no", planets=(), comp="2.7 optical/astrosil.dat 27.5",
          disks=(), blobs=(), stub="synthetic", graphics="no 100", out="1000.0 100.0 500.0", tend="2000",
          nstep="300", verbose="1", gpu="0", extra=""):
    lines = [HEADER, "# Verbose level\n", verbose + "\n\n", "# GPU\n", gpu + "\n", graphics + "\n", out + "\n",
             tend + "\n", nstep + "\n", star + "\n", geometry + "\n", waves + "\n", spec + "\n", physics + "\n",
             "begin_planets\n"] + [p + "\n" for p in planets] + ["end_planets\n", comp + "\n", "begin_disks\n"]
    lines += [d + "\n" for d in disks] + ["end_disks\n", "begin_blobs\n"] + [b + "\n" for b in blobs]
    lines += ["end_blobs\n", "# stub\n", stub + "\n", extra]
    return "".join(lines)


CASES = {
    "minimal": param(),
    "planets_disks_blobs": param(
        planets=("2.0 5.2 0.048 20.0 100.5 273.9 9.5e-4", "1.3 9.5 0.056 317.0 113.7 339.4 2.85e-4",
                 "0.0 1.0 0.0 0.0 0.0 0.0 3.0e-6"),
        disks=("38.0 43.0 0.05 0.2 10.0 1.0 3.65 2.0 0.0 0 500000",
               "80.0 120.0 0.1 0.05 100.0 2.5 3.5 0.5 -1.5 128 2000000"),
        blobs=("10.0 0.6 3.0 45.0 30.0 90.0 10.0 0.01 3.65 0.1 0 1000000 cloud 0.1",
               "25.0 0.1 1.0 0.0 10.0 200.0 5.0 0.5 3.5 0.01 16 50000 Collision 5.0")),
    "switch_spellings_and_quotes": param(
        graphics="YES 50", physics="Y FALSE TRUE", spec='"my spectra/star.dat"',
        comp='3.3 "optical/with space.dat" 12.0', star="1.92 A0V 9600 1.8 3.0 0.5 1.0e-13 600",
        planets=("5.0 30.0 0.2 45.0 60.0 90.0 1.0e-3",), stub='"quoted stub"'),
    "at_sign_separator": param(geometry="7.7@140.0@0.0@90.0@0.0@128@128", waves="3.0 3.35 4.44"),
    "kurucz_rounding_hot": param(star="2.4 B9V 12345 2.1 1.0 1.0 1.0e-12 800"),
    "kurucz_rounding_cool": param(star="0.31 M1 3600 0.82 1.0 30.0 6.0e-12 450.0"),
    "many_wavelengths": param(waves=" ".join(f"{w:.2f}" for w in (0.4, 0.5, 0.6, 0.8, 1.0, 1.25, 1.6, 2.2, 3.5,
                                                                    4.5, 8.0, 12.0, 24.0, 70.0, 100.0, 160.0))),
    "trailing_lines": param(extra="# after the stub\nextra tokens that are ignored\n"),
    "reject_star_tokens": param(star="1.0 G2V 5777 1.0 1.0 25.0"),
    "reject_blob_kind": param(blobs=("10.0 0.6 3.0 0.0 0.0 0.0 10.0 0.01 3.65 0.1 0 1000 puff 0.1",)),
    "reject_end_time": param(tend="0"),
    "reject_graphics": param(graphics="maybe 10"),
    "reject_library_teff": param(star="1.0 X 60000 1.0 1.0 25.0 2.0e-14 400.0"),
    "reject_truncated": HEADER + "1\n0\nno 100\n1000 100 100\n100\n",
}


def usage_messages() -> list[str]:
    """errmsg[] of the reference (src/error.cu), to name the code of an exit message."""
    from oracle.ref.paths import SRC
    txt = (SRC / "error.cu").read_text()
    body = txt[txt.index("errmsg"):]
    body = body[body.index("{") + 1: body.index("};")]
    return [m.replace("\\n", "").strip() for m in re.findall(r'"((?:[^"\\]|\\.)*)"', body)]


def main() -> None:
    import oracle.ref.build_param_ref as bp
    exe = bp.build()
    if exe is None:
        raise SystemExit("the reference sources are needed to build oracle/_ref/param_dump")
    msgs = usage_messages()
    OUT.mkdir(exist_ok=True)
    for name, text in CASES.items():
        pf = OUT / f"{name}.param"
        pf.write_text(text)
        r = subprocess.run([str(exe), str(pf)], capture_output=True, text=True)
        if r.returncode == 0:
            out = json.loads(r.stdout)
        else:
            m = re.search(r"Error:\t(.*)\n", r.stderr)
            msg = m.group(1).strip() if m else ""
            out = {"rejected": True, "message": msg, "usage_code": msgs.index(msg) if msg in msgs else None}
        (OUT / f"{name}.json").write_text(json.dumps(out, indent=1) + "\n")
        print(name, "rejected" if r.returncode else "ok")


if __name__ == "__main__":
    main()
