"""ORACLE -- test infrastructure.  Recipe for oracle/_ref/param_dump: the reference's own
parameter-file parser (src/read_in.cu with the helpers it calls: src/functions.cu,
src/ran3.cu, src/error.cu, src/print.cu, src/getMemorySize.cu), compiled unmodified where
the sources lie, linked with oracle/ref/param_dump.cu.  Host code only (the reference
declares its constant-memory tables in the shared header, so the objects are built with
relocatable device code).  Needs the reference sources: available only where they are.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
from .paths import SRC as REFSRC
EXE = OUT / "param_dump"
OPTICS_EXE = OUT / "optics_dump"
UNITS = ("read_in", "functions", "ran3", "error", "print", "getMemorySize")


def _build(harness: str, exe: Path) -> Path | None:
    if not (REFSRC / "read_in.cu").exists():
        return exe if exe.exists() else None
    OUT.mkdir(exist_ok=True)
    deps = [REFSRC / f"{u}.cu" for u in UNITS] + [REFSRC / "ddyn.cuh", HERE / harness]
    if exe.exists() and exe.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return exe
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    flags = ["-O2", "-rdc=true", "-D_GNU_SOURCE", "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(REFSRC)]
    objs = []
    for u in UNITS:
        o = OUT / f"ref_{u}.o"
        if not (o.exists() and o.stat().st_mtime >= (REFSRC / f"{u}.cu").stat().st_mtime):
            r = subprocess.run([nvcc, *flags, "-c", str(REFSRC / f"{u}.cu"), "-o", str(o)], capture_output=True,
                               text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference {u}.cu failed to build:\n{r.stderr}")
        objs.append(str(o))
    r = subprocess.run([nvcc, *flags, str(HERE / harness), *objs, "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{harness} failed to link:\n{r.stderr}")
    return exe


def build() -> Path | None:
    """oracle/_ref/param_dump: read_in_param and read_in_model."""
    return _build("param_dump.cu", EXE)


def build_optics() -> Path | None:
    """oracle/_ref/optics_dump: interpolate_stellar_to_grid, interpolate_dust_to_grid,
    calculate_beta."""
    return _build("optics_dump.cu", OPTICS_EXE)


def build_setup() -> Path | None:
    """oracle/_ref/setup_dump: the start-of-run set-up and Grid::setup's body generation."""
    return _build("setup_dump.cu", OUT / "setup_dump")


if __name__ == "__main__":
    print(build())
