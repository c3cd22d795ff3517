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
REFSRC = Path("/root/reference/src")
EXE = OUT / "param_dump"
UNITS = ("read_in", "functions", "ran3", "error", "print", "getMemorySize")


def build() -> Path | None:
    if not (REFSRC / "read_in.cu").exists():
        return EXE if EXE.exists() else None
    OUT.mkdir(exist_ok=True)
    deps = [REFSRC / f"{u}.cu" for u in UNITS] + [REFSRC / "ddyn.cuh", HERE / "param_dump.cu"]
    if EXE.exists() and EXE.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return EXE
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    flags = ["-O2", "-rdc=true", "-D_GNU_SOURCE", "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(REFSRC)]
    objs = []
    for u in UNITS:
        o = OUT / f"ref_{u}.o"
        r = subprocess.run([nvcc, *flags, "-c", str(REFSRC / f"{u}.cu"), "-o", str(o)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference {u}.cu failed to build:\n{r.stderr}")
        objs.append(str(o))
    r = subprocess.run([nvcc, *flags, str(HERE / "param_dump.cu"), *objs, "-o", str(EXE)], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"param_dump failed to link:\n{r.stderr}")
    return EXE


if __name__ == "__main__":
    print(build())
