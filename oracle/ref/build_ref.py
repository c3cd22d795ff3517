"""ORACLE -- test infrastructure.  Recipe for the reference-kernel oracle.

1. Where the reference sources are present (the development container), compile its
   kernels unmodified into oracle/_ref/ddyn_ref_sm103a.cubin (device code only, so the
   same file runs under the Arm host of the GPU machine).
2. On any machine with nvcc/g++, build oracle/_ref/libref_runner.so, the host runner
   that loads that cubin through the CUDA driver API and replays the reference's launch
   sequence (oracle/ref/ref_runner.cpp).

Outputs go to oracle/_ref/ only.  The runner is skipped if the cubin is absent.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
from .paths import SRC as REFSRC
CUBIN = OUT / "ddyn_ref_sm103a.cubin"
RUNNER = OUT / "libref_runner.so"


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_cubin() -> Path | None:
    if not (REFSRC / "gpu_functions.cu").exists():
        return CUBIN if CUBIN.exists() else None
    OUT.mkdir(exist_ok=True)
    src = HERE / "ref_kernels.cu"
    newest = max(src.stat().st_mtime, (REFSRC / "gpu_functions.cu").stat().st_mtime,
                 (REFSRC / "ddyn.cuh").stat().st_mtime)
    if CUBIN.exists() and CUBIN.stat().st_mtime >= newest:
        return CUBIN
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-cubin", "-O3",
           "-I", str(REFSRC), "-o", str(CUBIN), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference cubin build failed:\n{r.stderr}")
    return CUBIN


def build_runner() -> Path | None:
    OUT.mkdir(exist_ok=True)
    src = HERE / "ref_runner.cpp"
    if RUNNER.exists() and RUNNER.stat().st_mtime >= src.stat().st_mtime:
        return RUNNER
    cuda = Path(_nvcc()).resolve().parent.parent
    stubs = [p for p in (cuda / "lib64" / "stubs", cuda / "targets" / "sbsa-linux" / "lib" / "stubs",
                         cuda / "targets" / "x86_64-linux" / "lib" / "stubs") if p.exists()]
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(cuda / "include"),
           str(src), "-o", str(RUNNER)]
    for s in stubs:
        cmd += ["-L", str(s)]
    cmd += ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference runner build failed:\n{r.stderr}")
    return RUNNER


def build() -> dict:
    cub = build_cubin()
    run = build_runner()
    return {"cubin": cub, "runner": run}


if __name__ == "__main__":
    print(build())
