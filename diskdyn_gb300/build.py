"""Build libddx.so (the sm_103a kernels and the C ABI) in-tree with nvcc.

Each translation unit of csrc/ is compiled in parallel for sm_103a only, then linked into
diskdyn_gb300/libddx.so.  A unit is recompiled only when it, or a header, is newer than
its object file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libddx.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code without FP contraction, so host-side arithmetic (ddx_det_step) rounds the same
# on x86-64 and on Arm, like the reference's host code built for x86-64.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-diag-suppress", "1444", "-I", str(ROOT / "include")]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libddx.so")
    return cand


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


# Host-only sources (file formats): plain C++, no contraction, like the reference's host code.
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(ROOT / "include")]


def _compile(src: Path, hmt: float, verbose: bool) -> Path:
    obj = OBJ / (src.name + ".o")     # x.cu and x.cpp may share a stem
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hmt):
        return obj
    if src.suffix == ".cpp":
        cmd = [shutil.which("g++") or "g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hmt = _headers_mtime()
    # objects built with other flags are stale
    stamp = OBJ / "flags.txt"
    flags = " ".join(ARCH + NVCC_FLAGS + CXX_FLAGS)
    if not stamp.exists() or stamp.read_text() != flags:
        for o in OBJ.glob("*.o"):
            o.unlink()
        stamp.write_text(flags)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hmt, verbose), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libddx.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


DRIVER_SRC = PKG / "driver" / "ddyn_gb300.cpp"
DRIVER = PKG / "ddyn_gb300"


def build_driver(verbose: bool = False) -> Path:
    """The ddyn_gb300 program (a whole run from a parameter file through the C ABI), linked
    against libddx.so next to it."""
    lib = build(verbose)
    hs = [DRIVER_SRC] + list((ROOT / "include").glob("*.h"))
    if DRIVER.exists() and DRIVER.stat().st_mtime >= max(lib.stat().st_mtime, *(h.stat().st_mtime for h in hs)):
        return DRIVER
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include"),
           str(DRIVER_SRC), "-o", str(tmp), "-L", str(PKG), "-lddx", "-lcudart", "-Xlinker", "-rpath=$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build of ddyn_gb300 failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose=True))
    print(build_driver(verbose=True))
