"""ORACLE -- test infrastructure.  ctypes binding of the reference-kernel runner
(oracle/ref/ref_runner.cpp) that executes the reference's own CUDA kernels, compiled
unmodified for sm_103a into oracle/_ref/ddyn_ref_sm103a.cubin."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .cpu import OPhys, OView, phys as _phys, view as _view
from .ref.build_ref import CUBIN, build as _build

_lib = None


def available() -> bool:
    return CUBIN.exists()


def lib():
    global _lib
    if _lib is None:
        out = _build()
        if out["cubin"] is None or out["runner"] is None:
            raise RuntimeError("reference kernels unavailable (cubin not built)")
        _lib = C.CDLL(str(out["runner"]))
        _lib.ref_error.restype = C.c_char_p
        _lib.ref_load.argtypes = [C.c_char_p]
        if _lib.ref_load(str(out["cubin"]).encode()) != 0:
            raise RuntimeError("ref_load: " + _lib.ref_error().decode())
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(r, what):
    if r != 0:
        raise RuntimeError(f"{what}: {lib().ref_error().decode()}")


def step(arrays: dict, n_grav: int, dt: float, size_table: dict, phys_d: dict, n_steps: int = 1,
         return_kpos: bool = False, return_ms: bool = False):
    L = lib()
    st = {f: np.array(arrays[f], dtype=np.int32 if f == "id" else np.float64, copy=True)
          for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")}
    n_dust = len(st["x"]) - n_grav
    size = np.ascontiguousarray(size_table["size"], np.float64)
    b = np.ascontiguousarray(size_table["beta"], np.float32)
    bs = np.ascontiguousarray(size_table["betasw"], np.float32)
    q = np.ascontiguousarray(size_table["q"], np.float32)
    kpos = np.zeros((4, 3, n_grav))
    ms = C.c_double(0.0)
    ph = _phys(phys_d)
    r = L.ref_step(C.c_int(n_grav), C.c_int(n_dust), *[_p(st[f]) for f in ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")],
                   C.c_int(len(size)), _p(size), _p(b), _p(bs), _p(q), C.c_double(dt), C.c_int(n_steps),
                   C.byref(ph), _p(kpos), C.byref(ms))
    _check(r, "ref_step")
    out = [st]
    if return_kpos:
        out.append(kpos)
    if return_ms:
        out.append(ms.value)
    return out[0] if len(out) == 1 else tuple(out)


def _opt(o, size):
    keep = {k: np.ascontiguousarray(o[k], np.float64) for k in ("w", "in", "Qabs", "Qsca", "Qpfunc", "Td")}
    keep["size"] = np.ascontiguousarray(size, np.float64)
    return keep


def image(arrays: dict, n_grav: int, optics: dict, size, view_d: dict, wj):
    L = lib()
    st = {f: np.array(arrays[f], dtype=np.int32 if f == "id" else np.float64, copy=True)
          for f in ("x", "y", "z", "N", "id")}
    n_dust = len(st["x"]) - n_grav
    k = _opt(optics, size)
    v = _view(view_d)
    wj_a = np.ascontiguousarray(wj, np.int32)
    Fd = np.zeros((len(wj_a), v.xsize, v.ysize))
    n_grid, n_wav = k["Qabs"].shape
    r = L.ref_image(C.c_int(n_grav), C.c_int(n_dust), _p(st["x"]), _p(st["y"]), _p(st["z"]), _p(st["N"]),
                    _p(st["id"]), C.c_int(n_grid), C.c_int(n_wav), C.c_int(k["Qpfunc"].shape[1]),
                    _p(k["size"]), _p(k["w"]), _p(k["in"]), _p(k["Qabs"]), _p(k["Qsca"]), _p(k["Qpfunc"]),
                    _p(k["Td"]), C.c_double(optics["Rmin"]), C.c_double(optics["Rmax"]), C.byref(v),
                    _p(wj_a), C.c_int(len(wj_a)), _p(Fd))
    _check(r, "ref_image")
    return Fd


def sed(arrays: dict, n_grav: int, optics: dict, size, view_d: dict, return_ms: bool = False):
    L = lib()
    st = {f: np.array(arrays[f], dtype=np.int32 if f == "id" else np.float64, copy=True)
          for f in ("x", "y", "z", "N", "id")}
    n_dust = len(st["x"]) - n_grav
    k = _opt(optics, size)
    v = _view(view_d)
    n_grid, n_wav = k["Qabs"].shape
    out = np.zeros(n_wav)
    ms = C.c_double(0.0)
    r = L.ref_sed(C.c_int(n_grav), C.c_int(n_dust), _p(st["x"]), _p(st["y"]), _p(st["z"]), _p(st["N"]),
                  _p(st["id"]), C.c_int(n_grid), C.c_int(n_wav), C.c_int(k["Qpfunc"].shape[1]),
                  _p(k["size"]), _p(k["w"]), _p(k["in"]), _p(k["Qabs"]), _p(k["Qsca"]), _p(k["Qpfunc"]),
                  _p(k["Td"]), C.c_double(optics["Rmin"]), C.c_double(optics["Rmax"]), C.byref(v),
                  _p(out), C.byref(ms))
    _check(r, "ref_sed")
    return (out, ms.value) if return_ms else out
