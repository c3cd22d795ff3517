"""Python view of the reference-format file functions of libddx.so
(include/diskdyn_gb300_io.h): the parameter-file parser."""
from __future__ import annotations

import ctypes as C

from . import abi

MAX_PLANETS, MAX_DISKS, MAX_BLOBS, MAX_WAVS, STR = 64, 32, 32, 16, 512


class Planet(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("x", "y", "z", "vx", "vy", "vz", "m")]


DISK_F = ("Rin", "Rout", "dhdr", "sigmae", "amax", "mmax", "amin", "mmin", "dmax", "dmmax", "eta", "gammas", "C",
          "Mtot")
BLOB_F = ("a", "ecc", "inc", "w", "o", "nu", "sigma", "amax", "mmax", "amin", "mmin", "dmax", "dmmax", "eta", "C",
          "Mtot", "vkepp")


class Disk(C.Structure):
    _fields_ = [(k, C.c_double) for k in DISK_F] + [("Ngrav", C.c_longlong), ("Nsmall", C.c_longlong)]


class Blob(C.Structure):
    _fields_ = ([(k, C.c_double) for k in BLOB_F] +
                [("Ngrav", C.c_longlong), ("Nsmall", C.c_longlong), ("collcloud", C.c_int)])


class Param(C.Structure):
    _fields_ = [("verb", C.c_int), ("gpuid", C.c_int), ("gl", C.c_int),
                ("t_gl", C.c_double), ("t_write", C.c_double), ("t_fits", C.c_double), ("t_sed", C.c_double),
                ("t_end", C.c_double), ("n_step", C.c_int), ("sptype", C.c_char * STR),
                ("teff", C.c_double), ("rstar", C.c_double), ("Bstar", C.c_double), ("Wz", C.c_double),
                ("mloss", C.c_double), ("vsw", C.c_double),
                ("dist", C.c_double), ("fov", C.c_double), ("PA", C.c_double), ("inc", C.c_double),
                ("longitude", C.c_double), ("xsize", C.c_int), ("ysize", C.c_int),
                ("nwavs", C.c_int), ("wavs", C.c_double * MAX_WAVS), ("specfile", C.c_char * STR),
                ("radQ", C.c_int), ("SWQ", C.c_int), ("FLQ", C.c_int),
                ("n_planets", C.c_int), ("planets", Planet * MAX_PLANETS),
                ("rho", C.c_double), ("kqe", C.c_double), ("comp", C.c_char * STR),
                ("n_disks", C.c_int), ("disks", Disk * MAX_DISKS),
                ("n_blobs", C.c_int), ("blobs", Blob * MAX_BLOBS),
                ("name_stub", C.c_char * STR), ("usage_code", C.c_int)]


class ParamError(RuntimeError):
    def __init__(self, status: int, usage_code: int):
        super().__init__(f"parameter file rejected: status {status}, usage code {usage_code}")
        self.status, self.usage_code = status, usage_code


def read_param(path: str) -> dict:
    """Parse a DiskDyn parameter file with ddx_param_read; the reference's fields and units."""
    lib = abi.load()
    p = Param()
    st = lib.ddx_param_read(str(path).encode(), C.byref(p))
    if st != 0:
        raise ParamError(st, p.usage_code)
    d = {k: getattr(p, k) for k, _ in Param._fields_
         if k not in ("sptype", "specfile", "comp", "name_stub", "wavs", "planets", "disks", "blobs", "nwavs",
                      "n_planets", "n_disks", "n_blobs", "usage_code")}
    for k in ("sptype", "specfile", "comp", "name_stub"):
        d[k] = getattr(p, k).decode()
    d["wavs"] = [p.wavs[k] for k in range(p.nwavs)]
    d["planets"] = [[getattr(p.planets[k], f) for f, _ in Planet._fields_] for k in range(p.n_planets)]
    d["disks"] = [{f: getattr(p.disks[k], f) for f, _ in Disk._fields_} for k in range(p.n_disks)]
    d["blobs"] = [{f: getattr(p.blobs[k], f) for f, _ in Blob._fields_} for k in range(p.n_blobs)]
    return d
