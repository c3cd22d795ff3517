"""Python view of the reference-format file functions of libddx.so
(include/diskdyn_gb300_io.h): the parameter-file parser, the data (restart) file writer
and reader, the SED file and FITS image writers."""
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
                ("name_stub", C.c_char * STR), ("usage_code", C.c_int),
                ("amin", C.c_double), ("amax", C.c_double), ("mmin", C.c_double), ("mmax", C.c_double),
                ("f", C.c_double), ("n_grid", C.c_int), ("n_wav", C.c_int), ("n_theta", C.c_int),
                ("n_dust", C.c_int), ("seed", C.c_longlong)]


class DatRun(C.Structure):
    _fields_ = [("time", C.c_double), ("dt", C.c_double), ("tlastd", C.c_double), ("tlastf", C.c_double),
                ("tlasts", C.c_double), ("Rmax", C.c_double), ("nR", C.c_int), ("n_mass", C.c_int),
                ("n_dust", C.c_int), ("n_all", C.c_int)]


class HostState(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")] + [("cap", C.c_longlong)]


STATE_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")


def host_state(arrays: dict) -> HostState:
    """HostState over numpy arrays (float64; id int32), which must stay alive."""
    return HostState(*[arrays[k].ctypes.data for k in STATE_FIELDS], len(arrays["x"]))


class ParamError(RuntimeError):
    def __init__(self, status: int, usage_code: int):
        super().__init__(f"parameter file rejected: status {status}, usage code {usage_code}")
        self.status, self.usage_code = status, usage_code


def read_param_struct(path: str) -> Param:
    lib = abi.load()
    p = Param()
    st = lib.ddx_param_read(str(path).encode(), C.byref(p))
    if st != 0:
        raise ParamError(st, p.usage_code)
    return p


def read_param(path: str) -> dict:
    """Parse a DiskDyn parameter file with ddx_param_read; the reference's fields and units."""
    return param_dict(read_param_struct(path))


def param_dict(p: Param) -> dict:
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


def write_dat(path, version: str, p: Param, run: DatRun, arrays: dict, beta) -> None:
    """ddx_dat_write: the data file of state `arrays` (massive bodies first)."""
    import numpy as np
    beta = np.ascontiguousarray(beta, np.float32)
    st = abi.load().ddx_dat_write(str(path).encode(), version.encode(), C.byref(p), C.byref(run),
                                  C.byref(host_state(arrays)), C.c_void_p(beta.ctypes.data))
    abi.check(st, "ddx_dat_write")


def read_dat(path, version: str, nR: int = 100, Rmax: float = 0.0):
    """ddx_dat_read: (param struct, run struct, state arrays) of a data file.  Rmax (AU,
    the temperature table's outer radius) is not in the file and is passed through."""
    import numpy as np
    lib = abi.load()
    p, run = Param(), DatRun(nR=nR, Rmax=Rmax)
    st = lib.ddx_dat_read(str(path).encode(), version.encode(), C.byref(p), C.byref(run), None)
    if st != 0:
        raise ParamError(st, p.usage_code)
    arrays = {k: np.zeros(run.n_all, np.int32 if k == "id" else np.float64) for k in STATE_FIELDS}
    run.nR = nR
    st = lib.ddx_dat_read(str(path).encode(), version.encode(), C.byref(p), C.byref(run),
                          C.byref(host_state(arrays)))
    if st != 0:
        raise ParamError(st, p.usage_code)
    return p, run, arrays


def write_sed(path, version: str, w, influx, exc) -> None:
    import numpy as np
    w, influx, exc = (np.ascontiguousarray(a, np.float64) for a in (w, influx, exc))
    abi.check(abi.load().ddx_sed_write(str(path).encode(), version.encode(), len(w), C.c_void_p(w.ctypes.data),
                                       C.c_void_p(influx.ctypes.data), C.c_void_p(exc.ctypes.data)), "ddx_sed_write")


def write_fits(path, version: str, image, wavelength_m: float, fov_AU: float, dist_m: float) -> None:
    """ddx_fits_write of one x-major image (xsize, ysize), as ddx_image returns it."""
    import numpy as np
    F = np.ascontiguousarray(image, np.float64)
    xs, ys = F.shape
    abi.check(abi.load().ddx_fits_write(str(path).encode(), version.encode(), xs, ys, C.c_void_p(F.ctypes.data),
                                        float(wavelength_m), float(fov_AU), float(dist_m)), "ddx_fits_write")


def read_optical(path) -> dict:
    """ddx_optical_read: the Mie table file as a dict of s (m), w (m), Qabs, Qsca
    (n_size, n_wav), Qpfunc (n_size, n_theta, n_wav), dmin and dmax (m)."""
    import numpy as np
    lib = abi.load()
    t = abi.OpticalTable()
    dmin, dmax = C.c_double(), C.c_double()
    abi.check(lib.ddx_optical_read(str(path).encode(), C.byref(t), None, C.byref(dmin), C.byref(dmax)),
              "ddx_optical_read")
    nd, nw, nt = t.n_size, t.n_wav, t.n_theta
    d = {"s": np.zeros(nd), "w": np.zeros(nw), "Qabs": np.zeros((nd, nw)), "Qsca": np.zeros((nd, nw)),
         "Qpfunc": np.zeros((nd, nt, nw))}
    t.s, t.Qabs, t.Qsca, t.Qpfunc = (d[k].ctypes.data for k in ("s", "Qabs", "Qsca", "Qpfunc"))
    abi.check(lib.ddx_optical_read(str(path).encode(), C.byref(t), C.c_void_p(d["w"].ctypes.data), C.byref(dmin),
                                   C.byref(dmax)), "ddx_optical_read")
    d["dmin"], d["dmax"] = dmin.value, dmax.value
    return d


def read_spec(path, rstar_AU: float, dist_m: float):
    """ddx_spec_read: (wavelengths, fluxes scaled to the observer) of a spectrum file."""
    import numpy as np
    lib = abi.load()
    n = C.c_int()
    abi.check(lib.ddx_spec_read(str(path).encode(), rstar_AU, dist_m, C.byref(n), None, None, 0), "ddx_spec_read")
    w, F = np.zeros(n.value), np.zeros(n.value)
    abi.check(lib.ddx_spec_read(str(path).encode(), rstar_AU, dist_m, C.byref(n), C.c_void_p(w.ctypes.data),
                                C.c_void_p(F.ctypes.data), n.value), "ddx_spec_read")
    return w, F


def stellar_grid(w, spec_w, spec_F, wavs=()):
    """ddx_stellar_grid: (in[n_wav], wj[len(wavs)])."""
    import numpy as np
    w, spec_w, spec_F = (np.ascontiguousarray(a, np.float64) for a in (w, spec_w, spec_F))
    wavs = np.ascontiguousarray(wavs, np.float64)
    influx = np.zeros(w.size)
    wj = np.zeros(max(wavs.size, 1), np.int32)
    P = lambda a: C.c_void_p(a.ctypes.data)
    abi.check(abi.load().ddx_stellar_grid(w.size, P(w), spec_w.size, P(spec_w), P(spec_F), wavs.size, P(wavs),
                                          P(influx), P(wj)), "ddx_stellar_grid")
    return influx, wj[:wavs.size]


def param_grid(p: Param, dmin: float, dmax: float) -> None:
    """ddx_param_grid on a parsed parameter file, in place: grain ranges clipped to the
    optical table's [dmin, dmax] (m), the mass grid and the number constants."""
    abi.check(abi.load().ddx_param_grid(C.byref(p), float(dmin), float(dmax)), "ddx_param_grid")


def setup_count(p: Param, dmin: float, dmax: float) -> DatRun:
    run = DatRun()
    abi.check(abi.load().ddx_setup_count(C.byref(p), float(dmin), float(dmax), C.byref(run)), "ddx_setup_count")
    return run


def setup_host(p: Param, dmin: float, dmax: float, beta, seed: int = -2):
    """ddx_setup_host: (state arrays, run counts) of Grid::setup's bodies with the
    reference's generator."""
    import numpy as np
    run = setup_count(p, dmin, dmax)
    arrays = {k: np.zeros(run.n_all, np.int32 if k == "id" else np.float64) for k in STATE_FIELDS}
    beta = np.ascontiguousarray(beta, np.float32)
    abi.check(abi.load().ddx_setup_host(C.byref(p), float(dmin), float(dmax), C.c_void_p(beta.ctypes.data), int(seed),
                                        C.byref(host_state(arrays)), C.byref(run)), "ddx_setup_host")
    return arrays, run
