"""ctypes binding of libddx.so, the C ABI declared in include/diskdyn_gb300.h.

Device arrays are passed as torch CUDA tensors (their data pointers go straight into the
ABI structs) and the caller's current torch stream is used unless a stream is given.
Every call raises DDXError on a non-zero status; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libddx.so"

DDX_OK = 0
DDX_ERR_ARG, DDX_ERR_CUDA, DDX_ERR_NOMEM, DDX_ERR_STATE, DDX_ERR_RANGE, DDX_ERR_TIMEOUT = 1, 2, 3, 4, 5, 6
DDX_PREC_FP64 = 0
DDX_PREC_MIXED = 1
DDX_PREC_COMPENSATED = 2
DDX_MODE_FIXED = 0
DDX_MODE_REFERENCE = 1
DDX_MAX_SIZE_BINS = 2700
DDX_NR = 100

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "device allocation failed",
          4: "required table not set", 5: "size beyond limit", 6: "device-side wait timed out",
          7: "non-finite value", 8: "file could not be opened, read or written"}


class DDXError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS.get(status, 'unknown')} (status {status})")
        self.status = status


class State(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("vx", C.c_void_p), ("vy", C.c_void_p), ("vz", C.c_void_p),
                ("m", C.c_void_p), ("N", C.c_void_p), ("id", C.c_void_p)]


class Phys(C.Structure):
    _fields_ = [("radQ", C.c_int), ("SWQ", C.c_int), ("FLQ", C.c_int),
                ("Wz", C.c_double), ("Bstar", C.c_double), ("Rstar", C.c_double),
                ("rho", C.c_double), ("vsw_AUyr", C.c_double), ("Rmin", C.c_double),
                ("n_planets", C.c_int)]


class View(C.Structure):
    _fields_ = [("dist", C.c_double), ("fov", C.c_double), ("PA", C.c_double),
                ("inc", C.c_double), ("longitude", C.c_double),
                ("xsize", C.c_int), ("ysize", C.c_int)]


class OpticalTable(C.Structure):
    """ddx_optical_table: host pointers to s[n_size], Qabs/Qsca[n_size][n_wav] and
    Qpfunc[n_size][n_theta][n_wav]."""
    _fields_ = [("n_size", C.c_int), ("n_wav", C.c_int), ("n_theta", C.c_int), ("s", C.c_void_p),
                ("Qabs", C.c_void_p), ("Qsca", C.c_void_p), ("Qpfunc", C.c_void_p)]


class GridSetup(C.Structure):
    _fields_ = [("n_grid", C.c_int), ("amin", C.c_double), ("amax", C.c_double), ("dmax", C.c_double),
                ("kqe", C.c_double), ("radQ", C.c_int), ("SWQ", C.c_int), ("rho", C.c_double),
                ("dist", C.c_double), ("mstar", C.c_double), ("mloss", C.c_double), ("vsw", C.c_double)]


class Cadence(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("t_write", "t_fits", "t_sed", "t_end", "time", "tlastd", "tlastf",
                                          "tlasts", "model_dt")] + [("initial_outputs", C.c_int)]


class HostStateView(C.Structure):
    _fields_ = [(k, C.POINTER(C.c_double)) for k in ("x", "y", "z", "vx", "vy", "vz", "N", "m")] + \
               [("id", C.POINTER(C.c_int)), ("cap", C.c_longlong)]


class Output(C.Structure):
    _fields_ = [("kind", C.c_int), ("time", C.c_double), ("model_dt", C.c_double), ("tlastd", C.c_double),
                ("tlastf", C.c_double), ("tlasts", C.c_double), ("data", C.POINTER(C.c_double)),
                ("n", C.c_longlong), ("state", C.POINTER(HostStateView))]


OUTPUT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(Output))
DDX_OUT_IMAGES, DDX_OUT_SED, DDX_OUT_STATE = 1, 2, 3


# (name, restype, argtypes) of every symbol include/diskdyn_gb300.h declares.
SIGNATURES = [
    ("ddx_param_read", C.c_int, [C.c_char_p, C.c_void_p]),
    ("ddx_dat_write", C.c_int, [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddx_dat_read", C.c_int, [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddx_sed_write", C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddx_fits_write", C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double,
                                 C.c_double]),
    ("ddx_optical_read", C.c_int, [C.c_char_p, C.POINTER(OpticalTable), C.c_void_p, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]),
    ("ddx_spec_read", C.c_int, [C.c_char_p, C.c_double, C.c_double, C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                                C.c_int]),
    ("ddx_stellar_grid", C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_void_p]),
    ("ddx_param_grid", C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    ("ddx_setup_count", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_void_p]),
    ("ddx_setup_host", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_longlong, C.c_void_p,
                                 C.c_void_p]),
    ("ddx_setup_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_ulonglong,
                                   C.POINTER(State), C.c_longlong, C.c_void_p, C.c_void_p]),
    ("ddx_step_host", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                                C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_schedule", C.c_int, [C.POINTER(Cadence), C.c_double, C.c_longlong, C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_longlong)]),
    ("ddx_run", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double, C.POINTER(Phys), C.c_int,
                          C.c_int, C.POINTER(View), C.c_void_p, C.c_int, C.POINTER(Cadence), OUTPUT_FN, C.c_void_p,
                          C.c_void_p]),
    ("ddx_abi_version", C.c_int, []),
    ("ddx_status_string", C.c_char_p, [C.c_int]),
    ("ddx_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    ("ddx_destroy", C.c_int, [C.c_void_p]),
    ("ddx_set_size_table", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddx_set_optics", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6 + [C.c_double, C.c_double]),
    ("ddx_step", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                           C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_massive_rk4", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                                  C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_small_rk4", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                                C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_massive_final", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                                    C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_step_noalloc", C.c_int, [C.c_int, C.POINTER(State), C.c_int, C.c_int, C.c_double,
                                   C.POINTER(Phys), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int, C.c_int, C.c_void_p]),
    ("ddx_evolve", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double, C.c_int,
                             C.POINTER(Phys), C.c_int, C.c_int, C.c_void_p]),
    ("ddx_image", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.POINTER(View),
                            C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    ("ddx_sed", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.POINTER(View),
                          C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("ddx_collide", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double, C.c_void_p,
                              C.c_longlong, C.POINTER(C.c_longlong), C.c_void_p]),
    ("ddx_adjoint_forward", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_double, C.c_int,
                                      C.c_int, C.POINTER(Phys), C.POINTER(View), C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p]),
    ("ddx_adjoint_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ddx_debug_pixels", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.POINTER(View),
                                   C.c_void_p, C.c_void_p]),
    ("ddx_debug_exact_pixel_count", C.c_ulonglong, [C.c_void_p]),
    ("ddx_det_step", C.c_int, [C.c_void_p, C.POINTER(State), C.c_int, C.c_int, C.c_void_p, C.c_int,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double),
                               C.c_void_p]),
    ("ddx_dust_temp", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p, C.c_void_p]),
    ("ddx_dust_grid", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(OpticalTable),
                                C.POINTER(GridSetup), C.POINTER(OpticalTable), C.c_void_p, C.c_void_p, C.c_void_p,
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]),
    ("ddx_sync_status", C.c_int, [C.c_void_p, C.c_void_p]),
    ("ddx_debug_lose_tile_copy", C.c_int, [C.c_void_p, C.c_int, C.c_ulonglong]),
    ("ddx_noalloc_sync_status", C.c_int, [C.c_int, C.c_void_p]),
    ("ddx_debug_noalloc_lose_tile_copy", C.c_int, [C.c_int, C.c_int, C.c_ulonglong]),
    ("ddx_set_near_radius", C.c_int, [C.c_void_p, C.c_double]),
    ("ddx_set_compensated_radius", C.c_int, [C.c_void_p, C.c_double]),
    ("ddx_probe_fma_peak", C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
]

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libddx.so (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with diskdyn_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != DDX_OK:
        raise DDXError(status, where)
