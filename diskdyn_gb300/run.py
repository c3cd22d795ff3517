"""A whole run with the reference's output cadence (include/diskdyn_gb300_run.h).

`schedule` lists the steps and outputs of a cadence on the host; `file_writer` turns the
outputs of Engine.run into the reference's files under its names (src/grid.cu:449, 681,
src/fits.cu:29): <stub>_<time %.2f>.dat, <stub>_SED_<time %.2f>.dat and
<stub>_<wavelength um %.2f>_<time %.3f>.fits per image wavelength.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi, formats

CADENCE_KEYS = ("t_write", "t_fits", "t_sed", "t_end", "time", "tlastd", "tlastf", "tlasts", "model_dt")


def cadence_struct(cad: dict) -> abi.Cadence:
    return abi.Cadence(**{k: float(cad.get(k, 0.0)) for k in CADENCE_KEYS},
                       initial_outputs=int(cad.get("initial_outputs", 0)))


def schedule(cad: dict, dt: float):
    """ddx_schedule: (step sizes, output masks) of the run ddx_run makes."""
    lib = abi.load()
    c = cadence_struct(cad)
    n = C.c_longlong()
    abi.check(lib.ddx_schedule(C.byref(c), float(dt), 0, None, None, C.byref(n)), "ddx_schedule")
    h = np.zeros(n.value)
    m = np.zeros(n.value, np.int32)
    abi.check(lib.ddx_schedule(C.byref(c), float(dt), n.value, C.c_void_p(h.ctypes.data), C.c_void_p(m.ctypes.data),
                               C.byref(n)), "ddx_schedule")
    return h, m


def file_writer(directory, stub: str, version: str, param: formats.Param, w, influx, wj, beta, view: abi.View,
                n_mass: int, n_dust: int, Rmax: float, nR: int = 100):
    """A callback for Engine.run that writes every output as the reference writes it."""
    from pathlib import Path
    base = str(Path(directory) / stub)
    w = np.asarray(w, np.float64)
    wj = np.asarray(wj, np.int32)
    written = []

    def on_output(o):
        t = o["time"]
        if o["kind"] == abi.DDX_OUT_IMAGES:
            imgs = o["data"].reshape(len(wj), view.xsize, view.ysize)
            for j, k in enumerate(wj):
                path = f"{base}_{w[k] * 1e6:.2f}_{t:.3f}.fits"
                formats.write_fits(path, version, imgs[j], w[k], view.fov, view.dist)
                written.append(path)
        elif o["kind"] == abi.DDX_OUT_SED:
            path = f"{base}_SED_{t:.2f}.dat"
            formats.write_sed(path, version, w, influx, o["data"])
            written.append(path)
        else:
            st = o["state"]
            run = formats.DatRun(time=t, dt=o["model_dt"], tlastd=o["tlastd"], tlastf=o["tlastf"],
                                 tlasts=o["tlasts"], Rmax=Rmax, nR=nR, n_mass=n_mass, n_dust=n_dust,
                                 n_all=len(st["x"]))
            path = f"{base}_{t:.2f}.dat"
            formats.write_dat(path, version, param, run, st, beta)
            written.append(path)
        return False

    on_output.written = written
    return on_output
