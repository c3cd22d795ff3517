"""ORACLE -- test infrastructure.  ctypes binding of liboracle.so (ddx_oracle.c)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import LIB, build

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")


class OState(C.Structure):
    _fields_ = [(f, C.c_void_p) for f in FIELDS]


class OPhys(C.Structure):
    _fields_ = [("radQ", C.c_int), ("SWQ", C.c_int), ("FLQ", C.c_int), ("Wz", C.c_double),
                ("Bstar", C.c_double), ("Rstar", C.c_double), ("rho", C.c_double),
                ("vsw_AUyr", C.c_double), ("Rmin", C.c_double)]


class OView(C.Structure):
    _fields_ = [("dist", C.c_double), ("fov", C.c_double), ("PA", C.c_double),
                ("inc", C.c_double), ("longitude", C.c_double), ("xsize", C.c_int),
                ("ysize", C.c_int)]


class OOptics(C.Structure):
    _fields_ = [("w", C.c_void_p), ("in_", C.c_void_p), ("Qabs", C.c_void_p), ("Qsca", C.c_void_p),
                ("Qpfunc", C.c_void_p), ("Td", C.c_void_p), ("size", C.c_void_p),
                ("Rmin", C.c_double), ("Rmax", C.c_double), ("n_grid", C.c_int),
                ("n_wav", C.c_int), ("n_theta", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.ora_step.argtypes = [OState, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.POINTER(OPhys), C.c_int, C.c_void_p]
        _lib.ora_dust.argtypes = [OState, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(OPhys), C.c_int]
        _lib.ora_image.argtypes = [OState, C.c_int, C.c_int, C.POINTER(OOptics), C.POINTER(OView),
                                   C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.ora_sed.argtypes = [OState, C.c_int, C.c_int, C.POINTER(OOptics), C.POINTER(OView),
                                 C.c_void_p, C.c_int]
        _lib.ora_dust_temp.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]
        for f in ("ora_step", "ora_dust", "ora_image", "ora_sed", "ora_dust_temp"):
            getattr(_lib, f).restype = C.c_int
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def host_state(arrays: dict) -> tuple[dict, OState]:
    """Contiguous copies of a state dict and the struct pointing at them."""
    st = {f: np.array(arrays[f], dtype=np.int32 if f == "id" else np.float64, copy=True) for f in FIELDS}
    return st, OState(*[_ptr(st[f]) for f in FIELDS])


def phys(d: dict) -> OPhys:
    return OPhys(int(d["radQ"]), int(d["SWQ"]), int(d["FLQ"]), float(d["Wz"]), float(d["Bstar"]),
                 float(d["Rstar"]), float(d["rho"]), float(d["vsw_AUyr"]), float(d["Rmin"]))


def view(d: dict) -> OView:
    return OView(float(d["dist"]), float(d["fov"]), float(d["PA"]), float(d["inc"]),
                 float(d["longitude"]), int(d["xsize"]), int(d["ysize"]))


def step(arrays: dict, n_grav: int, dt: float, size_table: dict, phys_d: dict, n_steps: int = 1,
         ref_mode: bool = False, return_kpos: bool = False):
    """n_steps reference steps on a copy of `arrays`; returns the new state dict
    (and the massive stage positions of the last step, shape (4, 3, n_grav))."""
    st, os_ = host_state(arrays)
    n_dust = len(st["x"]) - n_grav
    b = np.ascontiguousarray(size_table["beta"], np.float32)
    bs = np.ascontiguousarray(size_table["betasw"], np.float32)
    q = np.ascontiguousarray(size_table["q"], np.float32)
    kpos = np.zeros((4, 3, n_grav))
    ph = phys(phys_d)
    for _ in range(n_steps):
        r = lib().ora_step(os_, n_grav, n_dust, float(dt), _ptr(b), _ptr(bs), _ptr(q), C.byref(ph),
                           int(ref_mode), _ptr(kpos))
        if r:
            raise RuntimeError("ora_step failed")
    return (st, kpos) if return_kpos else st


def dust(arrays: dict, n_grav: int, dt: float, kpos, size_table: dict, phys_d: dict,
         i0: int = 0, i1: int | None = None, ref_mode: bool = False) -> dict:
    """Dust half of a step with given massive stage positions (4, 3, n_grav)."""
    st, os_ = host_state(arrays)
    n_dust = len(st["x"]) - n_grav
    i1 = n_dust if i1 is None else i1
    kp = np.ascontiguousarray(kpos, np.float64)
    b = np.ascontiguousarray(size_table["beta"], np.float32)
    bs = np.ascontiguousarray(size_table["betasw"], np.float32)
    q = np.ascontiguousarray(size_table["q"], np.float32)
    ph = phys(phys_d)
    if lib().ora_dust(os_, n_grav, n_dust, i0, i1, float(dt), _ptr(kp), _ptr(b), _ptr(bs), _ptr(q),
                      C.byref(ph), int(ref_mode)):
        raise RuntimeError("ora_dust failed")
    return st


def _optics(o: dict, size):
    keep = {k: np.ascontiguousarray(o[k], np.float64) for k in ("w", "in", "Qabs", "Qsca", "Qpfunc", "Td")}
    keep["size"] = np.ascontiguousarray(size, np.float64)
    oo = OOptics(_ptr(keep["w"]), _ptr(keep["in"]), _ptr(keep["Qabs"]), _ptr(keep["Qsca"]),
                 _ptr(keep["Qpfunc"]), _ptr(keep["Td"]), _ptr(keep["size"]), float(o["Rmin"]),
                 float(o["Rmax"]), keep["Qabs"].shape[0], len(keep["w"]), keep["Qpfunc"].shape[1])
    return keep, oo


def image(arrays: dict, n_grav: int, optics: dict, size, view_d: dict, wj):
    """Images (n_img, xsize, ysize) and per-tracer pixel index (-1 = none)."""
    st, os_ = host_state(arrays)
    n_dust = len(st["x"]) - n_grav
    keep, oo = _optics(optics, size)
    v = view(view_d)
    wj_a = np.ascontiguousarray(wj, np.int32)
    Fd = np.zeros((len(wj_a), v.xsize, v.ysize))
    pix = np.zeros(max(n_dust, 1), np.int32)
    lib().ora_image(os_, n_grav, n_dust, C.byref(oo), C.byref(v), _ptr(wj_a), len(wj_a), _ptr(Fd), _ptr(pix))
    return Fd, pix[:n_dust]


def sed(arrays: dict, n_grav: int, optics: dict, size, view_d: dict, ref_mode: bool = False):
    st, os_ = host_state(arrays)
    n_dust = len(st["x"]) - n_grav
    keep, oo = _optics(optics, size)
    v = view(view_d)
    out = np.zeros(oo.n_wav)
    lib().ora_sed(os_, n_grav, n_dust, C.byref(oo), C.byref(v), _ptr(out), int(ref_mode))
    return out


def dust_temp(w, influx, Qabs, dist, Rmax_AU):
    """calculate_dust_temp (src/grid.cu:754-834): returns Td (n_grid, 100), Rmin, Rmax [AU]."""
    w = np.ascontiguousarray(w, np.float64)
    influx = np.ascontiguousarray(influx, np.float64)
    Qabs = np.ascontiguousarray(Qabs, np.float64)
    n_grid, n_wav = Qabs.shape
    Td = np.zeros((n_grid, 100))
    rmin = C.c_double(0.0)
    rmax = C.c_double(float(Rmax_AU))
    lib().ora_dust_temp(n_grid, n_wav, _ptr(w), _ptr(influx), _ptr(Qabs), float(dist), C.byref(rmin),
                        C.byref(rmax), _ptr(Td))
    return Td, rmin.value, rmax.value


def det_step(arrays: dict, n_grav: int, n_step: int, disk_Rin=(), blobs=()) -> float:
    """Grid::det_step (src/grid.cu:312-342); blobs is a sequence of (a, ecc, sigma)."""
    xs = [np.ascontiguousarray(arrays[k][:max(n_grav, 1)], np.float64) for k in ("x", "y", "z", "m")]
    rin = np.ascontiguousarray(disk_Rin, np.float64)
    bl = np.ascontiguousarray(np.reshape(blobs, (-1, 3)), np.float64)
    ba, be, bs = (np.ascontiguousarray(bl[:, k]) for k in range(3))
    f = lib().ora_det_step
    f.restype = C.c_double
    f.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 3 + [C.c_int]
    return f(*[_ptr(a) for a in xs], int(n_grav), int(n_step), _ptr(rin), rin.size, _ptr(ba), _ptr(be),
             _ptr(bs), ba.size)


def collide(arrays: dict, i0: int, i1: int, h: float, method: str = "brute", cap: int | None = None):
    """Collision pairs (m, 2) of live tracers i < j in [i0, i1) closer than h, (i, j) order."""
    st, os_ = host_state(arrays)
    f = lib().ora_collide_brute if method == "brute" else lib().ora_collide_grid
    f.restype = C.c_longlong
    f.argtypes = [OState, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_longlong]
    total = f(os_, i0, i1, float(h), None, 0)
    out = np.zeros((max(total, 1), 2), np.int32)
    f(os_, i0, i1, float(h), _ptr(out), total)
    return out[:total]


def stellar_grid(w, spec_w, spec_F, wavs=()):
    """interpolate_stellar_to_grid (src/functions.cu:302-336): (in[n_wav], wj[len(wavs)]);
    raises ValueError with the reference's usage code 43 for an image wavelength outside w."""
    w, spec_w, spec_F = (np.ascontiguousarray(a, np.float64) for a in (w, spec_w, spec_F))
    wavs = np.ascontiguousarray(wavs, np.float64)
    influx = np.zeros(w.size)
    wj = np.zeros(max(wavs.size, 1), np.int32)
    f = lib().ora_stellar_grid
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    r = f(w.size, _ptr(w), spec_w.size, _ptr(spec_w), _ptr(spec_F), wavs.size, _ptr(wavs), _ptr(influx), _ptr(wj))
    if r != 0:
        raise ValueError(f"usage code {r}")
    return influx, wj[:wavs.size]


def dust_grid(w, influx, table: dict, n_grid, amin, amax, dmax, kqe, radQ, SWQ, rho, dist, mstar, mloss, vsw):
    """interpolate_dust_to_grid + calculate_beta (src/functions.cu:243-300, 338-388) on the
    optical file's s, Qabs, Qsca, Qpfunc; returns the grid's s, q, Qabs, Qsca, Qpfunc, beta,
    betasw, Lum, betaswconst.  Raises ValueError with usage code 54 when the last bin
    overshoots dmax."""
    w, influx = (np.ascontiguousarray(a, np.float64) for a in (w, influx))
    src = {k: np.ascontiguousarray(table[k], np.float64) for k in ("s", "Qabs", "Qsca", "Qpfunc")}
    nd, nt, nw = src["Qpfunc"].shape
    o = {"s": np.zeros(n_grid), "q": np.zeros(n_grid, np.float32), "Qabs": np.zeros((n_grid, nw)),
         "Qsca": np.zeros((n_grid, nw)), "Qpfunc": np.zeros((n_grid, nt, nw)), "beta": np.zeros(n_grid, np.float32),
         "betasw": np.zeros(n_grid, np.float32)}
    lum, bsc = C.c_double(), C.c_double()
    f = lib().ora_dust_grid
    f.restype = C.c_int
    f.argtypes = ([C.c_int] * 3 + [C.c_void_p] * 6 + [C.c_int] + [C.c_double] * 4 + [C.c_int] * 2 +
                  [C.c_double] * 5 + [C.c_void_p] * 7 + [C.POINTER(C.c_double)] * 2)
    r = f(nd, nw, nt, _ptr(src["s"]), _ptr(w), _ptr(src["Qabs"]), _ptr(src["Qsca"]), _ptr(src["Qpfunc"]),
          _ptr(influx), int(n_grid), float(amin), float(amax), float(dmax), float(kqe), int(radQ), int(SWQ),
          float(rho), float(dist), float(mstar), float(mloss), float(vsw),
          *(_ptr(o[k]) for k in ("s", "q", "Qabs", "Qsca", "Qpfunc", "beta", "betasw")), C.byref(lum), C.byref(bsc))
    if r != 0:
        raise ValueError(f"usage code {r}")
    o["Lum"], o["betaswconst"] = lum.value, bsc.value
    return o


class ODisk(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("Rin", "Rout", "sigmae", "gammas", "dhdr")]


class OBlob(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("a", "ecc", "inc", "w", "o", "nu", "sigma", "vkepp")] + [("collcloud", C.c_int)]


def setup_populations(p, dmin: float, dmax: float):
    """Grid::setup's body order (src/grid.cu:79-190) after the planets, as (kind, index)
    per body: kind 0 = disk, 1 = blob; the gravitating bodies of every disk then blob, then
    round(Nsmall / Ngrid) grains per mass bin of every disk then blob.  p is a parsed
    parameter struct after the grid set-up (fields mmin, f, disks, blobs)."""
    import math
    kind, idx = [], []
    for k, n, pops in ((0, p.n_disks, p.disks), (1, p.n_blobs, p.blobs)):
        for j in range(n):
            kind += [k] * pops[j].Ngrav
            idx += [j] * pops[j].Ngrav
    for k, n, pops in ((0, p.n_disks, p.disks), (1, p.n_blobs, p.blobs)):
        for j in range(n):
            mmax = p.mmin * math.exp(round(math.log(pops[j].dmmax / p.mmin) / p.f) * p.f)
            mmin = p.mmin * math.exp(round(math.log(pops[j].mmin / p.mmin) / p.f) * p.f)
            ngrid = int(round(math.log(mmax / mmin) / math.log(1.1) + 1))
            npg = int(round(pops[j].Nsmall / ngrid))
            kind += [k] * (ngrid * npg)
            idx += [j] * (ngrid * npg)
    return np.asarray(kind, np.int32), np.asarray(idx, np.int32)


def setup_philox(p, kind, idx, m, beta, seed: int, first: int):
    """The GPU set-up's counter-based orbit draws for bodies first.. (oracle restatement):
    returns (n, 6) states x y z vx vy vz and the number of bodies whose rejections ran out."""
    disks = (ODisk * max(p.n_disks, 1))(*[ODisk(d.Rin, d.Rout, d.sigmae, d.gammas, d.dhdr)
                                          for d in list(p.disks)[:p.n_disks]])
    blobs = (OBlob * max(p.n_blobs, 1))(*[OBlob(b.a, b.ecc, b.inc, b.w, b.o, b.nu, b.sigma, b.vkepp, b.collcloud)
                                          for b in list(p.blobs)[:p.n_blobs]])
    kind, idx = (np.ascontiguousarray(a, np.int32) for a in (kind, idx))
    m, beta = (np.ascontiguousarray(a, np.float64) for a in (m, beta))
    out = np.zeros((len(kind), 6))
    f = lib().ora_setup_philox
    f.restype = C.c_longlong
    f.argtypes = [C.c_longlong, C.c_longlong] + [C.c_void_p] * 4 + [C.c_void_p, C.c_void_p, C.c_double,
                                                                    C.c_ulonglong, C.c_void_p]
    bad = f(len(kind), int(first), _ptr(kind), _ptr(idx), _ptr(m), _ptr(beta), C.cast(disks, C.c_void_p),
            C.cast(blobs, C.c_void_p), float(p.planets[0].m), int(seed) & (2 ** 64 - 1), _ptr(out))
    return out, bad


def philox4x32_10(ctr, key):
    f = lib().ora_philox4x32_10
    f.argtypes = [C.c_uint32 * 4, C.c_uint32 * 2, C.c_uint32 * 4]
    o = (C.c_uint32 * 4)()
    f((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), o)
    return tuple(o)


def cadence(cad: dict, dt: float):
    """Grid::evolve's step sizes and output triggers (src/grid.cu:375-434) restated: a list
    of (step size, outputs after it), outputs a tuple of "sed", "images", "state" in the
    order the reference writes them."""
    time = cad.get("time", 0.0)
    tlastd, tlastf, tlasts = cad.get("tlastd", 0.0), cad.get("tlastf", 0.0), cad.get("tlasts", 0.0)
    t_write, t_fits, t_sed, t_end = cad["t_write"], cad["t_fits"], cad["t_sed"], cad["t_end"]

    def clip(dttmp):
        if time + dttmp > tlastd + t_write:
            dttmp = t_write + tlastd - time
        if time + dttmp > tlastf + t_fits:
            dttmp = t_fits + tlastf - time
        if time + dttmp > tlasts + t_sed:
            dttmp = t_sed + tlasts - time
        if time + dttmp > t_end:
            dttmp = t_end - time
        return dttmp

    dttmp = clip(dt)
    out = []
    while True:
        h = dttmp
        time += dttmp
        due = []
        if time >= tlasts + t_sed or time >= t_end:
            due.append("sed")
            tlasts = time
            dttmp = dt
        if time >= tlastf + t_fits or time >= t_end:
            due.append("images")
            tlastf = time
            dttmp = dt
        if time >= tlastd + t_write or time >= t_end:
            due.append("state")
            tlastd = time
            dttmp = dt
        dttmp = clip(dttmp)
        out.append((h, tuple(due)))
        if not time < t_end:
            break
    return out
