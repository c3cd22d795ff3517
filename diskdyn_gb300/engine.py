"""Python host interface of the GB300 DiskDyn path, over the C ABI.

`Engine` mirrors the reference's `class Grid` where the hot path is concerned
(src/ddyn.cuh:213-275): it owns the device-side tables (size bins, optics) and runs the
step (`massive_RK4 + small_RK4 + massive_final`, src/grid.cu:387-389), the images
(`null_flux + calc_flux`, src/grid.cu:411-421) and the SED (src/grid.cu:396-406) through
libddx.so.  The particle state stays in caller-owned torch CUDA tensors in the
reference's layout: one array per field, massive bodies first, star at index 0.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import abi

STATE_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m", "N", "id")


@dataclass
class DeviceState:
    """SoA particle state on the GPU (float64 fields, int32 id), n_grav + n_dust long."""
    x: torch.Tensor
    y: torch.Tensor
    z: torch.Tensor
    vx: torch.Tensor
    vy: torch.Tensor
    vz: torch.Tensor
    m: torch.Tensor
    N: torch.Tensor
    id: torch.Tensor
    _abi: abi.State = field(default=None, repr=False)

    def __post_init__(self):
        n = self.x.numel()
        for name in STATE_FIELDS:
            t = getattr(self, name)
            want = torch.int32 if name == "id" else torch.float64
            if t.dtype != want or not t.is_cuda or not t.is_contiguous() or t.numel() != n:
                raise ValueError(f"state field {name}: need contiguous CUDA {want} of length {n}")
        self._abi = abi.State(*[getattr(self, f).data_ptr() for f in STATE_FIELDS])

    @property
    def n_all(self) -> int:
        return self.x.numel()

    @classmethod
    def from_numpy(cls, arrays: dict, device="cuda:0", pin: bool = False) -> "DeviceState":
        ts = {}
        for f in STATE_FIELDS:
            a = np.ascontiguousarray(arrays[f], dtype=np.int32 if f == "id" else np.float64)
            ts[f] = torch.from_numpy(a).to(device)
        return cls(**ts)

    def copy_from_(self, arrays: dict, non_blocking: bool = False) -> None:
        for f in STATE_FIELDS:
            src = arrays[f]
            if isinstance(src, np.ndarray):
                src = torch.from_numpy(np.ascontiguousarray(src))
            getattr(self, f).copy_(src, non_blocking=non_blocking)

    def to_numpy(self) -> dict:
        return {f: getattr(self, f).cpu().numpy() for f in STATE_FIELDS}

    def clone(self) -> "DeviceState":
        return DeviceState(**{f: getattr(self, f).clone() for f in STATE_FIELDS})


def make_phys(radQ=0, SWQ=0, FLQ=0, Wz=0.0, Bstar=0.0, Rstar=0.0, rho=0.0, vsw_AUyr=1.0,
              Rmin=0.0, n_planets=1) -> abi.Phys:
    return abi.Phys(int(radQ), int(SWQ), int(FLQ), float(Wz), float(Bstar), float(Rstar),
                    float(rho), float(vsw_AUyr), float(Rmin), int(n_planets))


def make_view(dist, fov, PA, inc, longitude, xsize, ysize) -> abi.View:
    return abi.View(float(dist), float(fov), float(PA), float(inc), float(longitude),
                    int(xsize), int(ysize))


def _stream_handle(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _host(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data_as(C.c_void_p)


def probe_fma_peak(device: int = 0) -> tuple[float, float]:
    """Measured FP32 and FP64 FMA throughput (TFLOP/s) of the device."""
    lib = abi.load()
    a, b = C.c_double(), C.c_double()
    abi.check(lib.ddx_probe_fma_peak(device, C.byref(a), C.byref(b)), "ddx_probe_fma_peak")
    return a.value, b.value


class Engine:
    """One libddx context on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = abi.load()
        self.device = device
        h = C.c_void_p()
        abi.check(self.lib.ddx_create(C.byref(h), device), "ddx_create")
        self.ctx = h
        self.n_grid = 0
        self.n_wav = 0

    def close(self) -> None:
        if self.ctx:
            abi.check(self.lib.ddx_destroy(self.ctx), "ddx_destroy")
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- tables -------------------------------------------------------------------------
    def set_size_table(self, size, beta, betasw, q) -> None:
        s, ps = _host(size, np.float64)
        b, pb = _host(beta, np.float32)
        bs, pbs = _host(betasw, np.float32)
        qq, pq = _host(q, np.float32)
        abi.check(self.lib.ddx_set_size_table(self.ctx, len(s), ps, pb, pbs, pq), "ddx_set_size_table")
        self.n_grid = len(s)

    def set_optics(self, w, influx, Qabs, Qsca, Qpfunc, Td, Rmin, Rmax) -> None:
        n_wav = len(w)
        n_grid = Qabs.shape[0]
        n_theta = Qpfunc.shape[1]
        arrs = [_host(a, np.float64) for a in (w, influx, Qabs, Qsca, Qpfunc, Td)]
        abi.check(self.lib.ddx_set_optics(self.ctx, n_grid, n_wav, n_theta,
                                          *[p for _, p in arrs], float(Rmin), float(Rmax)),
                  "ddx_set_optics")
        self.n_wav = n_wav

    # -- dynamics -----------------------------------------------------------------------
    def step(self, st: DeviceState, n_grav: int, dt: float, phys: abi.Phys,
             precision: int = abi.DDX_PREC_FP64, mode: int = abi.DDX_MODE_FIXED,
             stream=None) -> None:
        self.evolve(st, n_grav, dt, 1, phys, precision, mode, stream)

    def evolve(self, st: DeviceState, n_grav: int, dt: float, n_steps: int, phys: abi.Phys,
               precision: int = abi.DDX_PREC_FP64, mode: int = abi.DDX_MODE_FIXED,
               stream=None) -> None:
        n_dust = st.n_all - n_grav
        abi.check(self.lib.ddx_evolve(self.ctx, C.byref(st._abi), n_grav, n_dust, float(dt),
                                      int(n_steps), C.byref(phys), precision, mode,
                                      C.c_void_p(_stream_handle(stream))), "ddx_evolve")

    def stage(self, which: str, st: DeviceState, n_grav: int, dt: float, phys: abi.Phys,
              precision: int = abi.DDX_PREC_FP64, mode: int = abi.DDX_MODE_FIXED, stream=None) -> None:
        """One of the reference's three step calls: 'massive_rk4', 'small_rk4' or
        'massive_final' (src/grid.cu:387-389)."""
        fn = getattr(self.lib, "ddx_" + which)
        abi.check(fn(self.ctx, C.byref(st._abi), n_grav, st.n_all - n_grav, float(dt), C.byref(phys),
                     precision, mode, C.c_void_p(_stream_handle(stream))), "ddx_" + which)

    def collide(self, st: DeviceState, i0: int, i1: int, h: float, cap: int | None = None,
                stream=None) -> torch.Tensor:
        """Collision pairs (m, 2) int32 on the device, ordered by (i, j): live tracers
        i < j of [i0, i1) with squared separation < h^2.  With cap=None the buffer is
        sized from the previous call's count (twice it, at least 4,096 pairs) and the call
        is repeated with room for all pairs when that was too small."""
        n = C.c_longlong(0)
        sh = C.c_void_p(_stream_handle(stream))
        fixed = cap is not None
        if not fixed:
            cap = max(4096, 2 * getattr(self, "last_pair_count", 0))
        while True:
            out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=st.x.device)
            abi.check(self.lib.ddx_collide(self.ctx, C.byref(st._abi), i0, i1, float(h),
                                           C.c_void_p(out.data_ptr()), cap, C.byref(n), sh), "ddx_collide")
            if fixed or n.value <= cap:
                break
            cap = n.value
        self.last_pair_count = n.value
        return out[:min(cap, n.value)]

    def det_step(self, st: DeviceState, n_grav: int, n_step: int, disk_Rin=(), blobs=(), stream=None) -> float:
        """Time step of a run with n_step steps per orbit (Grid::det_step): the shortest
        of the massive bodies' Kepler periods about the star, the disks' sqrt(Rin/m0) terms
        and the blobs' sqrt((a(1-ecc)-sigma)/m0) terms, times 2 pi / n_step.  blobs is a
        sequence of (a, ecc, sigma)."""
        rin = np.ascontiguousarray(disk_Rin, dtype=np.float64)
        bl = np.ascontiguousarray(np.reshape(blobs, (-1, 3)), dtype=np.float64)
        ba, be, bs = (np.ascontiguousarray(bl[:, k]) for k in range(3))
        dt = C.c_double(0.0)

        def ptr(a):
            return C.c_void_p(a.ctypes.data) if a.size else None
        abi.check(self.lib.ddx_det_step(self.ctx, C.byref(st._abi), int(n_grav), int(n_step), ptr(rin), rin.size,
                                        ptr(ba), ptr(be), ptr(bs), ba.size, C.byref(dt),
                                        C.c_void_p(_stream_handle(stream))), "ddx_det_step")
        return dt.value

    def dust_temp(self, w, influx, Qabs, dist, Rmax_AU, stream=None):
        """Grid::calculate_dust_temp on the GPU: (Td (n_grid, 100), Rmin, Rmax) in AU."""
        w = np.ascontiguousarray(w, np.float64)
        influx = np.ascontiguousarray(influx, np.float64)
        Qabs = np.ascontiguousarray(Qabs, np.float64)
        n_grid, n_wav = Qabs.shape
        Td = np.zeros((n_grid, abi.DDX_NR))
        rmin, rmax = C.c_double(0.0), C.c_double(float(Rmax_AU))
        abi.check(self.lib.ddx_dust_temp(self.ctx, n_grid, n_wav, C.c_void_p(w.ctypes.data),
                                         C.c_void_p(influx.ctypes.data), C.c_void_p(Qabs.ctypes.data), float(dist),
                                         C.byref(rmin), C.byref(rmax), C.c_void_p(Td.ctypes.data),
                                         C.c_void_p(_stream_handle(stream))), "ddx_dust_temp")
        return Td, rmin.value, rmax.value

    def dust_grid(self, w, influx, table: dict, n_grid: int, amin: float, amax: float, dmax: float, kqe: float,
                  radQ: int, SWQ: int, rho: float, dist: float, mstar: float, mloss: float, vsw: float,
                  stream=None) -> dict:
        """interpolate_dust_to_grid + calculate_beta on the GPU.  `table` holds the optical
        file's s, Qabs, Qsca, Qpfunc (formats.read_optical); returns the grid's s, q,
        Qabs, Qsca, Qpfunc, beta, betasw, Lum and betaswconst."""
        w = np.ascontiguousarray(w, np.float64)
        influx = np.ascontiguousarray(influx, np.float64)
        src = {k: np.ascontiguousarray(table[k], np.float64) for k in ("s", "Qabs", "Qsca", "Qpfunc")}
        nd, nt, nw = src["Qpfunc"].shape
        out = {"s": np.zeros(n_grid), "Qabs": np.zeros((n_grid, nw)), "Qsca": np.zeros((n_grid, nw)),
               "Qpfunc": np.zeros((n_grid, nt, nw)), "q": np.zeros(n_grid, np.float32),
               "beta": np.zeros(n_grid, np.float32), "betasw": np.zeros(n_grid, np.float32)}
        ptr = lambda a: a.ctypes.data
        ft = abi.OpticalTable(nd, nw, nt, *(ptr(src[k]) for k in ("s", "Qabs", "Qsca", "Qpfunc")))
        gt = abi.OpticalTable(n_grid, nw, nt, *(ptr(out[k]) for k in ("s", "Qabs", "Qsca", "Qpfunc")))
        gs = abi.GridSetup(int(n_grid), float(amin), float(amax), float(dmax), float(kqe), int(radQ), int(SWQ),
                           float(rho), float(dist), float(mstar), float(mloss), float(vsw))
        lum, bsc = C.c_double(), C.c_double()
        abi.check(self.lib.ddx_dust_grid(self.ctx, nw, C.c_void_p(ptr(w)), C.c_void_p(ptr(influx)), C.byref(ft),
                                         C.byref(gs), C.byref(gt), C.c_void_p(ptr(out["q"])),
                                         C.c_void_p(ptr(out["beta"])), C.c_void_p(ptr(out["betasw"])), C.byref(lum),
                                         C.byref(bsc), C.c_void_p(_stream_handle(stream))), "ddx_dust_grid")
        out["Lum"], out["betaswconst"] = lum.value, bsc.value
        return out

    def setup_device(self, p, dmin: float, dmax: float, beta, seed: int, stream=None) -> tuple:
        """ddx_setup_device: the initial system of parameter struct p (after
        formats.param_grid) drawn on this GPU; returns (DeviceState, run counts)."""
        from . import formats
        run = formats.setup_count(p, dmin, dmax)
        dev = torch.device("cuda", self.device)
        ts = {f: torch.empty(run.n_all, dtype=torch.int32 if f == "id" else torch.float64, device=dev)
              for f in STATE_FIELDS}
        st = DeviceState(**ts)
        beta = np.ascontiguousarray(beta, np.float32)
        abi.check(self.lib.ddx_setup_device(self.ctx, C.byref(p), float(dmin), float(dmax),
                                            C.c_void_p(beta.ctypes.data), int(seed) & (2 ** 64 - 1),
                                            C.byref(st._abi), run.n_all, C.byref(run),
                                            C.c_void_p(_stream_handle(stream))), "ddx_setup_device")
        return st, run

    def step_host(self, st: DeviceState, host_in: dict, host_out: dict, n_grav: int, dt: float, phys: abi.Phys,
                  precision: int = abi.DDX_PREC_MIXED, mode: int = abi.DDX_MODE_FIXED, stream=None) -> None:
        """ddx_step_host: one step of the state in host_in (CPU tensors or arrays, page-locked
        for overlap), staged through the device state st, results into host_out."""
        from .formats import HostState

        def hs(d):
            ptr = lambda t: t.data_ptr() if isinstance(t, torch.Tensor) else t.ctypes.data
            return HostState(*[ptr(d[f]) for f in ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")], st.n_all)

        hin, hout = hs(host_in), hs(host_out)
        abi.check(self.lib.ddx_step_host(self.ctx, C.byref(hin), C.byref(hout), C.byref(st._abi), n_grav,
                                         st.n_all - n_grav, float(dt), C.byref(phys), precision, mode,
                                         C.c_void_p(_stream_handle(stream))), "ddx_step_host")

    def run(self, st: DeviceState, n_grav: int, dt: float, phys: abi.Phys, view: abi.View, wj, cadence: dict,
            on_output, precision: int = abi.DDX_PREC_MIXED, mode: int = abi.DDX_MODE_FIXED, stream=None) -> dict:
        """ddx_run: Grid::evolve with its output cadence.  cadence holds t_write, t_fits,
        t_sed, t_end, time, tlastd, tlastf, tlasts, model_dt, initial_outputs; on_output(out)
        gets a dict per output (kind, time, the run values, and `data` (numpy copy) or
        `state` (dict of numpy copies)) and returns True to stop.  Returns the clock reached."""
        wj_a, pwj = _host(wj, np.int32)
        cad = abi.Cadence(**{k: float(cadence.get(k, 0.0)) for k in ("t_write", "t_fits", "t_sed", "t_end", "time",
                                                                      "tlastd", "tlastf", "tlasts", "model_dt")},
                          initial_outputs=int(cadence.get("initial_outputs", 0)))
        errors = []

        def cb(_user, o):
            try:
                o = o.contents
                d = {"kind": o.kind, "time": o.time, "model_dt": o.model_dt, "tlastd": o.tlastd,
                     "tlastf": o.tlastf, "tlasts": o.tlasts}
                if o.kind == abi.DDX_OUT_STATE:
                    hs = o.state.contents
                    n = hs.cap
                    d["state"] = {f: np.ctypeslib.as_array(getattr(hs, f), shape=(n,)).copy() for f in STATE_FIELDS}
                else:
                    d["data"] = np.ctypeslib.as_array(o.data, shape=(o.n,)).copy()
                return 1 if on_output(d) else 0
            except Exception as e:   # surfaced after the call
                errors.append(e)
                return 1

        fn = abi.OUTPUT_FN(cb)
        r = self.lib.ddx_run(self.ctx, C.byref(st._abi), n_grav, st.n_all - n_grav, float(dt), C.byref(phys),
                             precision, mode, C.byref(view), pwj, len(wj_a), C.byref(cad), fn, None,
                             C.c_void_p(_stream_handle(stream)))
        if errors:
            raise errors[0]
        abi.check(r, "ddx_run")
        return {k: getattr(cad, k) for k in ("time", "tlastd", "tlastf", "tlasts")}

    def set_near_radius(self, eta: float) -> None:
        """Mixed and compensated precision: planetesimals nearer to a body than eta times its
        largest |coordinate| take the FP64 pair force (0 turns that off, a negative eta
        restores the defaults of each precision)."""
        abi.check(self.lib.ddx_set_near_radius(self.ctx, C.c_double(eta)), "ddx_set_near_radius")

    def set_compensated_radius(self, eta: float) -> None:
        """DDX_PREC_COMPENSATED: spans of planetesimals nearer to a tracer than eta times its
        largest |coordinate| take the float-float pull (inf: every span)."""
        abi.check(self.lib.ddx_set_compensated_radius(self.ctx, C.c_double(eta)), "ddx_set_compensated_radius")

    def sync_status(self, stream=None) -> int:
        """Synchronise the stream; DDX_ERR_TIMEOUT (6) if a kernel of this context gave up a
        bounded device-side wait since the last call, else 0."""
        return self.lib.ddx_sync_status(self.ctx, C.c_void_p(_stream_handle(stream)))

    # -- flux ---------------------------------------------------------------------------
    def image(self, st: DeviceState, n_grav: int, view: abi.View, wj, out: torch.Tensor | None = None,
              precision: int = abi.DDX_PREC_FP64, stream=None) -> torch.Tensor:
        wj_a, pwj = _host(wj, np.int32)
        n_img = len(wj_a)
        npix = view.xsize * view.ysize
        if out is None:
            out = torch.empty((n_img, view.xsize, view.ysize), dtype=torch.float64, device=st.x.device)
        assert out.is_contiguous() and out.numel() == n_img * npix and out.dtype == torch.float64
        abi.check(self.lib.ddx_image(self.ctx, C.byref(st._abi), n_grav, st.n_all - n_grav,
                                     C.byref(view), pwj, n_img, C.c_void_p(out.data_ptr()),
                                     precision, C.c_void_p(_stream_handle(stream))), "ddx_image")
        return out

    def sed(self, st: DeviceState, n_grav: int, view: abi.View, out: torch.Tensor | None = None,
            precision: int = abi.DDX_PREC_FP64, mode: int = abi.DDX_MODE_FIXED,
            stream=None) -> torch.Tensor:
        if out is None:
            out = torch.empty(self.n_wav, dtype=torch.float64, device=st.x.device)
        abi.check(self.lib.ddx_sed(self.ctx, C.byref(st._abi), n_grav, st.n_all - n_grav,
                                   C.byref(view), C.c_void_p(out.data_ptr()), precision, mode,
                                   C.c_void_p(_stream_handle(stream))), "ddx_sed")
        return out

    def pixels(self, st: DeviceState, n_grav: int, view: abi.View):
        """Per-tracer pixel index ysize*x + y (-1 outside / no optics) and whether the
        exact reference sequence decided it."""
        n_dust = st.n_all - n_grav
        pix = torch.empty(max(n_dust, 1), dtype=torch.int32, device=st.x.device)
        ex = torch.empty(max(n_dust, 1), dtype=torch.int32, device=st.x.device)
        abi.check(self.lib.ddx_debug_pixels(self.ctx, C.byref(st._abi), n_grav, n_dust,
                                            C.byref(view), C.c_void_p(pix.data_ptr()),
                                            C.c_void_p(ex.data_ptr())), "ddx_debug_pixels")
        torch.cuda.synchronize()
        return pix[:n_dust], ex[:n_dust]
