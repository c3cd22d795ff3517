"""Seeded synthetic systems and optical tables for the DiskDyn hot path.

No public dataset is involved: every workload is generated here from a counter-based
Philox stream with a recorded seed, in the reference's units (AU, yr, mass*4*pi^2 in
Msun) and state layout (star, planets, gravitating bodies, then dust).

Orbital elements go to Cartesian coordinates with the reference's `coe2rv`
(src/functions.cu:6-46); planets are moved to the centre-of-mass frame like
`recalc_COM` (src/read_in.cu:344-375); size bins follow the mass grid of `detminmax`
(src/read_in.cu:268-342, ratio mgrid = 1.1) and the bin assignment of src/grid.cu:284;
beta follows the `calculate_beta` scaling 0.57 Q_pr (L/M) / (s[um] rho[g/cc])
(src/functions.cu:375) with Q_pr = 1, and beta_sw = betaswconst / s (src/functions.cu:349,381).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Reference constants (src/ddyn.cuh:17-38).
MEarth = 5.97e24
AU = 1.49598e11
MSun = 1.98892e30
RSun = 695700000.0
YEAR = 3.1556926e7
LIGHT_AU = 63239.6717367
CSPEED = 299792458.0
KBOLTZ = 1.3806503e-23
HPLANK = 6.626068e-34
PI = 3.14159265358979323846
GRAV = 4.0 * PI * PI
PC = 3.08567758149137e16
NR = 100
MGRID = 1.1
CD = 2

SEED = 20251203


def rng(seed: int, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=seed + 1000003 * stream))


def coe2rv(M, m, a, e, i, w, o, nu, beta=0.0):
    """Orbital elements -> position, velocity (src/functions.cu:6-46), vectorised.
    M, m are mass*4pi^2; angles in radians; returns x, y, z, vx, vy, vz."""
    a, e, i, w, o, nu = (np.asarray(v, dtype=np.float64) for v in (a, e, i, w, o, nu))
    p = a * (1.0 - e * e)
    mu = (M + m) * (1.0 - beta)
    xe = p * np.cos(nu) / (1.0 + e * np.cos(nu))
    ye = p * np.sin(nu) / (1.0 + e * np.cos(nu))
    ze = 0.0
    vxe = -np.sqrt(mu / p) * np.sin(nu)
    vye = np.sqrt(mu / p) * (e + np.cos(nu))
    vze = 0.0
    co, so, cw, sw, ci, si = np.cos(o), np.sin(o), np.cos(w), np.sin(w), np.cos(i), np.sin(i)
    r11 = co * cw - so * sw * ci
    r12 = -co * sw - so * cw * ci
    r13 = so * si
    r21 = so * cw + co * sw * ci
    r22 = -so * sw + co * cw * ci
    r23 = -co * si
    r31 = sw * si
    r32 = cw * si
    r33 = ci
    x = xe * r11 + ye * r12 + ze * r13
    y = xe * r21 + ye * r22 + ze * r23
    z = xe * r31 + ye * r32 + ze * r33
    vx = vxe * r11 + vye * r12 + vze * r13
    vy = vxe * r21 + vye * r22 + vze * r23
    vz = vxe * r31 + vye * r32 + vze * r33
    return x, y, z, vx, vy, vz


def rv2coe(M, m, x, y, z, vx, vy, vz, beta=0.0):
    """Cartesian -> (a, e, i) for bound, inclined orbits (src/functions.cu:48-101)."""
    mu = (M + m) * (1.0 - beta)
    R = np.sqrt(x * x + y * y + z * z)
    V = np.sqrt(vx * vx + vy * vy + vz * vz)
    hx = y * vz - z * vy
    hy = z * vx - x * vz
    hz = x * vy - y * vx
    H = np.sqrt(hx * hx + hy * hy + hz * hz)
    c1 = V * V - mu / R
    rv = x * vx + y * vy + z * vz
    ex = (c1 * x - rv * vx) / mu
    ey = (c1 * y - rv * vy) / mu
    ez = (c1 * z - rv * vz) / mu
    e = np.sqrt(ex * ex + ey * ey + ez * ez)
    sme = V * V * 0.5 - mu / R
    a = -mu / 2.0 / sme
    inc = np.arccos(hz / H)
    return a, e, inc


def recalc_com(px, py, pz, pvx, pvy, pvz, pm):
    """Centre-of-mass correction of star + planets (src/read_in.cu:344-375): positions
    shifted to the barycentre, the star given the momentum that cancels the planets'."""
    if len(pm) == 1:
        return
    Mtot = pm.sum()
    Xc = (pm * px).sum() / Mtot
    Yc = (pm * py).sum() / Mtot
    Zc = (pm * pz).sum() / Mtot
    px -= Xc
    py -= Yc
    pz -= Zc
    pvx[0] = -(pm[1:] * pvx[1:]).sum() / pm[0]
    pvy[0] = -(pm[1:] * pvy[1:]).sum() / pm[0]
    pvz[0] = -(pm[1:] * pvz[1:]).sum() / pm[0]


def planck(T, w):
    """B_lambda(T) in W m^-2 m^-1 sr^-1 (src/functions.cu:390-397)."""
    with np.errstate(over="ignore"):
        return (2 * HPLANK * CSPEED * CSPEED) / (w ** 5 * (np.exp(HPLANK * CSPEED / (w * KBOLTZ * T)) - 1))


@dataclass
class System:
    """A synthetic workload: host state arrays plus the constants of its step."""
    name: str
    n_grav: int
    state: dict
    dt: float
    n_steps: int
    phys: dict
    size_table: dict                      # size, beta, betasw, q (n_grid)
    optics: dict | None = None
    view: dict | None = None
    image_wj: list | None = None
    meta: dict = field(default_factory=dict)

    @property
    def n_dust(self) -> int:
        return len(self.state["x"]) - self.n_grav


def _pack(px, py, pz, pvx, pvy, pvz, pm, dx, dy, dz, dvx, dvy, dvz, dm, dN, did):
    cat = lambda a, b: np.concatenate([np.asarray(a, np.float64), np.asarray(b, np.float64)])
    ng = len(pm)
    return {
        "x": cat(px, dx), "y": cat(py, dy), "z": cat(pz, dz),
        "vx": cat(pvx, dvx), "vy": cat(pvy, dvy), "vz": cat(pvz, dvz),
        "m": cat(pm, dm), "N": cat(np.ones(ng), dN),
        "id": np.concatenate([np.full(ng, -1, np.int32), np.asarray(did, np.int32)]),
    }


def _empty_size_table(n=1):
    return {"size": np.full(n, 1e-6), "beta": np.zeros(n, np.float32),
            "betasw": np.zeros(n, np.float32), "q": np.zeros(n, np.float32)}


def solar_like(n_dust: int = 16384, seed: int = SEED, with_ids: bool = False, n_bins: int = 64) -> System:
    """1 Msun star, 8 planets (1.7e-7..9.5e-4 Msun, a log-spaced 0.4-30 AU, e~U(0,0.1),
    i~U(0,3 deg)) and n_dust massless tracers with a~U(30,50) AU, e~U(0,0.1),
    i~U(0,5 deg), uniform angles; beta = 0; fixed dt = 0.05 yr, 1000 steps."""
    g = rng(seed, 1)
    M = 1.0 * GRAV
    n_pl = 8
    pm = np.concatenate([[M], np.logspace(np.log10(1.7e-7), np.log10(9.5e-4), n_pl) * GRAV])
    a = np.logspace(np.log10(0.4), np.log10(30.0), n_pl)
    e = g.uniform(0.0, 0.1, n_pl)
    inc = np.deg2rad(g.uniform(0.0, 3.0, n_pl))
    w, o, nu = (g.uniform(0.0, 2 * PI, n_pl) for _ in range(3))
    x, y, z, vx, vy, vz = coe2rv(M, pm[1:], a, e, inc, w, o, nu)
    px, py, pz = (np.concatenate([[0.0], v]) for v in (x, y, z))
    pvx, pvy, pvz = (np.concatenate([[0.0], v]) for v in (vx, vy, vz))
    recalc_com(px, py, pz, pvx, pvy, pvz, pm)
    gd = rng(seed, 2)
    a = gd.uniform(30.0, 50.0, n_dust)
    e = gd.uniform(0.0, 0.1, n_dust)
    inc = np.deg2rad(gd.uniform(0.0, 5.0, n_dust))
    w, o, nu = (gd.uniform(0.0, 2 * PI, n_dust) for _ in range(3))
    dx, dy, dz, dvx, dvy, dvz = coe2rv(M, 0.0, a, e, inc, w, o, nu)
    did = gd.integers(0, n_bins, n_dust) if with_ids else np.full(n_dust, -1)
    state = _pack(px, py, pz, pvx, pvy, pvz, pm, dx, dy, dz, dvx, dvy, dvz,
                  np.zeros(n_dust), np.ones(n_dust), did)
    phys = dict(radQ=0, SWQ=0, FLQ=0, Wz=0.0, Bstar=0.0, Rstar=RSun / AU, rho=2700.0,
                vsw_AUyr=400e3 * YEAR / AU, Rmin=0.05, n_planets=n_pl + 1)
    return System("solar_like", n_pl + 1, state, 0.05, 1000, phys, _empty_size_table(n_bins),
                  meta={"seed": seed})


def _mass_grid(amin, amax, rho):
    """Global dust mass grid of detminmax (src/read_in.cu:335-340); sizes in m, rho kg/m^3."""
    kappa = 4.0 * PI * rho / 3.0
    mmin = kappa * amin ** 3
    mmax = kappa * amax ** 3
    n_grid = int(math.log(mmax / mmin) / math.log(MGRID) + 1.0)
    f = math.log(mmax / mmin) / (n_grid - 1.0)
    return mmin, mmax, n_grid, f


def dusty_ring(n_dust: int = 1048576, n_plsml: int = 4096, seed: int = SEED, n_steps: int = 2000) -> System:
    """1.5 Msun star at L = 8.7 Lsun; planets of 1e-3 and 3e-4 Msun on circular coplanar
    orbits at 20 and 60 AU; n_plsml gravitating planetesimals (mass log-uniform 1e-10 to
    1e-8 Msun, a~U(120,140) AU, e~U(0,0.05), i~U(0,3 deg)); n_dust grains in the same ring
    with radius log-uniform 1-1000 um, density 2.7 g/cc, beta from L/M and radius; radiation
    pressure, PR drag and stellar-wind drag on (Mdot = 2e-14 Msun/yr, v_sw = 400 km/s);
    dt = one 300th of the orbital period at 120 AU."""
    Ms, L, rho = 1.5, 8.7, 2700.0
    M = Ms * GRAV
    g = rng(seed, 11)
    pm = np.array([M, 1e-3 * GRAV, 3e-4 * GRAV])
    ap = np.array([20.0, 60.0])
    nu_p = g.uniform(0.0, 2 * PI, 2)
    x, y, z, vx, vy, vz = coe2rv(M, pm[1:], ap, np.zeros(2), np.zeros(2), np.zeros(2), np.zeros(2), nu_p)
    px, py, pz = (np.concatenate([[0.0], v]) for v in (x, y, z))
    pvx, pvy, pvz = (np.concatenate([[0.0], v]) for v in (vx, vy, vz))
    recalc_com(px, py, pz, pvx, pvy, pvz, pm)
    # gravitating planetesimals
    gp = rng(seed, 12)
    mm = 10 ** gp.uniform(-10.0, -8.0, n_plsml) * GRAV
    a = gp.uniform(120.0, 140.0, n_plsml)
    e = gp.uniform(0.0, 0.05, n_plsml)
    inc = np.deg2rad(gp.uniform(0.0, 3.0, n_plsml))
    w, o, nu = (gp.uniform(0.0, 2 * PI, n_plsml) for _ in range(3))
    bx, by, bz, bvx, bvy, bvz = coe2rv(M, mm, a, e, inc, w, o, nu)
    # size bins
    mmin, mmax, n_grid, f = _mass_grid(1e-6, 1e-3, rho)
    mbin = mmin * np.exp(np.arange(n_grid) * f)
    sbin = (mbin * 3.0 / 4.0 / PI / rho) ** (1.0 / 3.0)
    beta = (0.57 * 1.0 * (L / Ms) / (sbin * 1e6) / (rho / 1000.0)).astype(np.float32)
    mloss, vsw = 2e-14, 400e3
    betaswconst = 3.0 * mloss * CD * MSun * YEAR * vsw / 32.0 / PI / M / rho / AU / AU / AU
    betasw = (betaswconst / sbin).astype(np.float32)
    # grains
    gd = rng(seed, 13)
    s = 10 ** gd.uniform(-6.0, -3.0, n_dust)
    mg = 4.0 / 3.0 * PI * rho * s ** 3
    did = np.clip(np.rint(np.log(mg / mmin) / f).astype(np.int64), 0, n_grid - 1)
    bg = beta[did].astype(np.float64) + betasw[did].astype(np.float64)
    bg = np.where(bg >= 0.5, 0.0, bg)  # src/functions.cu:186
    dm = mbin[did] * GRAV / MSun
    a = gd.uniform(120.0, 140.0, n_dust)
    e = gd.uniform(0.0, 0.05, n_dust)
    inc = np.deg2rad(gd.uniform(0.0, 3.0, n_dust))
    w, o, nu = (gd.uniform(0.0, 2 * PI, n_dust) for _ in range(3))
    dx, dy, dz, dvx, dvy, dvz = coe2rv(M, dm, a, e, inc, w, o, nu, bg)
    state = _pack(np.concatenate([px, bx]), np.concatenate([py, by]), np.concatenate([pz, bz]),
                  np.concatenate([pvx, bvx]), np.concatenate([pvy, bvy]), np.concatenate([pvz, bvz]),
                  np.concatenate([pm, mm]), dx, dy, dz, dvx, dvy, dvz, dm, np.ones(n_dust), did)
    dt = math.sqrt(120.0 ** 3 / Ms) / 300.0
    phys = dict(radQ=1, SWQ=1, FLQ=0, Wz=365.2422 / 25.0, Bstar=0.0, Rstar=2.0 * RSun / AU,
                rho=rho, vsw_AUyr=vsw * YEAR / AU, Rmin=0.5, n_planets=3)
    size_table = {"size": sbin, "beta": beta, "betasw": betasw,
                  "q": np.zeros(n_grid, np.float32)}
    return System("dusty_ring", 3 + n_plsml, state, dt, n_steps, phys, size_table,
                  meta={"seed": seed, "L": L, "Mstar": Ms, "n_grid": n_grid, "mass_grid_f": f,
                        "mloss": mloss, "vsw_ms": vsw})


def hg_optics(n_grid=64, n_theta=181, n_wav=200, wmin=0.5e-6, wmax=850e-6, Teff=5770.0,
              Rstar=RSun, dist=10 * PC, L=1.0, Rmin=0.1, Rmax=100.0, smin=1e-6, smax=1e-3):
    """Synthetic optics standing in for a Mie table: Henyey-Greenstein phase functions on
    the reference's uniform cos(theta) grid with g rising linearly 0.1 -> 0.9 over the size
    bins, Q_abs = Q_sca = 1, a blackbody star seen from `dist`, and grains at
    T = 278.3 L^(1/4) (r/AU)^(-1/2) K on the reference's nR = 100 log-radius grid."""
    w = np.logspace(np.log10(wmin), np.log10(wmax), n_wav)
    mu = np.arange(n_theta) * 2.0 / (n_theta - 1) - 1.0
    gg = np.linspace(0.1, 0.9, n_grid)
    P = (1 - gg[:, None] ** 2) / (4 * PI * (1 + gg[:, None] ** 2 - 2 * gg[:, None] * mu[None, :]) ** 1.5)
    Qp = np.repeat(P[:, :, None], n_wav, axis=2)
    Qabs = np.ones((n_grid, n_wav))
    Qsca = np.ones((n_grid, n_wav))
    influx = PI * planck(Teff, w) * (Rstar / dist) ** 2
    R = Rmin * np.exp(np.log(Rmax / Rmin) * np.arange(NR) / (NR - 1.0))
    Td = np.repeat((278.3 * L ** 0.25 * R ** -0.5)[None, :], n_grid, axis=0)
    size = np.logspace(np.log10(smin), np.log10(smax), n_grid)
    return {"w": w, "in": influx, "Qabs": Qabs, "Qsca": Qsca, "Qpfunc": Qp, "Td": Td,
            "Rmin": Rmin, "Rmax": Rmax, "size": size, "g": gg}


def mie_table(n_size=40, n_wav=200, n_theta=181, smin=1e-7, smax=1e-4, Teff=9000.0, Rstar=1.8 * RSun,
              dist=7.7 * PC, seed=SEED):
    """An optical table file's contents at the size a Mie run gives (n_size radii from smin
    to smax, n_wav wavelengths from 0.1 um to 1 mm, n_theta angles): Q_abs and Q_sca smooth in
    the size parameter x = 2 pi s / lambda, Henyey-Greenstein phase functions with g rising
    with x, every value positive; with a blackbody star seen from `dist`.
    Returns (w, in, {"s", "Qabs", "Qsca", "Qpfunc"})."""
    rng = np.random.default_rng(seed)
    s = smin * np.exp(np.log(smax / smin) * np.arange(n_size) / (n_size - 1))
    w = 1e-7 * np.exp(np.log(1e4) * np.arange(n_wav) / (n_wav - 1))
    x = 2 * PI * s[:, None] / w[None, :]
    Qabs = x / (1 + x) * (1 + 0.1 * rng.random((n_size, n_wav))) + 1e-5
    Qsca = 2 * x ** 4 / (1 + x ** 4) + 1e-8
    mu = np.arange(n_theta) * 2.0 / (n_theta - 1) - 1.0
    gg = (0.85 * x / (1 + x))[:, None, :]
    Qp = Qsca[:, None, :] * (1 - gg ** 2) / (1 + gg ** 2 - 2 * gg * mu[None, :, None]) ** 1.5
    influx = PI * planck(Teff, w) * (Rstar / dist) ** 2
    return w, influx, {"s": s, "Qabs": Qabs, "Qsca": Qsca, "Qpfunc": Qp}


def setup_param_text(n_grains: int = 16777216, n_gravitating: int = 4096) -> str:
    """A parameter file (the reference's format) of an A-star debris system whose set-up
    makes about n_grains grain tracers and n_gravitating gravitating bodies: a planet, a
    narrow belt (Fomalhaut-like, 70% of both), a wide halo disk and a collisional blob."""
    ng = [int(n_gravitating * f) for f in (0.7, 0.3)]
    # tracers per mass bin x bins: the set-up rounds Nsmall / Ngrid, so ask per disk
    ns = [int(n_grains * f) for f in (0.7, 0.25, 0.05)]
    return "\n".join([
        "# A-star debris system for set-up timing", "1", "0", "no 100", "1000.0 100.0 500.0", "2000", "300",
        "1.92 A3V 8590 1.84 1.0 25.0 1.0e-13 500.0", "7.7 400.0 0.0 65.6 0.0 1024 1024", "0.55 24.0 70.0",
        "Library", "yes yes no", "begin_planets", "0.0 115.0 0.12 0.0 0.0 0.0 3.0e-6", "end_planets",
        "3.3 optical/astrosil.dat 27.5", "begin_disks",
        f"130.0 145.0 0.03 0.1 10.0 0.3 3.65 3.0 0.0 {ng[0]} {ns[0]}",
        f"30.0 200.0 0.15 0.05 1.0 0.3 3.5 0.3 -1.0 {ng[1]} {ns[1]}", "end_disks", "begin_blobs",
        f"140.0 0.1 1.0 30.0 45.0 90.0 1.0 0.5 3.65 0.01 0 {ns[2]} Collision 5.0", "end_blobs", "synthetic", ""])


def ring_imaging(s: System, xsize=512, ysize=512) -> System:
    """Attach optics and a view to a `dusty_ring` system: HG tables on its grains' size
    bins, grey grains at T = 278.3 L^(1/4) (r/AU)^(-1/2) K, a 7500 K star of 2 Rsun at
    10 pc; an image 300 AU across at 30 deg inclination, at 1.25 um (scattered light) and
    100 um (thermal)."""
    n_grid = len(s.size_table["size"])
    opt = hg_optics(n_grid=n_grid, n_wav=200, dist=10 * PC, L=8.7, Rmin=0.1, Rmax=400.0,
                    Teff=7500.0, Rstar=2.0 * RSun, smin=s.size_table["size"][0],
                    smax=s.size_table["size"][-1])
    opt["size"] = s.size_table["size"]
    w = opt["w"]
    s.optics = opt
    s.view = dict(dist=10 * PC, fov=300.0, PA=0.0, inc=np.deg2rad(30.0), longitude=0.0,
                  xsize=xsize, ysize=ysize)
    s.image_wj = [int(np.argmin(abs(w - 1.25e-6))), int(np.argmin(abs(w - 100e-6)))]
    return s


def imaging(n_dust: int = 4194304, seed: int = SEED, xsize=1024, ysize=1024, n_img=10) -> System:
    """n_dust tracers from the solar-like dust distribution (ids uniform over 64 bins,
    N = 1e15 grains each), a 1024x1024 image at 30 deg inclination, PA 0, longitude 0,
    10 pc, FOV 120 AU, synthetic HG optics (64 x 181 x 200), 10 image wavelengths
    log-spaced over the table."""
    sysm = solar_like(n_dust=n_dust, seed=seed, with_ids=True, n_bins=64)
    sysm.state["N"][sysm.n_grav:] = 1e15
    opt = hg_optics()
    sysm.optics = opt
    sysm.size_table = {"size": opt["size"], "beta": np.zeros(64, np.float32),
                       "betasw": np.zeros(64, np.float32), "q": np.zeros(64, np.float32)}
    sysm.view = dict(dist=10 * PC, fov=120.0, PA=0.0, inc=np.deg2rad(30.0), longitude=0.0,
                     xsize=xsize, ysize=ysize)
    sysm.image_wj = [int(round(k)) for k in np.linspace(0, len(opt["w"]) - 2, n_img)]
    sysm.name = "imaging"
    return sysm
