"""Known-answer checks of the CPU oracle (the reference has no tests of its own): Kepler
closure, energy conservation, the beta = 0.5 escape threshold, coe2rv/rv2coe round trip,
the HG normalisation, a point source's pixel and a blackbody SED."""
import math

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import synth

PHYS0 = dict(radQ=0, SWQ=0, FLQ=0, Wz=0.0, Bstar=0.0, Rstar=0.0, rho=2700.0, vsw_AUyr=84.0, Rmin=0.01)
TAB0 = {"size": np.array([1e-6]), "beta": np.zeros(1, np.float32), "betasw": np.zeros(1, np.float32),
        "q": np.zeros(1, np.float32)}


def two_body(a=1.0, mp=1e-3):
    M = synth.GRAV
    m = mp * synth.GRAV
    x, y, z, vx, vy, vz = synth.coe2rv(M, m, a, 0.0, 0.0, 0.0, 0.0, 0.0)
    px = np.array([0.0, float(x)]); py = np.array([0.0, float(y)]); pz = np.zeros(2)
    pvx = np.array([0.0, float(vx)]); pvy = np.array([0.0, float(vy)]); pvz = np.zeros(2)
    pm = np.array([M, m])
    synth.recalc_com(px, py, pz, pvx, pvy, pvz, pm)
    return {"x": px, "y": py, "z": pz, "vx": pvx, "vy": pvy, "vz": pvz, "m": pm,
            "N": np.ones(2), "id": np.full(2, -1, np.int32)}


def rel_period(st):
    # recalc_COM (src/read_in.cu:344-375) gives only the star the balancing momentum, so
    # the relative orbit is not exactly the one coe2rv drew; take its own period.
    mu = st["m"].sum()
    rx, ry = st["x"][1] - st["x"][0], st["y"][1] - st["y"][0]
    vx, vy = st["vx"][1] - st["vx"][0], st["vy"][1] - st["vy"][0]
    a = 1.0 / (2.0 / math.hypot(rx, ry) - (vx * vx + vy * vy) / mu)
    return 2 * math.pi * math.sqrt(a ** 3 / mu)


def test_kepler_orbit_closes_after_one_period():
    st0 = two_body()
    P = rel_period(st0)
    n = 400
    st = oc.step(st0, 2, P / n, TAB0, PHYS0, n_steps=n)
    dx = st["x"][1] - st["x"][0] - (st0["x"][1] - st0["x"][0])
    dy = st["y"][1] - st["y"][0] - (st0["y"][1] - st0["y"][0])
    assert math.hypot(dx, dy) < 1e-8  # RK4 error ~ (2 pi / n)^4 per orbit


def test_rk4_error_scales_as_dt_to_the_fourth():
    st0 = two_body()
    P = rel_period(st0)
    errs = []
    for n in (100, 200):
        st = oc.step(st0, 2, P / n, TAB0, PHYS0, n_steps=n)
        errs.append(math.hypot(st["x"][1] - st["x"][0] - (st0["x"][1] - st0["x"][0]),
                               st["y"][1] - st["y"][0] - (st0["y"][1] - st0["y"][0])))
    assert 10 < errs[0] / errs[1] < 40   # 2^4 = 16 (2^5 for the phase error of a circle)


def test_massive_energy_conserved():
    s = synth.solar_like(n_dust=0)
    def energy(st):
        m = st["m"][:9]; x, y, z = st["x"][:9], st["y"][:9], st["z"][:9]
        K = 0.5 * (m * (st["vx"][:9] ** 2 + st["vy"][:9] ** 2 + st["vz"][:9] ** 2)).sum() / synth.GRAV
        U = 0.0
        for i in range(9):
            for j in range(i + 1, 9):
                U -= m[i] * m[j] / math.sqrt((x[i] - x[j]) ** 2 + (y[i] - y[j]) ** 2 + (z[i] - z[j]) ** 2) / synth.GRAV
        return K + U
    E0 = energy(s.state)
    st = oc.step(s.state, 9, 0.001, s.size_table, s.phys, n_steps=1000)
    assert abs(energy(st) - E0) / abs(E0) < 1e-9


@pytest.mark.parametrize("beta,bound", [(0.3, True), (0.6, False)])
def test_beta_half_escape_threshold(beta, bound):
    # A grain released on the circular velocity of a parent body stays bound for
    # beta < 0.5 and escapes for beta > 0.5 (radiation pressure only, no drag terms).
    M = synth.GRAV
    x, y, z, vx, vy, vz = synth.coe2rv(M, 0.0, 10.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    st = {"x": np.array([0.0, x]), "y": np.array([0.0, y]), "z": np.zeros(2),
          "vx": np.array([0.0, vx]), "vy": np.array([0.0, vy]), "vz": np.zeros(2),
          "m": np.array([M, 0.0]), "N": np.ones(2), "id": np.array([-1, 0], np.int32)}
    tab = dict(TAB0, beta=np.array([beta], np.float32))
    phys = dict(PHYS0, radQ=1, Rmin=0.01)
    P = 2 * math.pi * math.sqrt(1000.0)
    out = oc.step(st, 1, P / 400, tab, phys, n_steps=800)
    r = math.hypot(out["x"][1], out["y"][1])
    v2 = out["vx"][1] ** 2 + out["vy"][1] ** 2
    energy = 0.5 * v2 - (1 - beta) * M / r
    assert (energy < 0) == bound


def test_coe2rv_rv2coe_round_trip():
    g = synth.rng(7)
    n = 200
    a = g.uniform(0.5, 100, n); e = g.uniform(0.0, 0.9, n); i = g.uniform(0.05, 3.0, n)
    w, o, nu = (g.uniform(0, 2 * math.pi, n) for _ in range(3))
    M = 1.3 * synth.GRAV
    x, y, z, vx, vy, vz = synth.coe2rv(M, 0.0, a, e, i, w, o, nu)
    a2, e2, i2 = synth.rv2coe(M, 0.0, x, y, z, vx, vy, vz)
    np.testing.assert_allclose(a2, a, rtol=1e-10)
    np.testing.assert_allclose(e2, e, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(i2, i, rtol=1e-10)


def test_hg_phase_tables_are_normalised():
    o = synth.hg_optics(n_grid=8, n_wav=4)
    mu = np.arange(181) * 2.0 / 180 - 1.0
    fine = np.linspace(-1.0, 1.0, 2_000_001)
    for k in range(8):
        g = o["g"][k]
        hg = lambda m: (1 - g * g) / (4 * math.pi * (1 + g * g - 2 * g * m) ** 1.5)
        np.testing.assert_allclose(o["Qpfunc"][k, :, 0], hg(mu), rtol=1e-14)
        assert abs(2 * math.pi * np.trapezoid(hg(fine), fine) - 1.0) < 1e-6


def _single_tracer(x, y, z, ident=0, N=1.0):
    return {"x": np.array([0.0, x]), "y": np.array([0.0, y]), "z": np.array([0.0, z]),
            "vx": np.zeros(2), "vy": np.zeros(2), "vz": np.zeros(2), "m": np.array([synth.GRAV, 0.0]),
            "N": np.array([1.0, N]), "id": np.array([-1, ident], np.int32)}


def test_point_source_lands_in_hand_computed_pixel():
    o = synth.hg_optics(n_grid=2, n_wav=8)
    view = dict(dist=10 * synth.PC, fov=100.0, PA=0.0, inc=0.0, longitude=0.0, xsize=100, ysize=80)
    # face-on, no rotation: pixel = floor((coord + FOV/2 * size/max)/psca), psca = 1 AU
    st = _single_tracer(12.3, -7.6, 0.0)
    F, pix = oc.image(st, 1, o, o["size"], view, [3])
    xim, yim = math.floor(12.3 + 50.0), math.floor(-7.6 + 40.0)
    assert pix[0] == 80 * xim + yim
    assert F[0, xim, yim] > 0 and np.count_nonzero(F) == 1


def test_blackbody_sed_of_uniform_temperature_grains():
    # Qsca = 0, Qabs = 1, T = 100 K everywhere: F_lambda = N pi B(T) s^2 / d^2 in Jy.
    o = synth.hg_optics(n_grid=1, n_wav=50, smin=1e-5, smax=1e-5)
    o["Qsca"][:] = 0.0
    o["Td"][:] = 100.0
    view = dict(dist=10 * synth.PC, fov=100.0, PA=0.0, inc=0.3, longitude=0.0, xsize=64, ysize=64)
    st = _single_tracer(20.0, 5.0, 1.0, N=1e10)
    F = oc.sed(st, 1, o, o["size"], view)
    w = o["w"]
    expect = 1e10 * synth.PI * synth.planck(100.0, w) * 1e-10 / view["dist"] ** 2 * 1e26 * w * w / synth.CSPEED
    np.testing.assert_allclose(F, expect, rtol=1e-12)


def test_dust_temperature_table_follows_equilibrium_scaling():
    # Grey grains (Qabs = 1) around a 5770 K star at 10 pc: T ~ 278 K (r/AU)^-1/2.
    o = synth.hg_optics(n_grid=2, n_wav=400, wmin=0.1e-6, wmax=3000e-6)
    Td, Rmin, Rmax = oc.dust_temp(o["w"], o["in"], o["Qabs"], 10 * synth.PC, 50.0)
    assert Rmax == pytest.approx(100.0)
    R = Rmin * np.exp(np.log(Rmax / Rmin) * np.arange(100) / 99.0)
    k = np.searchsorted(R, 1.0)
    assert Td[0, k] * math.sqrt(R[k]) == pytest.approx(278.6, rel=0.02)
    assert Td[0, 0] == pytest.approx(2000.0, rel=0.01)   # Rmin is the sublimation radius


def test_det_step_is_the_shortest_kepler_period_over_n_step():
    # Grid::det_step: 2 pi sqrt(r^3 / (m0 + mi)) / n_step with masses carrying 4 pi^2 is
    # the orbital period in years over n_step; the innermost body sets it
    st = two_body(a=1.0, mp=0.0)
    st = {k: np.concatenate([v, v[1:]]) for k, v in st.items()}
    st["x"][2] = 4.0                                    # a second body at 4 AU
    dt = oc.det_step(st, 3, 100)
    assert dt == pytest.approx(0.01, rel=1e-15)
    # disks and blobs enter as 2 pi sqrt(R / m0) / n_step, the reference's expression
    assert oc.det_step(st, 3, 100, disk_Rin=[0.5]) == pytest.approx(2 * math.pi * math.sqrt(0.5 / synth.GRAV) / 100,
                                                                    rel=1e-15)
    assert oc.det_step(st, 3, 100, blobs=[(2.0, 0.5, 0.5)]) == pytest.approx(
        2 * math.pi * math.sqrt(0.5 / synth.GRAV) / 100, rel=1e-15)
    assert oc.det_step(st, 1, 100) == 1e137           # a lone star, no disk: the initial value
