"""RK4 step on the GPU through the C ABI, against the CPU oracle and the reference's own
kernels (compiled unmodified for sm_103a).

Tolerances: the FP64 path differs from the oracle only by rounding (rsqrt instead of
m/RR/sqrt(RR), FMA contraction, massive-set summation order), so positions agree to
1e-13 relative after one step and 1e-11 after 20; the reference-arithmetic dust path is
bit-identical to the reference kernel when the massive stage positions are identical
(star-only systems).  The mixed path (star and planets FP64, planetesimals FP32) is
checked against FP64 at 1e-13 relative (median) after 20 steps.
"""
import numpy as np
import pytest
import torch

import oracle.cpu as oc
from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_phys

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz")


def run_gpu(engine, sysm, n_steps=1, precision=abi.DDX_PREC_FP64, mode=abi.DDX_MODE_FIXED, state=None):
    st = DeviceState.from_numpy(state if state is not None else sysm.state)
    engine.set_size_table(**sysm.size_table)
    engine.evolve(st, sysm.n_grav, sysm.dt, n_steps, make_phys(**sysm.phys), precision, mode)
    torch.cuda.synchronize()
    return st.to_numpy()


def rel_err(a, b, sl=slice(None)):
    pa = np.stack([a[f][sl] for f in ("x", "y", "z")])
    pb = np.stack([b[f][sl] for f in ("x", "y", "z")])
    return np.linalg.norm(pa - pb, axis=0) / np.linalg.norm(pb, axis=0)


def small_ring(n_dust=4096, n_plsml=256, seed=5):
    return synth.dusty_ring(n_dust=n_dust, n_plsml=n_plsml, seed=seed, n_steps=20)


@pytest.mark.parametrize("mode", [abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE])
def test_fp64_one_step_matches_oracle_solar(engine, mode):
    s = synth.solar_like(n_dust=4096)
    g = run_gpu(engine, s, 1, abi.DDX_PREC_FP64, mode)
    o = oc.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 1, ref_mode=mode == abi.DDX_MODE_REFERENCE)
    assert rel_err(g, o).max() < 1e-13
    np.testing.assert_array_equal(g["N"], o["N"])


@pytest.mark.parametrize("mode", [abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE])
def test_fp64_twenty_steps_match_oracle_ring(engine, mode):
    s = small_ring()
    g = run_gpu(engine, s, 20, abi.DDX_PREC_FP64, mode)
    o = oc.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 20, ref_mode=mode == abi.DDX_MODE_REFERENCE)
    alive = o["N"] != 0
    np.testing.assert_array_equal(g["N"] != 0, alive)
    assert rel_err(g, o, slice(0, s.n_grav)).max() < 1e-11
    e = rel_err(g, o)[s.n_grav:][alive[s.n_grav:]]
    assert np.median(e) < 1e-13 and e.max() < 1e-9


def test_dust_bit_identical_to_reference_kernel_star_only(engine, refk):
    # n_grav = 1: the reference runs no massive stage (src/grid.cu:698), so the dust kernel
    # sees identical inputs; radiation pressure, PR + wind drag and the Lorentz force on.
    s = small_ring(n_dust=8192, n_plsml=0)
    st = {k: v.copy() for k, v in s.state.items()}
    for k in st:
        st[k] = np.concatenate([st[k][:1], st[k][s.n_grav:]])
    st["x"][0] = st["y"][0] = st["z"][0] = 0.0
    st["vx"][0] = st["vy"][0] = st["vz"][0] = 0.0
    sysm = synth.System("star_only", 1, st, s.dt, 5, dict(s.phys, FLQ=1, Bstar=5e-20, Wz=14.6, n_planets=1),
                        dict(s.size_table, q=np.linspace(1e-3, 2e-3, len(s.size_table["q"])).astype(np.float32)))
    g = run_gpu(engine, sysm, 5, abi.DDX_PREC_FP64, abi.DDX_MODE_REFERENCE)
    r = refk.step(sysm.state, 1, sysm.dt, sysm.size_table, sysm.phys, 5)
    for f in FIELDS + ("N",):
        np.testing.assert_array_equal(g[f], r[f], err_msg=f)


def test_step_matches_reference_kernel_with_massive_set(engine, refk):
    s = small_ring(n_dust=4096, n_plsml=64)
    g = run_gpu(engine, s, 10, abi.DDX_PREC_FP64, abi.DDX_MODE_REFERENCE)
    r = refk.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 10)
    np.testing.assert_array_equal(g["N"] != 0, r["N"] != 0)
    assert rel_err(g, r, slice(0, s.n_grav)).max() < 1e-12
    alive = r["N"][s.n_grav:] != 0
    assert rel_err(g, r)[s.n_grav:][alive].max() < 1e-10


def test_oracle_matches_reference_kernel(refk):
    """Pins the oracle: it agrees with the reference's own kernels on the same GPU."""
    s = small_ring(n_dust=2048, n_plsml=32)
    o = oc.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 5, ref_mode=True)
    r = refk.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 5)
    np.testing.assert_array_equal(o["N"] != 0, r["N"] != 0)
    alive = r["N"] != 0
    assert rel_err(o, r)[alive].max() < 1e-11


def test_mixed_precision_close_to_fp64(engine):
    # star and planets in FP64, planetesimals in FP32 (n_planets = 3)
    s = small_ring(n_dust=16384, n_plsml=512)
    f = run_gpu(engine, s, 20, abi.DDX_PREC_FP64)
    m = run_gpu(engine, s, 20, abi.DDX_PREC_MIXED)
    alive = (f["N"] != 0) & (m["N"] != 0)
    e = rel_err(m, f)[alive]
    assert np.median(e) < 1e-13
    assert np.quantile(e, 0.99) < 1e-12
    assert rel_err(m, f, slice(0, s.n_grav)).max() < 1e-12


def test_mixed_planets_in_fp64_cut_the_error(engine):
    """With only the star in FP64 the planets' pull (1e-3 of the star's) carries FP32
    rounding; n_planets = 3 moves it to FP64 and the error against FP64 drops by orders
    of magnitude."""
    s = small_ring(n_dust=16384, n_plsml=512)
    f = run_gpu(engine, s, 20, abi.DDX_PREC_FP64)
    errs = {}
    for npl in (1, 3):
        sp = synth.System(s.name, s.n_grav, s.state, s.dt, 20, dict(s.phys, n_planets=npl), s.size_table)
        m = run_gpu(engine, sp, 20, abi.DDX_PREC_MIXED)
        alive = (f["N"] != 0) & (m["N"] != 0)
        errs[npl] = np.median(rel_err(m, f)[alive])
    assert errs[3] * 50 < errs[1], errs


def test_deterministic(engine):
    s = small_ring(n_dust=4096, n_plsml=128)
    for prec in (abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED):
        a = run_gpu(engine, s, 3, prec)
        b = run_gpu(engine, s, 3, prec)
        for fld in FIELDS + ("N",):
            np.testing.assert_array_equal(a[fld], b[fld])


def test_sublimation_and_accretion_remove_tracers(engine):
    s = synth.solar_like(n_dust=64)
    st = {k: v.copy() for k, v in s.state.items()}
    ng = s.n_grav
    # tracer 0 inside the sublimation radius, tracer 1 exactly on planet 3
    st["x"][ng], st["y"][ng], st["z"][ng] = 0.01, 0.0, 0.0
    for f in ("x", "y", "z"):
        st[f][ng + 1] = st[f][3]
    for prec in (abi.DDX_PREC_FP64, abi.DDX_PREC_MIXED):
        for mode in (abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE):
            g = run_gpu(engine, s, 1, prec, mode, state=st)
            assert g["N"][ng] == 0 and g["N"][ng + 1] == 0
            assert g["x"][ng] == st["x"][ng] and g["x"][ng + 1] == st["x"][ng + 1]
            assert np.all(g["N"][ng + 2:] == 1)


def test_reference_mode_reproduces_stage4_sublimation_index(engine):
    # A grain that crosses Rmin only at stage 4 keeps its state; the reference zeroes
    # N[i] (i = dust-relative index) instead of its own N (src/gpu_functions.cu:878).
    M = synth.GRAV
    ng = 1
    n_dust = 4
    st = {f: np.zeros(ng + n_dust) for f in ("x", "y", "z", "vx", "vy", "vz", "m")}
    st["m"][0] = M
    st["N"] = np.ones(ng + n_dust)
    st["id"] = np.full(ng + n_dust, -1, np.int32)
    st["x"][1:] = [5.0, 6.0, 7.0, 1.0]
    st["vy"][1:] = [np.sqrt(M / 5), np.sqrt(M / 6), np.sqrt(M / 7), 0.0]
    # tracer 3 falls inward: stage positions 1.0, 0.70, 0.699, 0.396 AU with Rmin = 0.5,
    # so only stage 4 is inside the sublimation radius
    st["vx"][4] = -60.0
    sysm = synth.System("q", ng, st, 0.01, 1, dict(synth.solar_like(n_dust=1).phys, Rmin=0.5, n_planets=1),
                        synth._empty_size_table())
    o_ref = oc.step(st, ng, 0.01, sysm.size_table, sysm.phys, 1, ref_mode=True)
    o_fix = oc.step(st, ng, 0.01, sysm.size_table, sysm.phys, 1, ref_mode=False)
    assert o_fix["N"][4] == 0 and o_ref["N"][4] == 1 and o_ref["N"][3] == 0
    g_ref = run_gpu(engine, sysm, 1, abi.DDX_PREC_FP64, abi.DDX_MODE_REFERENCE, state=st)
    g_fix = run_gpu(engine, sysm, 1, abi.DDX_PREC_FP64, abi.DDX_MODE_FIXED, state=st)
    np.testing.assert_array_equal(g_ref["N"], o_ref["N"])
    np.testing.assert_array_equal(g_fix["N"], o_fix["N"])


def test_star_only_fixed_mode_moves_star_ballistically(engine):
    s = synth.solar_like(n_dust=32)
    st = {k: np.concatenate([v[:1], v[s.n_grav:]]) for k, v in s.state.items()}
    st["vx"][0] = 0.1
    sysm = synth.System("s", 1, st, 0.05, 1, dict(s.phys, n_planets=1), s.size_table)
    g = run_gpu(engine, sysm, 4, abi.DDX_PREC_FP64, abi.DDX_MODE_FIXED, state=st)
    assert g["x"][0] == pytest.approx(st["x"][0] + 0.1 * 0.2, rel=1e-14)
    o = oc.step(st, 1, 0.05, sysm.size_table, sysm.phys, 4, ref_mode=False)
    assert rel_err(g, o).max() < 1e-13


def test_lost_tile_copy_reports_timeout_and_context_recovers(engine):
    """Failure detection without a fault: one TMA tile copy is left unissued, the bounded
    mbarrier waits (20 ms here) run out, every block reports through the status word and
    leaves its tracers untouched, and the next step on the same context is normal."""
    s = small_ring(n_dust=2048, n_plsml=1100)          # 552 pair records: 2 tiles per stage
    engine.set_size_table(**s.size_table)
    phys = make_phys(**s.phys)
    st = DeviceState.from_numpy(s.state)
    assert engine.sync_status() == 0
    abi.check(engine.lib.ddx_debug_lose_tile_copy(engine.ctx, 1, 20_000_000), "inject")
    engine.step(st, s.n_grav, s.dt, phys, abi.DDX_PREC_MIXED)
    assert engine.sync_status() == 6
    after = st.to_numpy()
    ng = s.n_grav
    for f in FIELDS + ("N",):
        np.testing.assert_array_equal(after[f][ng:], s.state[f][ng:])
    assert engine.sync_status() == 0                    # the report was cleared
    engine.step(st, s.n_grav, s.dt, phys, abi.DDX_PREC_MIXED)
    assert engine.sync_status() == 0
    moved = st.to_numpy()
    assert np.all(moved["x"][ng:] != after["x"][ng:])


def test_zero_dust_and_bad_arguments(engine):
    s = synth.solar_like(n_dust=0)
    g = run_gpu(engine, s, 2)
    o = oc.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 2)
    assert rel_err(g, o).max() < 1e-13
    st = DeviceState.from_numpy(s.state)
    with pytest.raises(abi.DDXError) as ei:
        engine.evolve(st, 0, 0.1, 1, make_phys(**s.phys))
    assert ei.value.status == 1
    with pytest.raises(abi.DDXError):
        engine.evolve(st, s.n_grav, 0.1, 1, make_phys(**s.phys), precision=7)
    big = {k: np.zeros(2701, np.float32) for k in ("beta", "betasw", "q")}
    with pytest.raises(abi.DDXError) as ei:
        engine.set_size_table(np.zeros(2701), **big)
    assert ei.value.status == 5
