"""Images and SEDs on the GPU through the C ABI, against the CPU oracle and the
reference's own flux kernels.

Pixel indices must equal the reference kernel's bit for bit on the same GPU; against the
CPU oracle (libm instead of the CUDA math library) they may differ only for tracers
within 1e-9 pixel of an edge.  Fluxes: 1e-11 relative per pixel against both (the
reference's atomics add in a varying order; the T(R) and phase-function interpolations
here use tabulated logs).
"""
import math

import numpy as np
import pytest
import torch

import oracle.cpu as oc
from diskdyn_gb300 import abi, synth
from diskdyn_gb300.engine import DeviceState, make_view

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def img_sys():
    return synth.imaging(n_dust=65536, xsize=256, ysize=200)


def setup_engine(engine, s):
    engine.set_size_table(**s.size_table)
    o = s.optics
    engine.set_optics(o["w"], o["in"], o["Qabs"], o["Qsca"], o["Qpfunc"], o["Td"], o["Rmin"], o["Rmax"])


def gpu_image(engine, s, state=None, wj=None):
    setup_engine(engine, s)
    st = DeviceState.from_numpy(state if state is not None else s.state)
    F = engine.image(st, s.n_grav, make_view(**s.view), wj if wj is not None else s.image_wj)
    torch.cuda.synchronize()
    return F.cpu().numpy()


def gpu_pixels(engine, s, state=None):
    setup_engine(engine, s)
    st = DeviceState.from_numpy(state if state is not None else s.state)
    pix, ex = engine.pixels(st, s.n_grav, make_view(**s.view))
    return pix.cpu().numpy(), ex.cpu().numpy()


def test_image_matches_oracle(engine, img_sys):
    s = img_sys
    F = gpu_image(engine, s)
    Fo, pix_o = oc.image(s.state, s.n_grav, s.optics, s.size_table["size"], s.view, s.image_wj)
    pix, _ = gpu_pixels(engine, s)
    assert (pix != pix_o).sum() == 0
    np.testing.assert_allclose(F, Fo, rtol=1e-11, atol=0)


def test_sed_matches_oracle_both_modes(engine, img_sys):
    s = img_sys
    setup_engine(engine, s)
    st = DeviceState.from_numpy(s.state)
    for mode in (abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE):
        F = engine.sed(st, s.n_grav, make_view(**s.view), mode=mode).cpu().numpy()
        Fo = oc.sed(s.state, s.n_grav, s.optics, s.size_table["size"], s.view, ref_mode=mode == abi.DDX_MODE_REFERENCE)
        np.testing.assert_allclose(F, Fo, rtol=1e-11)


def test_image_and_sed_match_reference_kernels(engine, refk, img_sys):
    s = img_sys
    F = gpu_image(engine, s)
    Fr = refk.image(s.state, s.n_grav, s.optics, s.size_table["size"], s.view, s.image_wj)
    assert np.array_equal(F != 0, Fr != 0)
    np.testing.assert_allclose(F, Fr, rtol=1e-11, atol=0)
    setup_engine(engine, s)
    st = DeviceState.from_numpy(s.state)
    Fs = engine.sed(st, s.n_grav, make_view(**s.view), mode=abi.DDX_MODE_REFERENCE).cpu().numpy()
    Fsr = refk.sed(s.state, s.n_grav, s.optics, s.size_table["size"], s.view)
    np.testing.assert_allclose(Fs, Fsr, rtol=1e-11)


def spread_batches(pix, min_sep, ysize):
    """Greedy batches of tracers whose pixels are at least min_sep apart (Chebyshev), so
    a tracer that the reference puts one pixel away cannot land on another's pixel."""
    order = np.flatnonzero(pix >= 0)
    batches = []
    remaining = list(order)
    r = min_sep - 1
    while remaining:
        taken, blocked, rest = [], set(), []
        for i in remaining:
            x, y = divmod(int(pix[i]), ysize)
            if (x, y) in blocked:
                rest.append(i)
                continue
            taken.append(i)
            for dx in range(-r, r + 1):
                for dy in range(-r, r + 1):
                    blocked.add((x + dx, y + dy))
        batches.append(np.array(taken))
        remaining = rest
    return batches


def check_pixels_against_reference(engine, refk, s, state, max_batches=40):
    pix, ex = gpu_pixels(engine, s, state)
    ng = s.n_grav
    ysize = s.view["ysize"]
    R = np.sqrt(state["x"][ng:] ** 2 + state["y"][ng:] ** 2 + state["z"][ng:] ** 2)
    lit = R > s.optics["Rmin"]          # tracers inside Rmin add no flux (src/gpu_functions.cu:1077)
    batches = spread_batches(np.where(lit, pix, -1), 3, ysize)
    assert len(batches) <= max_batches
    bad = []
    for b in batches:
        sub = {k: np.concatenate([v[:ng], v[ng:][b]]) for k, v in state.items()}
        Fr = refk.image(sub, ng, s.optics, s.size_table["size"], s.view, [s.image_wj[0]])[0]
        nz = set(np.flatnonzero(Fr.ravel()).tolist())
        bad += [(int(i), int(pix[i]), int(ex[i])) for i in b if int(pix[i]) not in nz]
    assert not bad, f"{len(bad)} tracers (index, our pixel, exact path) differ: {bad[:20]}"
    # a tracer the GPU puts outside the image must also be outside in the reference
    out = np.flatnonzero((pix < 0) & lit & (state["id"][ng:] >= 0))
    if len(out):
        sub = {k: np.concatenate([v[:ng], v[ng:][out]]) for k, v in state.items()}
        Fr = refk.image(sub, ng, s.optics, s.size_table["size"], s.view, [s.image_wj[0]])[0]
        assert np.count_nonzero(Fr) == 0
    return ex


def test_pixel_indices_bit_identical_to_reference(engine, refk, img_sys):
    s = img_sys
    sub = {k: np.concatenate([v[:s.n_grav], v[s.n_grav:s.n_grav + 6000]]) for k, v in s.state.items()}
    check_pixels_against_reference(engine, refk, s, sub)


def edge_tracers(s, n=3000, seed=3, spread=None):
    """Tracers placed so that their projected coordinates fall within ~1e-13 pixel of a
    pixel edge (x, y or both), by inverting the projection of the view.  spread=(lo, hi):
    at a distance log-uniform in [lo, hi] pixel from the edge instead, on either side."""
    v = s.view
    g = synth.rng(seed)
    psca = v["fov"] / max(v["xsize"], v["ysize"])
    ix = g.integers(1, v["xsize"] - 1, n).astype(np.float64)
    iy = g.integers(1, v["ysize"] - 1, n).astype(np.float64)
    frac = lambda: g.uniform(0.2, 0.8, n)
    tiny = g.uniform(-3e-13, 3e-13, n)
    if spread is not None:
        tiny = np.sign(g.uniform(-1, 1, n)) * 10.0 ** g.uniform(math.log10(spread[0]), math.log10(spread[1]), n)
    kind = g.integers(0, 3, n)
    u = np.where(kind != 1, ix + tiny, ix + frac())
    w = np.where(kind != 0, iy + tiny, iy + frac())
    X = u * psca - 0.5 * psca * v["xsize"]
    Y = w * psca - 0.5 * psca * v["ysize"]
    ca, sa = math.cos(v["PA"]), math.sin(v["PA"])
    x1 = X * ca + Y * sa
    y2 = -X * sa + Y * ca
    ci, si = math.cos(v["inc"]), math.sin(v["inc"])
    depth = g.uniform(-20.0, 20.0, n)
    y1 = y2 * ci - depth * si
    z = y2 * si + depth * ci
    cr, sr = math.cos(v["longitude"]), math.sin(v["longitude"])
    x = x1 * cr + y1 * sr
    y = -x1 * sr + y1 * cr
    st = {k: arr[:s.n_grav].copy() for k, arr in s.state.items()}
    ids = g.integers(0, 64, n).astype(np.int32)
    for k, val in (("x", x), ("y", y), ("z", z), ("vx", 0 * x), ("vy", 0 * x), ("vz", 0 * x),
                   ("m", 0 * x), ("N", np.full(n, 1e15))):
        st[k] = np.concatenate([st[k], val])
    st["id"] = np.concatenate([st["id"], ids])
    return st


def test_pixel_indices_at_pixel_edges_bit_identical_to_reference(engine, refk):
    s = synth.imaging(n_dust=16, xsize=300, ysize=240)
    s.view.update(inc=math.radians(37.0), PA=math.radians(23.0), longitude=math.radians(11.0))
    st = edge_tracers(s)
    ex = check_pixels_against_reference(engine, refk, s, st, max_batches=400)
    assert ex.sum() > 0.9 * len(ex)      # the guard band sent them down the exact path


def gpu_image_prec(engine, s, state, precision, wj=None):
    setup_engine(engine, s)
    st = DeviceState.from_numpy(state)
    F = engine.image(st, s.n_grav, make_view(**s.view), wj if wj is not None else s.image_wj, precision=precision)
    torch.cuda.synchronize()
    return F.cpu().numpy()


def test_mixed_image_matches_fp64(engine, img_sys):
    """FP32 photometry: every pixel within 1e-5 of the FP64 image (a pixel is a sum of
    positive terms, each within ~1e-6), the same pixels lit, total flux within 1e-6."""
    s = img_sys
    F = gpu_image_prec(engine, s, s.state, abi.DDX_PREC_FP64)
    Fm = gpu_image_prec(engine, s, s.state, abi.DDX_PREC_MIXED)
    assert np.array_equal(F != 0, Fm != 0)
    np.testing.assert_allclose(Fm, F, rtol=1e-5, atol=0)
    for k in range(len(F)):
        assert abs(Fm[k].sum() / F[k].sum() - 1.0) < 1e-6


@pytest.mark.parametrize("spread", [None, (1e-7, 1e-2)])
def test_mixed_pixel_indices_match_fp64_near_edges(engine, spread):
    """The mixed image puts every tracer in the FP64 kernel's pixel (which is the
    reference's): tracers within 3e-13 pixel of an edge, and tracers at 1e-7..1e-2 pixel
    on either side, across the FP32 guard band.  Batches of tracers at least 3 pixels
    apart, so equal lit-pixel sets mean equal pixels tracer by tracer."""
    s = synth.imaging(n_dust=16, xsize=300, ysize=240)
    s.view.update(inc=math.radians(37.0), PA=math.radians(23.0), longitude=math.radians(11.0))
    st = edge_tracers(s, n=2000, seed=4, spread=spread)
    pix, _ = gpu_pixels(engine, s, st)
    ng = s.n_grav
    R = np.sqrt(st["x"][ng:] ** 2 + st["y"][ng:] ** 2 + st["z"][ng:] ** 2)
    batches = spread_batches(np.where(R > s.optics["Rmin"], pix, -1), 3, s.view["ysize"])
    for b in batches:
        sub = {k: np.concatenate([v[:ng], v[ng:][b]]) for k, v in st.items()}
        F = gpu_image_prec(engine, s, sub, abi.DDX_PREC_FP64, [s.image_wj[0]])
        Fm = gpu_image_prec(engine, s, sub, abi.DDX_PREC_MIXED, [s.image_wj[0]])
        assert np.array_equal(F != 0, Fm != 0)


def test_mixed_sed_matches_fp64_both_modes(engine, img_sys):
    s = img_sys
    setup_engine(engine, s)
    st = DeviceState.from_numpy(s.state)
    for mode in (abi.DDX_MODE_FIXED, abi.DDX_MODE_REFERENCE):
        F = engine.sed(st, s.n_grav, make_view(**s.view), mode=mode).cpu().numpy()
        Fm = engine.sed(st, s.n_grav, make_view(**s.view), precision=abi.DDX_PREC_MIXED, mode=mode).cpu().numpy()
        np.testing.assert_allclose(Fm, F, rtol=1e-5)


def test_image_rejects_bad_arguments(engine, img_sys):
    s = img_sys
    setup_engine(engine, s)
    st = DeviceState.from_numpy(s.state)
    with pytest.raises(abi.DDXError):
        engine.image(st, s.n_grav, make_view(**s.view), [10_000])
    with pytest.raises(abi.DDXError) as ei:
        engine.image(st, s.n_grav, make_view(**s.view), list(range(65)))
    assert ei.value.status == 5
    bad = dict(s.view, xsize=0)
    with pytest.raises(abi.DDXError):
        engine.image(st, s.n_grav, make_view(**bad), [1])


def test_mixed_image_aggregates_lanes_on_one_pixel(engine, img_sys):
    """Tracers sorted by their pixel put whole warps on one pixel, so most of the flux goes
    through the warp-aggregated path (the lanes of a pixel added by shuffles, one atomic per
    pixel and warp).  The image of the sorted state has the same lit pixels as the FP64 image
    and every pixel within 1e-5 of it, like the unsorted state's."""
    s = img_sys
    pix, _ = gpu_pixels(engine, s)
    ng = s.n_grav
    order = np.argsort(np.where(pix < 0, np.iinfo(np.int32).max, pix), kind="stable")
    st = {k: np.concatenate([np.asarray(v)[:ng], np.asarray(v)[ng:][order]]) for k, v in s.state.items()}
    F64 = gpu_image_prec(engine, s, s.state, abi.DDX_PREC_FP64)
    Fm = gpu_image_prec(engine, s, st, abi.DDX_PREC_MIXED)
    lit = F64 != 0
    assert np.array_equal(lit, Fm != 0)
    assert np.max(np.abs(Fm[lit] / F64[lit] - 1.0)) < 1e-5
    # many warps did share pixels
    ps = pix[order][:len(pix) // 32 * 32].reshape(-1, 32)
    assert np.mean([len(np.unique(r[r >= 0])) < 16 for r in ps]) > 0.5


def test_images_and_sed_skip_nan_tracers(engine, img_sys):
    """Tracers with NaN coordinates add nothing to the images and the SED (FP64 and mixed):
    the results equal those of the same state without them, to the summation order."""
    s = img_sys
    ng = s.n_grav
    st = {k: np.asarray(v).copy() for k, v in s.state.items()}
    bad = np.arange(ng, ng + 64)
    st["x"][bad[:32]] = np.nan
    st["z"][bad[32:]] = np.nan
    keep = np.ones(len(st["x"]), bool)
    keep[bad] = False
    clean = {k: v[keep] for k, v in st.items()}
    setup_engine(engine, s)
    view = make_view(**s.view)
    for prec, tol in ((abi.DDX_PREC_FP64, 1e-12), (abi.DDX_PREC_MIXED, 1e-5)):
        a = engine.image(DeviceState.from_numpy(st), ng, view, s.image_wj, precision=prec).cpu().numpy()
        b = engine.image(DeviceState.from_numpy(clean), ng, view, s.image_wj, precision=prec).cpu().numpy()
        assert np.array_equal(a != 0, b != 0)
        lit = b != 0
        assert np.max(np.abs(a[lit] / b[lit] - 1.0)) < tol
        sa = engine.sed(DeviceState.from_numpy(st), ng, view, precision=prec).cpu().numpy()
        sb = engine.sed(DeviceState.from_numpy(clean), ng, view, precision=prec).cpu().numpy()
        np.testing.assert_allclose(sa, sb, rtol=tol)
