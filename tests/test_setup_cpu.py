"""Start-of-run set-up on the host, pinned to the reference.

tests/golden/setup/ holds parameter files and the system the reference's own set-up built
from them with the table and spectrum of tests/golden/optics/ (detminmax, confCdisks,
confCblobs, calculate_beta and Grid::setup's generation with ran3 seeded at -2;
tests/golden/make_setup_golden.py).  ddx_param_grid and ddx_setup_host give the same
values to the bit; the oracle's restatement of the GPU generator's counter-based draws is
checked against the Philox known-answer vectors and, statistically, against the
reference's generator."""
import importlib.util
import shutil
from pathlib import Path

import numpy as np
import pytest

import oracle.cpu as oc
from diskdyn_gb300 import formats

GOLD = Path(__file__).resolve().parent / "golden" / "setup"
CASES = ("disks_blobs", "rejections")
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "N", "m", "id")


def load(case):
    d = np.load(GOLD / f"{case}.npz")
    return {k: d[k] for k in d.files}


def gridded(case, d):
    p = formats.read_param_struct(GOLD / f"{case}.param")
    formats.param_grid(p, float(d["dmin"]), float(d["dmax"]))
    return p


@pytest.mark.parametrize("case", CASES)
def test_param_grid_bit_exact(built_lib, case):
    d = load(case)
    p = gridded(case, d)
    assert p.n_grid == d["n_grid"]
    assert [p.amin, p.amax, p.mmin, p.mmax, p.f] == [d[k] for k in ("amin", "amax", "mmin", "mmax", "f")]
    for j in range(p.n_disks):
        k = p.disks[j]
        assert [k.amin, k.mmin, k.dmax, k.dmmax, k.C] == list(d["disks"][j])
    for j in range(p.n_blobs):
        k = p.blobs[j]
        assert [k.amin, k.mmin, k.dmax, k.dmmax, k.C] == list(d["blobs"][j])


@pytest.mark.parametrize("case", CASES)
def test_setup_host_bit_exact(built_lib, case):
    d = load(case)
    p = gridded(case, d)
    a, run = formats.setup_host(p, float(d["dmin"]), float(d["dmax"]), d["beta"])
    assert (run.n_all, run.n_mass, run.n_dust) == (d["n_all"], d["n_mass"], d["n_dust"])
    for k in FIELDS:
        np.testing.assert_array_equal(a[k], d[k], err_msg=k)


def test_eta_two_gravitating_masses_are_nan_as_in_the_reference(built_lib):
    """eta_a = 4 (eta = 2) makes getbod divide by 1 + (1 - eta) = 0: the reference's
    gravitating bodies of that disk get NaN masses, and so do ours."""
    d = load("rejections")
    p = gridded("rejections", d)
    assert p.disks[0].eta == 2.0
    a, _ = formats.setup_host(p, float(d["dmin"]), float(d["dmax"]), d["beta"])
    ng = p.disks[0].Ngrav
    assert np.isnan(a["m"][1:1 + ng]).all() and np.isnan(d["m"][1:1 + ng]).all()


def test_populations_follow_the_reference_order(built_lib):
    d = load("disks_blobs")
    p = gridded("disks_blobs", d)
    kind, idx = oc.setup_populations(p, float(d["dmin"]), float(d["dmax"]))
    assert len(kind) == d["n_all"] - p.n_planets
    assert (d["id"][p.n_planets:][:d["n_mass"]] == -1).all()
    assert list(kind[:d["n_mass"]]) == [0] * 30 + [1] * 8
    run = formats.setup_count(p, float(d["dmin"]), float(d["dmax"]))
    assert (run.n_all, run.n_mass, run.n_dust) == (d["n_all"], d["n_mass"], d["n_dust"])


def test_philox_known_answers():
    """The known-answer vectors that accompany the published Philox4x32-10."""
    assert oc.philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)
    assert oc.philox4x32_10((0xffffffff,) * 4, (0xffffffff,) * 2) == (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)
    assert oc.philox4x32_10((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0)) == \
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)


def big_system(scale=40):
    d = load("disks_blobs")
    p = formats.read_param_struct(GOLD / "disks_blobs.param")
    for j in range(p.n_disks):
        p.disks[j].Nsmall *= scale
    for j in range(p.n_blobs):
        p.blobs[j].Nsmall *= scale
    formats.param_grid(p, float(d["dmin"]), float(d["dmax"]))
    return d, p


def philox_state(d, p, host, seed):
    kind, idx = oc.setup_populations(p, float(d["dmin"]), float(d["dmax"]))
    npl = p.n_planets
    ids = host["id"][npl:]
    beta = np.where(ids >= 0, d["beta"][np.maximum(ids, 0)].astype(np.float64), 0.0)
    beta[beta >= 0.5] = 0.0
    out, bad = oc.setup_philox(p, kind, idx, host["m"][npl:], beta, seed, npl)
    return out, bad, kind, idx


def test_counter_based_draws_match_the_reference_distributions(built_lib):
    """Same populations drawn by ran3 (the reference's generator) and by the counter-based
    generator: the radius, height and speed distributions of every disk and blob agree
    (two-sample Kolmogorov-Smirnov, each p > 1e-4)."""
    stats = pytest.importorskip("scipy.stats")
    d, p = big_system()
    host, run = formats.setup_host(p, float(d["dmin"]), float(d["dmax"]), d["beta"])
    out, bad, kind, idx = philox_state(d, p, host, seed=12345)
    assert bad == 0
    npl = p.n_planets
    pos = np.stack([host[k][npl:] for k in ("x", "y", "z")], 1)
    vel = np.stack([host[k][npl:] for k in ("vx", "vy", "vz")], 1)
    for k in (0, 1):
        for j in range(p.n_disks if k == 0 else p.n_blobs):
            sel = (kind == k) & (idx == j)
            sel[:run.n_mass] = False                    # the grains
            assert sel.sum() > 1000
            for name, a, b in (("r", np.linalg.norm(pos[sel], axis=1), np.linalg.norm(out[sel, :3], axis=1)),
                               ("z/r", pos[sel, 2] / np.linalg.norm(pos[sel], axis=1),
                                out[sel, 2] / np.linalg.norm(out[sel, :3], axis=1)),
                               ("v", np.linalg.norm(vel[sel], axis=1), np.linalg.norm(out[sel, 3:], axis=1))):
                assert stats.ks_2samp(a, b).pvalue > 1e-4, (k, j, name)


def test_counter_based_draws_are_per_body(built_lib):
    """A body's draws depend on the seed and its index only."""
    d = load("disks_blobs")
    p = gridded("disks_blobs", d)
    host, _ = formats.setup_host(p, float(d["dmin"]), float(d["dmax"]), d["beta"])
    full, _, kind, idx = philox_state(d, p, host, seed=7)
    npl = p.n_planets
    ids = host["id"][npl:]
    beta = np.where(ids >= 0, d["beta"][np.maximum(ids, 0)].astype(np.float64), 0.0)
    beta[beta >= 0.5] = 0.0
    part, _ = oc.setup_philox(p, kind[500:], idx[500:], host["m"][npl + 500:], beta[500:], 7, npl + 500)
    np.testing.assert_array_equal(part, full[500:])
    other, _, _, _ = philox_state(d, p, host, seed=8)
    assert not np.any(np.all(other == full, axis=1))       # (collision blobs keep x, not v)


from oracle.ref.paths import SRC as _REF_SRC  # noqa: E402

REF_SRC = _REF_SRC / "read_in.cu"


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc absent")
@pytest.mark.parametrize("case", CASES)
def test_reference_reproduces_fixtures(tmp_path, case):
    from oracle.ref import paths
    paths.require(REF_SRC)
    spec = importlib.util.spec_from_file_location("msg", Path(__file__).parent / "golden" / "make_setup_golden.py")
    msg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(msg)
    from oracle.ref import build_param_ref
    got = msg.run_reference(build_param_ref.build_setup(), GOLD / f"{case}.param", tmp_path / "out.bin")
    d = load(case)
    for k, v in got.items():
        np.testing.assert_array_equal(v, d[k], err_msg=k)
