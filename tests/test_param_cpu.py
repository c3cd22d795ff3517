"""ddx_param_read against the reference's own parser (read_in_param, src/read_in.cu).

The fixtures in tests/golden/params/ are synthetic parameter files and the reference
parser's output for each (tests/golden/make_param_golden.py); every value must agree to
the bit, including the planets' Cartesian states from coe2rv and the centre-of-mass
correction, and rejected files must be rejected with the reference's usage code.  Where
the reference sources are present, the reference's own 13 test systems are parsed by
both as well."""
import json
import subprocess
from pathlib import Path

import pytest

from diskdyn_gb300 import formats

GOLD = Path(__file__).resolve().parent / "golden" / "params"
from oracle.ref.paths import TESTS as REF_TESTS  # noqa: E402


def as_float(v):
    return float.fromhex(v) if isinstance(v, str) else float(v)


def compare(ours: dict, ref: dict, where: str):
    for k in ("verb", "gpuid", "gl", "n_step", "xsize", "ysize", "radQ", "SWQ", "FLQ"):
        assert ours[k] == ref[k], (where, k)
    for k in ("t_gl", "t_write", "t_fits", "t_sed", "t_end", "teff", "rstar", "Bstar", "Wz", "mloss", "vsw", "dist",
              "fov", "PA", "inc", "longitude", "rho", "kqe"):
        assert ours[k] == as_float(ref[k]), (where, k, ours[k], as_float(ref[k]))
    for k in ("sptype", "specfile", "comp", "name_stub"):
        assert ours[k] == ref[k], (where, k)
    assert ours["wavs"] == [as_float(v) for v in ref["wavs"]], where
    assert len(ours["planets"]) == len(ref["planets"]), where
    for a, b in zip(ours["planets"], ref["planets"]):
        assert a == [as_float(v) for v in b], (where, "planet")
    assert len(ours["disks"]) == len(ref["disks"]), where
    for a, b in zip(ours["disks"], ref["disks"]):
        for k, v in b.items():
            assert a[k] == (v if k in ("Ngrav", "Nsmall") else as_float(v)), (where, "disk", k)
    assert len(ours["blobs"]) == len(ref["blobs"]), where
    for a, b in zip(ours["blobs"], ref["blobs"]):
        for k, v in b.items():
            assert a[k] == (v if k in ("Ngrav", "Nsmall", "collcloud") else as_float(v)), (where, "blob", k)


CASES = sorted(p.stem for p in GOLD.glob("*.param"))


@pytest.mark.parametrize("name", CASES)
def test_parse_matches_reference_parser(name):
    ref = json.loads((GOLD / f"{name}.json").read_text())
    if ref.get("rejected"):
        with pytest.raises(formats.ParamError) as e:
            formats.read_param(GOLD / f"{name}.param")
        assert e.value.usage_code == ref["usage_code"]
        return
    compare(formats.read_param(GOLD / f"{name}.param"), ref, name)


def test_missing_file_is_usage_code_3():
    with pytest.raises(formats.ParamError) as e:
        formats.read_param(GOLD / "does_not_exist.param")
    assert e.value.status == 8 and e.value.usage_code == 3


def reference_parser():
    import oracle.ref.build_param_ref as bp
    try:
        return bp.build()
    except RuntimeError:
        return None


def test_reference_test_systems_present():
    from oracle.ref import paths
    paths.require(REF_TESTS, "the reference's test systems")


@pytest.mark.skipif(not REF_TESTS.exists(), reason="the reference's test systems are not on this machine")
@pytest.mark.parametrize("name", sorted(p.stem for p in REF_TESTS.glob("*.param")) if REF_TESTS.exists() else [])
def test_reference_test_systems_parse_identically(name):
    exe = reference_parser()
    if exe is None:
        pytest.skip("the reference parser could not be built")
    path = REF_TESTS / f"{name}.param"
    ref = json.loads(subprocess.run([str(exe), str(path)], capture_output=True, text=True, check=True).stdout)
    compare(formats.read_param(path), ref, name)
