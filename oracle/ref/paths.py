"""ORACLE -- test infrastructure.  Where the reference checkout lies.

DDX_REFERENCE_ROOT names the checkout of the reference (its src/ and tests/ folders); it
defaults to /root/reference, where the development container mounts it read-only.  The
recipes compile from those sources in place and write only under oracle/_ref/.  Machines
without a copy (the GPU hosts) use what was built from it, or skip what needs the sources;
when DDX_REFERENCE_ROOT is set explicitly the sources are expected, and a test that needs
them fails instead of skipping.
"""
from __future__ import annotations

import os
from pathlib import Path

ROOT = Path(os.environ.get("DDX_REFERENCE_ROOT", "/root/reference"))
SRC = ROOT / "src"
TESTS = ROOT / "tests"
EXPECTED = "DDX_REFERENCE_ROOT" in os.environ


def require(path: Path, what: str = "reference sources") -> None:
    """For tests: return when `path` exists; otherwise fail if the reference was named
    explicitly, else skip."""
    if path.exists():
        return
    import pytest
    msg = f"{what} absent: {path}"
    if EXPECTED:
        pytest.fail(msg + " (DDX_REFERENCE_ROOT is set)")
    pytest.skip(msg)
