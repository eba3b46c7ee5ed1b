"""Shared fixtures. Tests marked ``gpu`` need a CUDA device (they run on the
GB300 host); everything else runs on CPU only."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
REGS = ("singular", "winckelmans", "planetary", "gaussian")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


@pytest.fixture(scope="session")
def built():
    from cvortex_gb300 import build
    build.build()
    import oracle
    oracle.build()
    return True


@pytest.fixture(scope="session")
def cv(built):
    from cvortex_gb300.abi import Cvtx
    c = Cvtx()
    c.initialise()
    return c


@pytest.fixture()
def gpu(cv):
    """The library with accelerator 0 enabled; fails (does not skip) when no
    CUDA device is visible, so a GPU run can never pass on a host path."""
    n = cv.num_accelerators()
    assert n >= 1, "no CUDA device visible to libcvortex"
    cv.set_accelerated(True)
    cv.lib.cvtx_gb300_clear_error()
    yield cv
    err = cv.last_error()
    cv.lib.cvtx_gb300_clear_error()
    assert err == "", f"library reported an error: {err}"


@pytest.fixture()
def host(cv):
    """The library with every accelerator disabled (the ABI's host path)."""
    cv.set_accelerated(False)
    yield cv
    cv.set_accelerated(True)


def golden(name: str):
    return np.load(GOLDEN / f"{name}.npz")
