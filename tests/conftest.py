"""Shared fixtures.  Tests that need a GPU are marked ``gpu``; everything else runs on CPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
# full-size fixtures made by tests/golden/make_fixtures.py / make_vp_fixtures.py (git-ignored)
FULL_DIR = GOLDEN / "full"
FULL_FIXTURE = FULL_DIR / "cells_zs1_gauss_full.npz"
VP_FULL = FULL_DIR / "vp_zs1_full.npz"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine")


@pytest.fixture(scope="session")
def ref_sub():
    """Reference outputs on the committed z_s=1 population subset (tests/golden/make_golden.py)."""
    return dict(np.load(GOLDEN / "ref_zs1_sub.npz"))


@pytest.fixture(scope="session")
def pop_sub():
    from sgl_analytic_gb300.population import Population
    return Population.load(GOLDEN / "pop_zs1_sub.npz")


@pytest.fixture(scope="session")
def cli_grid():
    return np.concatenate([np.linspace(-1.0, 1.0, 1601), np.linspace(1.005, 9.0, 1600)])
