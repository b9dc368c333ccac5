import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN / "reference_cases.npz")


@pytest.fixture(scope="session")
def legacy_kernels():
    return np.load(GOLDEN / "legacy_kernels.npz")


@pytest.fixture(scope="session")
def legacy_towers():
    return np.load(GOLDEN / "legacy_towers.npz")


@pytest.fixture(scope="session")
def legacy_grid():
    return np.load(GOLDEN / "legacy_grid.npz")


def legacy_grid_points(g):
    """The 32^3 grid of tests/legacy/test_phase1_port.py:77-87, x fastest (meshgrid(z, y, x, 'ij'))."""
    xs, ys, zs = (np.linspace(a[0], a[1], int(a[2])) for a in (g["x_axis"], g["y_axis"], g["z_axis"]))
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return (xs, ys, zs), np.c_[X.ravel(), Y.ravel(), Z.ravel()]


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def assert_close(a, b, rtol, atol_rel=None):
    """Elementwise |a - b| <= rtol |b| + atol, atol = atol_rel * max|b| (default rtol)."""
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(np.abs(b).max(), 1e-300)
    atol = (rtol if atol_rel is None else atol_rel) * scale
    bad = np.abs(a - b) > rtol * np.abs(b) + atol
    assert not bad.any(), f"max rel err {rel_err(a, b):.3e} at {np.argwhere(bad)[:3].tolist()}"
