import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def dem_lib_path():
    from taichi_dem_julia_port_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    from oracle.build import build
    build()
    return oracle.load()


@pytest.fixture(scope="session")
def gpu(dem_lib_path):
    """Skips unless a CUDA device is present; the library then must load."""
    from taichi_dem_julia_port_gb300 import _abi
    lib = _abi.load_library()
    return lib


def assert_rows_close(a, b, rtol, what="", atol_frac=None):
    """Row-wise |a-b| <= rtol·max(|a_row|,|b_row|) + atol, atol = atol_frac·max|b|.

    atol covers rows whose true value is ~0 (cancelling contributions)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, f"{what}: shapes {a.shape} vs {b.shape}"
    if a.ndim == 1:
        a, b = a[:, None], b[:, None]
    if a.size == 0:
        return
    na, nb = np.linalg.norm(a, axis=1), np.linalg.norm(b, axis=1)
    scale = float(np.max(nb)) if nb.size else 0.0
    atol = (atol_frac if atol_frac is not None else rtol) * scale
    d = np.linalg.norm(a - b, axis=1)
    lim = rtol * np.maximum(na, nb) + atol
    bad = np.nonzero(~(d <= lim))[0]
    assert bad.size == 0, (f"{what}: {bad.size} rows differ; first row {bad[0]}: "
                           f"{a[bad[0]]} vs {b[bad[0]]} (|d|={d[bad[0]]:.3e}, lim={lim[bad[0]]:.3e})")
