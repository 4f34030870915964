"""Failure detection on the GPU, in the forms that fault, trap or hang nothing.

* Bounded device waits: the grid barrier of the fused pair search and the
  decoupled look-back of the bucket scan give up after a wait limit and
  raise DEM_ERR_TIMEOUT, which the host reads back; the context stays
  usable.  The tests shorten the limit (a few thousand polls, well under a
  millisecond) and leave one party out, so the wait has to run out.
* Invalid input (NaN positions, non-positive volume or mass) is refused on
  the host with DEM_ERR_INVALID before anything reaches the device.
* Capacity overflow (too many contacts for max_coordinate_number) is covered
  in tests/test_gpu_parity.py (test_capacity_overflow_reports_error).
"""
import ctypes as C

import numpy as np
import pytest

from taichi_dem_julia_port_gb300 import GlobalData, scenes
from taichi_dem_julia_port_gb300._abi import (DEM_ERR_INVALID, DEM_ERR_TIMEOUT, DEM_OK,
                                              DemError)

pytestmark = pytest.mark.gpu


def wait_status(lib, which, missing, limit):
    st = C.c_int(-1)
    assert lib.dem_selftest_wait_timeout(which, missing, limit, C.byref(st)) == DEM_OK
    return st.value


@pytest.mark.parametrize("which", [0, 1], ids=["grid_barrier", "scan_lookback"])
def test_bounded_wait_runs_out_and_reports_timeout(gpu, which):
    # a party never arrives: the wait gives up after 4096 polls
    assert wait_status(gpu, which, 1, 4096) == DEM_ERR_TIMEOUT
    # everyone arrives: no timeout, even with the limit raised
    assert wait_status(gpu, which, 0, 1 << 20) == DEM_OK
    # and again after the timeout: the device is still usable
    assert wait_status(gpu, which, 1, 4096) == DEM_ERR_TIMEOUT


def test_library_usable_after_a_timeout(gpu):
    assert wait_status(gpu, 0, 1, 1024) == DEM_ERR_TIMEOUT
    sc = scenes.bonded_cube(4, steps=0)
    g = GlobalData(sc.cfg, sc.particles)
    g.initialize()
    g.simulate(20)
    assert g.stats()["error"] == 0
    assert g.stats()["bonded"] == 3 * 4 * 4 * 3
    g.close()


def test_wait_selftest_rejects_bad_arguments(gpu):
    st = C.c_int(0)
    assert gpu.dem_selftest_wait_timeout(2, 1, 100, C.byref(st)) == DEM_ERR_INVALID
    assert gpu.dem_selftest_wait_timeout(0, 1, 0, C.byref(st)) == DEM_ERR_INVALID
    assert gpu.dem_selftest_wait_timeout(0, 1, (1 << 20) + 1, C.byref(st)) == DEM_ERR_INVALID


@pytest.mark.parametrize("field,value", [("pos", np.nan), ("vel", np.inf), ("volume", 0.0),
                                         ("mass", -1.0)])
def test_invalid_grain_rejected_at_create(gpu, field, value):
    sc = scenes.bonded_cube(3, steps=0)
    p = sc.particles.copy()
    arr = getattr(p, field)
    if arr.ndim == 2:
        arr[5, 1] = value
    else:
        arr[5] = value
    with pytest.raises(DemError) as e:
        GlobalData(sc.cfg, p)
    assert e.value.code == DEM_ERR_INVALID
    assert "grain 5" in str(e.value)


def test_nan_rejected_by_set_particles(gpu):
    sc = scenes.bonded_cube(3, steps=0)
    g = GlobalData(sc.cfg, sc.particles)
    g.initialize()
    before = g.particles()
    pos = before["pos"].copy()
    pos[7, 2] = np.nan
    with pytest.raises(DemError) as e:
        g.set_particles(pos=pos)
    assert e.value.code == DEM_ERR_INVALID
    after = g.particles()
    np.testing.assert_array_equal(after["pos"], before["pos"])  # nothing was uploaded
    g.simulate(5)
    assert g.stats()["error"] == 0
    g.close()
