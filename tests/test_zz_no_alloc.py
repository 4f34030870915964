"""The allocation-free bucket sort (dem_bucket_sort_noalloc) against the
library's regular broad phase (dem_debug_broadphase).

The entry point exists for callers that cannot allocate device memory (hosts
that reserve every GPU buffer up front, or whose allocator belongs to another
framework): they pass their own device buffers and the library's temporary
memory is a fixed array inside the library.  This test plays such a caller:
its device buffers are made beforehand (here with torch), and it calls the
entry point through the C ABI twice in a row on different scenes, so the
second call runs on the array the first call left behind.

This file is named so that pytest collects it after every other test file.
"""
import ctypes as C

import numpy as np
import pytest

from taichi_dem_julia_port_gb300 import GlobalData, _abi, scenes
from taichi_dem_julia_port_gb300.config import DEMConfig
from taichi_dem_julia_port_gb300.scenes import ParticleInput

pytestmark = pytest.mark.gpu


def _cloud(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.002, 0.004, n)
    pos = rng.uniform(0.0, 0.3, (n, 3))
    cfg = DEMConfig(domain_min=[-0.05] * 3, domain_max=[0.35] * 3, max_coordinate_number=32)
    return cfg, ParticleInput.from_arrays(r, pos, np.zeros((n, 3)), 2500.0)


def _run_noalloc(lib, torch, p, derived, cfg):
    n = p.n
    pos = torch.tensor(p.pos, dtype=torch.float64, device="cuda")
    px, py, pz = (pos[:, k].contiguous() for k in range(3))
    bucket = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    order = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    dmin = (C.c_double * 3)(*cfg.domain_min)  # a host array, as the entry point reads it
    torch.cuda.synchronize()
    rc = lib.dem_bucket_sort_noalloc(px.data_ptr(), py.data_ptr(), pz.data_ptr(), n, dmin,
                                     derived["cell_size"], derived["hash_table_size"],
                                     bucket.data_ptr(), order.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == _abi.DEM_OK, lib.dem_strerror(rc)
    return (bucket.cpu().numpy().view(np.uint32).copy(),
            order.cpu().numpy().view(np.uint32).copy())


def test_noalloc_bucket_sort_matches_regular_broadphase(gpu):
    torch = pytest.importorskip("torch")
    lib = _abi.load_library()
    cases = [(scenes.bonded_cube(12, steps=0).cfg, scenes.bonded_cube(12, steps=0).particles),
             _cloud(20000, seed=4)]
    for cfg, p in cases:  # two calls in a row on the shared array
        g = GlobalData(cfg, p)
        ref = g.debug_broadphase(with_pairs=False)
        d = g.derived()
        g.close()
        bucket, order = _run_noalloc(lib, torch, p, d, cfg)
        np.testing.assert_array_equal(bucket, ref["bucket"])
        np.testing.assert_array_equal(order, ref["sorted"])


def test_noalloc_rejects_sizes_beyond_its_array(gpu):
    lib = _abi.load_library()
    dmin = (C.c_double * 3)(0.0, 0.0, 0.0)
    # no work is queued: the sizes are checked before any pointer is used
    rc = lib.dem_bucket_sort_noalloc(None, None, None, (1 << 20) + 1, dmin, 0.1, 1 << 20,
                                     None, None, None)
    assert rc == _abi.DEM_ERR_CAPACITY
    rc = lib.dem_bucket_sort_noalloc(None, None, None, 10, dmin, 0.1, (1 << 20) + 1,
                                     None, None, None)
    assert rc == _abi.DEM_ERR_CAPACITY


def _hashcode(pos, dmin, cell, H):
    """src/utils.jl:1-2 restated: ceil((x - dmin) / cell) per axis, then the
    1-based Morton code (x in bit 0) modulo H, plus 1."""
    from oracle import oracle as O
    ijk = np.ceil((pos - np.asarray(dmin)) / cell).astype(np.int64)
    return np.array([O.morton1(int(x), int(y), int(z)) % H + 1 for x, y, z in ijk], np.uint32)


@pytest.mark.parametrize("H,cell", [(3001, 0.013), (65537, 0.011), (1, 0.02), (1024, 0.5)])
def test_noalloc_small_tables_and_crowded_buckets(gpu, H, cell):
    """Tables the regular path never uses (any H from 1 up; non-powers of two
    take the modulo path, H = 1 and a cell as large as the domain put every
    particle in one bucket), against a restatement of hashcode and a stable
    argsort by bucket, twice in a row."""
    torch = pytest.importorskip("torch")
    lib = _abi.load_library()
    for seed in (7, 8):
        cfg, p = _cloud(20000, seed=seed)
        bucket, order = _run_noalloc(lib, torch, p, {"cell_size": cell, "hash_table_size": H},
                                     cfg)
        want = _hashcode(p.pos, cfg.domain_min, cell, H)
        np.testing.assert_array_equal(bucket, want)
        np.testing.assert_array_equal(order, np.argsort(want, kind="stable").astype(np.uint32))
