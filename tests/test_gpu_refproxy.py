"""The reference-structured GPU proxy (the stand-in timed beside the library
for the reference's CUDA.jl path) computes the reference step: contact and
bond sets equal to the CPU oracle's, positions and velocities within the
short-horizon tolerance."""
import numpy as np
import pytest

from oracle.oracle import OracleScene
from taichi_dem_julia_port_gb300 import scenes
from tests.conftest import assert_rows_close
from tests.test_gpu_parity import bonded_set, pair_set, random_cloud

pytestmark = pytest.mark.gpu

RTOL = 1e-5  # FP64 atomics in a free order: the short-horizon bound


@pytest.fixture(scope="module")
def proxy(gpu):
    from baseline import refproxy
    refproxy.build()
    return refproxy


def compare(p, o, what):
    cp, co = p.contacts(), o.contacts()
    assert len(cp["i"]) == len(pair_set(cp)), f"{what}: duplicate contacts"
    assert pair_set(cp) == pair_set(co), f"{what}: contact sets differ"
    assert bonded_set(cp) == bonded_set(co), f"{what}: bond sets differ"
    sp, so = p.particles(), o.particles()
    assert_rows_close(sp["pos"], so["pos"], RTOL, f"{what} pos")
    assert_rows_close(sp["vel"], so["vel"], RTOL, f"{what} vel", atol_frac=RTOL)


def test_proxy_bonded_cube_impact(proxy):
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    p, o = proxy.RefProxy(sc.cfg, sc.particles), OracleScene(sc.cfg, sc.particles)
    p.initialize()
    o.initialize()
    assert bonded_set(p.contacts()) == bonded_set(o.contacts())
    for _ in range(3):
        p.simulate(60)
        o.simulate(60)
        compare(p, o, "cube")
    assert len(o.contacts()["i"]) > 0
    p.close()


def test_proxy_granular_cloud(proxy):
    cfg, parts = random_cloud(1500, (0.04, 0.04, 0.04), 0.0008, 0.0015, seed=9, v=0.5,
                              cfg_kw=dict(pp_coefficient_friction=0.3))
    p, o = proxy.RefProxy(cfg, parts), OracleScene(cfg, parts)
    for _ in range(3):
        p.simulate(10)
        o.simulate(10)
        compare(p, o, "cloud")
    s = o.stats()
    assert s["contacts_created"] > 0 and s["contacts_ended"] > 0
    t = p.simulate_timed(5)
    assert t > 0.0
    p.close()


def test_proxy_rejects_oversized_bit_tables(proxy):
    sc = scenes.bonded_cube(41, steps=0)  # 68,921 spheres: BitTables past 512 MiB each
    with pytest.raises(ValueError):
        proxy.RefProxy(sc.cfg, sc.particles)
