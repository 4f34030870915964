"""Scenes with their own material, surface and wall tables (dem_create_tables;
the reference's GlobalData.materials / surfaces / walls and Grain.mid, read
per contact at src/kernels.jl:175-177, 255-263 and per wall at
src/kernels.jl:317-426) against the CPU oracle with the same tables."""
import numpy as np
import pytest

from oracle.oracle import OracleScene
from taichi_dem_julia_port_gb300 import GlobalData, Material, Surface, Tables, Wall, scenes
from taichi_dem_julia_port_gb300._abi import DEM_ERR_INVALID, DemError
from tests.conftest import assert_rows_close
from tests.test_gpu_parity import (RTOL_HORIZON, RTOL_STEP, assert_runs_identical, bonded_set,
                                   compare_state, copy_state, pair_set, random_cloud,
                                   run_layouts)

pytestmark = pytest.mark.gpu


def two_material_tables(grain_material, walls):
    """Materials A, B (grains) and C (walls); every surface distinct."""
    mats = [Material(2500.0, 1e8, 0.30), Material(2700.0, 4e8, 0.22), Material(7800.0, 2e11, 0.25)]

    def bond(mu, e, ratio, E, nu, sc, st, ss):
        return Surface(mu, e, 0.0, ratio, E, nu, sc, st, ss)

    AA = bond(0.30, 0.90, 0.50, 1e8, 0.20, 1e7, 1e6, 1e6)
    AB = bond(0.50, 0.70, 0.40, 3e8, 0.25, 5e6, 4e5, 6e5)
    BB = bond(0.40, 0.80, 0.60, 5e8, 0.30, 2e7, 3e6, 3e6)
    AC, BC = Surface(0.35, 0.60), Surface(0.60, 0.50)
    CC = Surface(0.0, 0.0)
    surf = [[AA, AB, AC], [AB, BB, BC], [AC, BC, CC]]
    return Tables(mats, surf, walls, np.asarray(grain_material, np.int32))


def compare_walls(g, o, nwall, rtol, what):
    for w in range(nwall):
        assert_rows_close(g.wall_shear(w), o.wall_shear(w), rtol, f"{what} wall {w} shear",
                          atol_frac=rtol)


def test_standard_tables_equal_dem_create(gpu):
    """The reference's hard-coded tables through dem_create_tables give the
    same results as dem_create, bit for bit."""
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    a = GlobalData(sc.cfg, sc.particles)
    b = GlobalData(sc.cfg, sc.particles, tables=Tables.standard(sc.cfg, sc.particles))
    for g in (a, b):
        g.initialize()
        g.simulate(250)  # into the wall impact
    pa, pb = a.particles(), b.particles()
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
    ca, cb = a.contacts(), b.contacts()
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k], err_msg=k)
    assert np.abs(pa["wall_shear"]).sum() > 0
    a.close()
    b.close()


def test_rolling_resistance_declared_not_applied(gpu):
    """The reference declares the rolling-resistance coefficients
    (src/config.jl:26, 30; Surface.μᵣ, src/types.jl:20) and applies them in no
    force law (src/kernels.jl:170-426): results do not depend on them, whether
    they come through the config (dem_create) or the surface table
    (dem_create_tables), for bonds, Hertz contacts and wall contacts alike."""
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    cl_cfg, cl = random_cloud(1500, (0.03, 0.03, 0.03), 0.0008, 0.0015, seed=7, v=0.5)
    for cfg, p, steps, bond in ((sc.cfg, sc.particles, 250, True), (cl_cfg, cl, 100, False)):
        rr = cfg.replace(pp_coefficient_rolling_resistance=0.5,
                         pw_coefficient_rolling_resistance=0.3)
        t = Tables.standard(cfg, p)
        for row in t.surfaces:
            for s in row:
                s.rolling_resistance = 0.7
        runs = [GlobalData(cfg, p), GlobalData(rr, p), GlobalData(cfg, p, tables=t)]
        outs = []
        for g in runs:
            if bond:
                g.initialize()
            g.simulate(steps)
            outs.append((g.particles(), g.contacts()))
            g.close()
        for pa, ca in outs[1:]:
            for k in pa:
                np.testing.assert_array_equal(pa[k], outs[0][0][k], err_msg=k)
            for k in ca:
                np.testing.assert_array_equal(ca[k], outs[0][1][k], err_msg=k)
        c0 = outs[0][1]
        assert len(c0["i"]) > 0 and np.abs(outs[0][0]["wall_shear"]).sum() > 0
        assert c0["bonded"].all() if bond else not c0["bonded"].any()


def test_two_materials_two_walls_granular(gpu):
    """A polydisperse cloud of two materials thrown into the corner of two
    walls of a third material: Hertz-Mindlin per material pair and per wall,
    one step from an identical state, then a short horizon."""
    cfg, p = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=31, v=0.5,
                          cfg_kw=dict(domain_min=[-0.01] * 3, domain_max=[0.07] * 3))
    p.vel[:] += np.array([-1.0, 0.0, -1.0])
    rng = np.random.default_rng(31)
    gm = rng.integers(0, 2, p.n)
    walls = [Wall([0.0, 0.0, -1.0], 0.0, 2), Wall([-1.0, 0.0, 0.0], 0.0, 2)]
    t = two_material_tables(gm, walls)
    g, o = GlobalData(cfg, p, tables=t), OracleScene(cfg, p, tables=t)
    o.simulate(5)
    for _ in range(2):
        copy_state(o, g)
        for w in range(2):
            g.set_wall_shear(w, o.wall_shear(w))
        g.simulate(1)
        o.simulate(1)
        cg = compare_state(g, o, RTOL_STEP, "two materials one step")
        compare_walls(g, o, 2, RTOL_STEP, "two materials one step")
        assert len(cg["i"]) > 100
        o.simulate(20)
    # both walls touched by grains of both materials
    for w in range(2):
        touching = np.any(o.wall_shear(w) != 0, axis=1)
        assert set(gm[touching].tolist()) == {0, 1}, w
    g.close()


def test_two_materials_bonded_cube_two_walls(gpu):
    """A bonded cube of two materials (alternating layers: bonds A-A, A-B and
    B-B with their own radius ratio, modulus and strengths) thrown at an
    inclined wall and the floor: bond sets, breakage and forces over a
    horizon."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=12)
    cfg = sc.cfg
    z = sc.particles.pos[:, 2]
    layer = np.round((z - z.min()) / 0.02).astype(int)
    gm = layer % 2
    floor = Wall(list(cfg.wall_normal), cfg.wall_distance, 2)
    nrm = np.array([-1.0, 0.0, -1.0]) / np.sqrt(2.0)
    incline = Wall(nrm.tolist(), 0.0105, 2)  # 0.5 mm from the cube's lower front edge
    t = two_material_tables(gm, [floor, incline])
    g, o = GlobalData(cfg, sc.particles, tables=t), OracleScene(cfg, sc.particles, tables=t)
    g.initialize()
    o.initialize()
    cg, co = g.contacts(), o.contacts()
    assert bonded_set(cg) == bonded_set(co) and len(cg["i"]) == 3 * 8 * 8 * 7
    for _ in range(6):
        g.simulate(50)
        o.simulate(50)
        compare_state(g, o, RTOL_HORIZON, "two-material cube")
        compare_walls(g, o, 2, RTOL_HORIZON, "two-material cube")
    so, sg = o.stats(), g.stats()
    assert so["bonds_broken"] > 0 and sg["bonds_broken"] == so["bonds_broken"]
    assert pair_set(g.contacts()) == pair_set(o.contacts())
    g.close()


def test_tables_integrate_layouts_bit_identical(gpu):
    """A two-material cube against two walls: the integrator with one thread
    per particle and split over four warps give the same results bit for
    bit."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=12)
    cfg = sc.cfg
    z = sc.particles.pos[:, 2]
    gm = np.round((z - z.min()) / 0.02).astype(int) % 2
    nrm = np.array([-1.0, 0.0, -1.0]) / np.sqrt(2.0)
    t = two_material_tables(gm, [Wall(list(cfg.wall_normal), cfg.wall_distance, 2),
                                 Wall(nrm.tolist(), 0.0105, 2)])
    outs = run_layouts(cfg, sc.particles, 300, True, "integrate_lanes", tables=t)
    assert_runs_identical(outs, "two-material cube")
    assert outs[0][2]["bonds_broken"] > 0


def test_tables_reject_fp32_and_bad_indices(gpu):
    sc = scenes.bonded_cube(3, steps=0)
    t = two_material_tables(np.zeros(sc.n, np.int32), [Wall([0.0, 0.0, -1.0], 0.0, 2)])
    g = GlobalData(sc.cfg, sc.particles, tables=t)
    with pytest.raises(DemError) as e:
        g.set_precision("fp32")
    assert e.value.code == DEM_ERR_INVALID
    g.close()
    bad = two_material_tables(np.full(sc.n, 3, np.int32), [Wall([0.0, 0.0, -1.0], 0.0, 2)])
    with pytest.raises(DemError) as e:
        GlobalData(sc.cfg, sc.particles, tables=bad)
    assert e.value.code == DEM_ERR_INVALID and "grain 0" in str(e.value)
    badw = two_material_tables(np.zeros(sc.n, np.int32), [Wall([0.0, 0.0, -1.0], 0.0, 5)])
    with pytest.raises(DemError) as e:
        GlobalData(sc.cfg, sc.particles, tables=badw)
    assert e.value.code == DEM_ERR_INVALID
