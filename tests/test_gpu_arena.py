"""GPU: scenes in a shared arena give the results they give alone.

A scene stepped inside an arena (with other scenes, added or removed while it
runs, with a smaller search grid) must produce, bit for bit, the particle
state and contact list that a single-scene handle (dem_create) produces for
it; the single-scene handle is itself checked against the oracle in
test_gpu_parity.py, and one arena scene is checked against the oracle here."""
import numpy as np
import pytest

from oracle.oracle import OracleScene
from taichi_dem_julia_port_gb300 import Arena, GlobalData, scenes
from taichi_dem_julia_port_gb300._abi import DEM_ERR_CAPACITY, DemError
from tests.conftest import assert_rows_close

pytestmark = pytest.mark.gpu

PARTICLE_KEYS = ("pos", "vel", "omega", "quat", "force", "moment", "wall_shear")
CONTACT_KEYS = ("i", "j", "bonded", "point", "force", "torque_i", "torque_j", "shear")


def small_cube(side=5, speed=20.0, seed=1, **kw):
    sc = scenes.bonded_cube(side, speed=speed, steps=0, seed=seed, **kw)
    # strong impact on the wall right away: bonds stressed, Hertz contacts form
    sc.cfg = sc.cfg.replace(bond_tensile_strength=3e5, bond_shear_strength=3e5)
    return sc


def small_pour(n=600, seed=5, **kw):
    """Unbonded spheres with narrow gaps and 5 m/s random velocities: Hertz
    contacts form and end within tens of steps."""
    sc = scenes.granular_pour(n, box=(0.03, 0.03, 0.04), seed=seed, steps=0, rmin=0.8e-3,
                              rmax=1.2e-3, **kw)
    sc.cfg = sc.cfg.replace(dt=1e-6)
    pv = sc.particles.copy()
    rng = np.random.default_rng(seed)
    pv.vel = rng.normal(0, 5.0, pv.vel.shape)
    sc.particles = pv
    return sc


def alone(sc, steps, init=True, precision="fp64"):
    g = GlobalData(sc.cfg, sc.particles, precision=precision)
    if init:
        g.initialize()
    g.simulate(steps)
    out = (g.particles(), g.contacts(), g.stats())
    g.close()
    return out


def assert_same(arena, sid, ref, what):
    p, c = arena.particles(sid), arena.contacts(sid)
    rp, rc, _ = ref
    for k in PARTICLE_KEYS:
        np.testing.assert_array_equal(p[k], rp[k], err_msg=f"{what}: particles.{k}")
    assert len(c["i"]) == len(rc["i"]), f"{what}: contact count {len(c['i'])} vs {len(rc['i'])}"
    for k in CONTACT_KEYS:
        np.testing.assert_array_equal(c[k], rc[k], err_msg=f"{what}: contacts.{k}")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_scene_arena_equals_alone(gpu, precision):
    sc = small_cube()
    ref = alone(sc, 60, precision=precision)
    with Arena(4096, max_scenes=4, precision=precision) as a:
        s = a.add(sc.cfg, sc.particles)
        a.step(60)
        assert a.info(s)["steps_done"] == 60
        assert_same(a, s, ref, f"arena {precision}")
        st = a.stats(s)
        assert st["bonded"] == ref[2]["bonded"] and st["contacts"] == ref[2]["contacts"]
        assert st["bonds_broken"] == ref[2]["bonds_broken"]


def test_mixed_scenes_each_equal_alone(gpu):
    cube_a = small_cube(5, seed=1)
    cube_b = small_cube(6, speed=25.0, seed=2, E=5e8, friction=0.3)
    pour = small_pour(600, seed=7)
    steps = 80
    refs = [alone(cube_a, steps), alone(cube_b, steps), alone(pour, steps, init=False)]
    with Arena(8192, max_scenes=8) as a:
        ids = [a.add(cube_a.cfg, cube_a.particles), a.add(cube_b.cfg, cube_b.particles),
               a.add(pour.cfg, pour.particles, init_bonds=False)]
        a.step(steps)
        for sid, ref, name in zip(ids, refs, ("cube_a", "cube_b", "pour")):
            assert_same(a, sid, ref, name)
    # something happened: bonds in the cubes, Hertz contacts made and ended in the pour
    assert refs[0][2]["bonded"] > 0
    assert refs[2][2]["contacts"] > 0 and refs[2][2]["contacts_ended"] > 0


def test_scenes_join_and_leave_while_running(gpu):
    """Continuous batching: A runs; B joins after 30 steps; A leaves; C takes
    A's freed slots (C is no larger than A).  B and C match their alone runs."""
    A, B, C = small_cube(5, seed=11), small_cube(5, speed=15.0, seed=12), small_pour(120, seed=13)
    ref_b = alone(B, 70)
    ref_c = alone(C, 40, init=False)
    with Arena(4096, max_scenes=4) as a:
        sa = a.add(A.cfg, A.particles)
        a.step(30)
        sb = a.add(B.cfg, B.particles)
        a.step(30)
        first_a = a.info(sa)["first_slot"]
        a.remove(sa)
        sc_ = a.add(C.cfg, C.particles, init_bonds=False)
        assert a.info(sc_)["first_slot"] == first_a, "C should reuse A's slots"
        a.step(40)
        assert_same(a, sb, ref_b, "B")
        assert_same(a, sc_, ref_c, "C")


def test_step_target_freezes_scene(gpu):
    sc = small_cube(5, seed=21)
    ref = alone(sc, 25)
    with Arena(2048, max_scenes=2) as a:
        s = a.add(sc.cfg, sc.particles, steps=25)
        a.step(40)
        info = a.info(s)
        assert info["mode"] == "frozen" and info["steps_done"] == 25
        assert_same(a, s, ref, "frozen at target")


def test_smaller_search_cells_same_results(gpu):
    """cell_factor < 1: a finer search grid, the reference's cp_list rules
    still decide contact ends, so every result is unchanged."""
    cube, pour = small_cube(6, seed=31), small_pour(800, seed=32)
    steps = 60
    refs = [alone(cube, steps), alone(pour, steps, init=False)]
    with Arena(4096, max_scenes=4, cell_factor=0.3) as a:
        ids = [a.add(cube.cfg, cube.particles), a.add(pour.cfg, pour.particles, init_bonds=False)]
        a.step(steps)
        for sid, ref, name in zip(ids, refs, ("cube", "pour")):
            assert_same(a, sid, ref, f"fine grid {name}")


def test_arena_scene_against_oracle(gpu):
    sc = small_cube(5, seed=41)
    o = OracleScene(sc.cfg, sc.particles)
    o.initialize()
    o.simulate(40)
    with Arena(2048, max_scenes=2, cell_factor=0.5) as a:
        s = a.add(sc.cfg, sc.particles)
        a.step(40)
        cg, co = a.contacts(s), o.contacts()
        assert set(zip(cg["i"].tolist(), cg["j"].tolist())) == \
            set(zip(co["i"].tolist(), co["j"].tolist()))
        pg, po = a.particles(s), o.particles()
        assert_rows_close(pg["pos"], po["pos"], 1e-9, "pos")
        assert_rows_close(pg["force"], po["force"], 1e-5, "force", atol_frac=1e-5)


def test_arena_capacity_errors(gpu):
    sc = small_cube(5)  # 125 particles
    with Arena(130, max_scenes=4) as a:
        a.add(sc.cfg, sc.particles)
        with pytest.raises(DemError) as e:
            a.add(sc.cfg, sc.particles)  # no particle slots left
        assert e.value.code == DEM_ERR_CAPACITY
    with Arena(1000, max_scenes=1) as a:
        a.add(sc.cfg, sc.particles)
        with pytest.raises(DemError) as e:
            a.add(sc.cfg, sc.particles)  # no scene record left
        assert e.value.code == DEM_ERR_CAPACITY


def test_arena_empty_steps(gpu):
    pour = small_pour(100, seed=3)
    ref = alone(pour, 3, init=False)
    with Arena(1024, max_scenes=2) as a:
        a.step(5)  # nothing to step
        a.sync()
        s = a.add(pour.cfg, pour.particles, init_bonds=False)
        a.step(3)
        assert a.info(s)["steps_done"] == 3
        assert_same(a, s, ref, "after empty steps")


def test_tuning_knobs_keep_results(gpu):
    """Launch shape and search-cell changes in the middle of a run (what the
    autotuner does) leave every result unchanged."""
    cube, pour = small_cube(5, seed=51), small_pour(400, seed=52)
    refs = [alone(cube, 40), alone(pour, 40, init=False)]
    with Arena(4096, max_scenes=4) as a:
        ids = [a.add(cube.cfg, cube.particles), a.add(pour.cfg, pour.particles, init_bonds=False)]
        a.step(15)
        a.set_launch_shape(force_block=128, force_grid=152 * 4, compact_block=64,
                           compact_grid=152 * 2, integrate_block=128, list_lanes=1,
                           integrate_lanes=1)
        a.set_cell_factor(0.4)
        a.step(15)
        a.set_cell_factor(0.7, scene=ids[0])
        a.set_launch_shape(force_block=256, force_grid=152 * 32, integrate_block=256,
                           dependent_launch=2, list_lanes=4, integrate_lanes=4)
        a.step(10)
        for sid, ref, name in zip(ids, refs, ("cube", "pour")):
            assert_same(a, sid, ref, f"retuned {name}")
    g = GlobalData(cube.cfg, cube.particles)
    g.initialize()
    g.simulate(20)
    g.set_launch_shape(force_block=96, force_grid=100, compact_grid=50, integrate_block=64,
                       dependent_launch=1)
    g.simulate(10)
    g.set_launch_shape(dependent_launch=2, list_lanes=1, integrate_lanes=1)
    g.simulate(10)
    p, c = g.particles(), g.contacts()
    for k in PARTICLE_KEYS:
        np.testing.assert_array_equal(p[k], refs[0][0][k], err_msg=f"single retuned {k}")
    np.testing.assert_array_equal(c["force"], refs[0][1]["force"])


def test_neighbour_lists_equal_full_search(gpu):
    """Steps that test neighbour lists give the results of a full pair search
    every step (skin factor 0), bit for bit, while the scenes move enough to
    rebuild their lists several times."""
    cube = small_cube(6, speed=40.0, seed=61)
    pour = small_pour(600, seed=62)
    steps = 150

    def run(skin):
        out = []
        for sc, init in ((cube, True), (pour, False)):
            g = GlobalData(sc.cfg, sc.particles)
            g.set_skin_factor(skin)
            if init:
                g.initialize()
            g.simulate(steps)
            out.append((g.particles(), g.contacts(), g.stats()))
            g.close()
        return out

    full, lists = run(0.0), run(0.9)
    for (pf, cf, sf), (pl, cl, sl), name in zip(full, lists, ("cube", "pour")):
        for k in PARTICLE_KEYS:
            np.testing.assert_array_equal(pl[k], pf[k], err_msg=f"{name} {k}")
        for k in CONTACT_KEYS:
            np.testing.assert_array_equal(cl[k], cf[k], err_msg=f"{name} contacts {k}")
        assert sf["full_searches"] == steps, (name, sf["full_searches"])
        assert 1 <= sl["full_searches"] < steps, (name, sl["full_searches"])
        assert sl["contacts_ended"] == sf["contacts_ended"]
    assert full[1][2]["contacts_created"] > 0 and full[1][2]["contacts_ended"] > 0
    # the same inside an arena, with per-scene skins
    with Arena(4096, max_scenes=4) as a:
        ids = [a.add(cube.cfg, cube.particles), a.add(pour.cfg, pour.particles, init_bonds=False)]
        a.set_skin_factor(0.5, scene=ids[1])
        a.step(steps)
        for sid, ref, name in zip(ids, full, ("cube", "pour")):
            assert_same(a, sid, ref, f"arena lists {name}")


def test_state_exchange_every_step(gpu):
    """Reading the state into page-locked arrays and writing it back every
    step (the end-to-end loop) leaves the run bit-identical to uninterrupted
    stepping, and does not force full searches while nothing moved."""
    import torch
    sc = small_pour(800, seed=71)
    steps = 40
    ref = GlobalData(sc.cfg, sc.particles)
    ref.simulate(steps)
    want = (ref.particles(), ref.contacts(), ref.stats())
    ref.close()
    g = GlobalData(sc.cfg, sc.particles)
    keys = ("pos", "vel", "omega", "quat", "wall_shear")
    host = {k: torch.empty((sc.n, 4 if k == "quat" else 3), dtype=torch.float64,
                           pin_memory=True).numpy() for k in keys}
    for _ in range(steps):
        g.particles(out=host)
        g.set_particles(**host)
        g.simulate(1)
    got = (g.particles(), g.contacts(), g.stats())
    for k in PARTICLE_KEYS:
        np.testing.assert_array_equal(got[0][k], want[0][k], err_msg=k)
    for k in CONTACT_KEYS:
        np.testing.assert_array_equal(got[1][k], want[1][k], err_msg=f"contacts {k}")
    assert got[2]["full_searches"] == want[2]["full_searches"] < steps
    out = {"pos": np.empty((sc.n, 4))}
    with pytest.raises(ValueError):
        g.particles(out=out)
    g.close()


def test_set_particles_far_move_searches(gpu):
    """Positions written from the host that leave the skin trigger a full
    search: results equal a handle that searches every step."""
    sc = small_pour(800, seed=72)
    runs = []
    for skin in (0.0, 0.9):
        g = GlobalData(sc.cfg, sc.particles)
        g.set_skin_factor(skin)
        g.simulate(10)
        st = g.particles()
        pos = st["pos"].copy()
        pos[::7] += np.array([3e-4, -2e-4, 1e-4])  # beyond half a skin (~0.1 mm)
        g.set_particles(pos=pos)
        s0 = g.stats()["full_searches"]
        g.simulate(1)
        assert g.stats()["full_searches"] == s0 + 1
        g.simulate(19)
        runs.append((g.particles(), g.contacts(), g.stats()))
        g.close()
    (pf, cf, sf), (pl, cl, sl) = runs
    for k in PARTICLE_KEYS:
        np.testing.assert_array_equal(pl[k], pf[k], err_msg=k)
    for k in CONTACT_KEYS:
        np.testing.assert_array_equal(cl[k], cf[k], err_msg=f"contacts {k}")
    assert sl["full_searches"] < sf["full_searches"]


def test_state_exchange_device_buffers(gpu):
    """dem_get_particles / dem_set_particles with device buffers (written and
    read in place) agree with pageable host buffers."""
    import ctypes as C
    import torch
    from taichi_dem_julia_port_gb300 import _abi
    sc = small_pour(700, seed=73)
    g = GlobalData(sc.cfg, sc.particles)
    g.simulate(12)
    want = g.particles()
    dev = {k: torch.empty((sc.n, 4 if k == "quat" else 3), dtype=torch.float64, device="cuda")
           for k in PARTICLE_KEYS}
    dptr = {k: t.data_ptr() for k, t in dev.items()}
    st = _abi.DemParticleState(sc.n, *(dptr[k] for k in PARTICLE_KEYS))
    assert g.lib.dem_get_particles(g.h, C.byref(st)) == 0
    torch.cuda.synchronize()
    for k in PARTICLE_KEYS:
        np.testing.assert_array_equal(dev[k].cpu().numpy(), want[k], err_msg=k)
    # write back a changed velocity from the device and read it through the host path
    dev["vel"].mul_(0.5)
    torch.cuda.synchronize()
    st_in = _abi.DemParticleState(sc.n, None, dptr["vel"], None, None, None, None, None)
    assert g.lib.dem_set_particles(g.h, C.byref(st_in)) == 0
    np.testing.assert_array_equal(g.particles()["vel"], 0.5 * want["vel"])
    g.close()


def test_state_buffers_loop(gpu):
    """StateBuffers (page-locked arrays, asynchronous upload): the exchange
    loop is bit-identical to uninterrupted stepping, and a change written into
    the arrays reaches the device."""
    sc = small_pour(800, seed=74)
    steps = 30
    ref = GlobalData(sc.cfg, sc.particles)
    ref.simulate(steps)
    want = ref.particles()
    ref.close()
    g = GlobalData(sc.cfg, sc.particles)
    buf = g.state_buffers()
    for s_ in range(steps):
        if s_ % 2:
            buf.upload()
            g.simulate(1)
            buf.download()
        else:
            buf.step(1)
    for k in ("pos", "vel", "omega", "quat", "wall_shear"):
        np.testing.assert_array_equal(getattr(buf, k), want[k], err_msg=k)
    buf.vel[:] *= 0.25
    expect = buf.vel.copy()
    buf.upload()
    np.testing.assert_array_equal(g.particles()["vel"], expect)
    buf.close()
    g.close()


@pytest.mark.slow
def test_full_size_pour_properties(gpu):
    """The 2,000,000-sphere pour at full size, FP32 force mode: two runs are
    bit-identical, and the neighbour-list schedule gives the results of a
    full pair search every step."""
    sc = scenes.c3()
    steps = 12
    runs = []
    for skin in (0.9, 0.9, 0.0):
        g = GlobalData(sc.cfg, sc.particles, precision="fp32")
        g.set_skin_factor(skin)
        g.simulate(steps)
        st = g.stats()
        assert st["error"] == 0
        runs.append((g.particles(forces=False), st))
        g.close()
    for k in ("pos", "vel", "omega", "quat"):
        np.testing.assert_array_equal(runs[0][0][k], runs[1][0][k], err_msg=f"rerun {k}")
        np.testing.assert_array_equal(runs[0][0][k], runs[2][0][k], err_msg=f"lists {k}")
    assert runs[2][1]["full_searches"] == steps
    assert runs[0][1]["full_searches"] < steps


def test_list_update_large_scenes(gpu):
    """Scenes with more particles than one pass of the list update's 4-lane
    groups: a sparse 64,000-sphere pour (fewer contacts than a quarter of its
    particles: the wide pass, which reads 32 particles per warp and hands only
    those with contacts or list partners to the groups) and a 64,000-sphere
    bonded cube (dense: the per-group pass).  Their neighbour-list steps give
    the results of a full pair search every step, bit for bit, while contacts
    form and end (the pour) and an impact breaks bonds (the cube); the pour
    gives the same results inside an arena with a small cube."""
    pour = scenes.granular_pour(64_000, box=(0.14, 0.14, 0.19), seed=83, steps=0, rmin=0.8e-3,
                                rmax=1.2e-3)
    pour.cfg = pour.cfg.replace(dt=1e-6)
    pv = pour.particles.copy()
    pv.vel = np.random.default_rng(83).normal(0, 5.0, pv.vel.shape)
    pour.particles = pv
    cube = small_cube(40, speed=40.0, seed=81)
    # weak in compression too: the impact face breaks before the wave returns
    cube.cfg = cube.cfg.replace(bond_compressive_strength=3e5)
    steps = 150

    def run(sc, init, skin):
        g = GlobalData(sc.cfg, sc.particles)
        g.set_skin_factor(skin)
        if init:
            g.initialize()
        g.simulate(steps)
        out = (g.particles(), g.contacts(), g.stats())
        g.close()
        return out

    fulls = []
    for sc, init, name in ((pour, False, "pour"), (cube, True, "cube")):
        full, lists = run(sc, init, 0.0), run(sc, init, 0.9)
        for k in PARTICLE_KEYS:
            np.testing.assert_array_equal(lists[0][k], full[0][k], err_msg=f"{name} lists {k}")
        for k in CONTACT_KEYS:
            np.testing.assert_array_equal(lists[1][k], full[1][k],
                                          err_msg=f"{name} lists contacts {k}")
        assert full[2]["full_searches"] == steps
        assert 1 <= lists[2]["full_searches"] < steps, (name, lists[2]["full_searches"])
        for k in ("bonds_broken", "contacts_created", "contacts_ended"):
            assert lists[2][k] == full[2][k], (name, k)
        fulls.append(full)
    assert fulls[0][2]["contacts_created"] > 0 and fulls[0][2]["contacts_ended"] > 0
    assert len(fulls[0][1]["i"]) * 4 < pour.n
    assert fulls[1][2]["bonds_broken"] > 0
    # an arena whose contacts stay sparse (the pour and a small cube) takes
    # the wide pass too
    small = small_cube(5, seed=84)
    small_ref = alone(small, steps)
    with Arena(pour.n + 4096, max_scenes=2) as a:
        ids = [a.add(pour.cfg, pour.particles, init_bonds=False), a.add(small.cfg, small.particles)]
        a.step(steps)
        assert_same(a, ids[0], fulls[0], "arena pour")
        assert_same(a, ids[1], small_ref, "arena small cube")


def test_stats_counts_equal_the_contact_read(gpu):
    """dem_get_stats counts a scene's active contacts and bonds on the device:
    they equal the counts of the full contact read, for a single scene and for
    each scene of an arena (bonds broken, Hertz contacts, scenes side by side)."""
    cube = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    g = GlobalData(cube.cfg, cube.particles)
    g.initialize()
    g.simulate(1000)  # bonds start to break near step 900
    st, c = g.stats(), g.contacts()
    assert st["bonds_broken"] > 0 and np.count_nonzero(c["bonded"] == 0) > 0
    assert st["contacts"] == len(c["i"]) and st["bonded"] == int(np.count_nonzero(c["bonded"]))
    g.close()
    with Arena(20000, max_scenes=4) as a:
        ids = [a.add(small_cube().cfg, small_cube().particles),
               a.add(cube.cfg, cube.particles),
               a.add(small_pour(800, seed=74).cfg, small_pour(800, seed=74).particles,
                     init_bonds=False)]
        a.step(1000)
        for s in ids:
            st, c = a.stats(s), a.contacts(s)
            assert st["contacts"] == len(c["i"]), s
            assert st["bonded"] == int(np.count_nonzero(c["bonded"])), s
        assert a.stats(ids[1])["bonds_broken"] > 0
        assert a.stats(ids[2])["contacts"] > 0
