"""GPU parity: the CUDA DEM step (through the C ABI) against the CPU oracle.

Bit-exact: cell ijk, Morton codes, buckets, bucket counts, sorted order, the
cp_list multiset, contact sets and bond sets.  Within tolerance: forces,
positions and velocities (FP64: rtol 1e-9 for one step from an identical
state, 1e-5 over a short horizon; FP32 force mode: 1e-3)."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle.oracle import OracleScene, host_threads
from taichi_dem_julia_port_gb300 import GlobalData, scenes
from taichi_dem_julia_port_gb300.executor import enumeration_checksum
from taichi_dem_julia_port_gb300._abi import DEM_ERR_CAPACITY, DemError
from taichi_dem_julia_port_gb300.config import DEMConfig
from taichi_dem_julia_port_gb300.scenes import ParticleInput
from tests.conftest import assert_rows_close

pytestmark = pytest.mark.gpu

RTOL_STEP = 1e-9      # one step from an identical state (FP64)
RTOL_HORIZON = 1e-5   # short horizon (FP64): the stated force bound of the FP64 path
RTOL_FP32 = 1e-3      # FP32 force mode vs the FP64 oracle


def pair_set(c):
    return set(zip(c["i"].tolist(), c["j"].tolist()))


def bonded_set(c):
    b = c["bonded"].astype(bool)
    return set(zip(c["i"][b].tolist(), c["j"][b].tolist()))


def random_cloud(n, box, rmin, rmax, seed, v=0.0, cfg_kw=None):
    rng = np.random.default_rng(seed)
    r = rng.uniform(rmin, rmax, n)
    pos = rng.uniform(0, 1, (n, 3)) * np.asarray(box)
    vel = rng.normal(0, v, (n, 3)) if v else np.zeros((n, 3))
    kw = dict(domain_min=[-0.02] * 3, domain_max=(np.asarray(box) + 0.02).tolist(),
              max_coordinate_number=64, wall_distance=0.0, gravity=[0.0, 0.0, -9.81],
              dt=1e-6, particle_elastic_modulus=1e8, bond_elastic_modulus=1e8,
              bond_tensile_strength=1e6, bond_shear_strength=1e6)
    kw.update(cfg_kw or {})
    return DEMConfig(**kw), ParticleInput.from_arrays(r, pos, vel, 2500.0)


def both(cfg, p, precision="fp64", threads=1):
    return GlobalData(cfg, p, precision=precision), OracleScene(cfg, p, threads=threads)


def copy_state(o, g):
    """The oracle's particle and contact state onto the GPU handle."""
    p, c = o.particles(), o.contacts()
    g.set_particles(pos=p["pos"], vel=p["vel"], omega=p["omega"], quat=p["quat"],
                    wall_shear=p["wall_shear"])
    g.set_contacts(c)


def compare_broadphase(g, o):
    a, b = g.debug_broadphase(), o.debug_broadphase()
    for k in ("cell", "morton", "bucket", "bucket_count", "sorted"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert a["cp_count"] == b["cp_count"]
    ca = a["cp"][np.lexsort((a["cp"][:, 1], a["cp"][:, 0]))]
    cb = b["cp"][np.lexsort((b["cp"][:, 1], b["cp"][:, 0]))]
    np.testing.assert_array_equal(ca, cb)
    return a


def compare_state(g, o, rtol, what=""):
    cg, co = g.contacts(), o.contacts()
    assert pair_set(cg) == pair_set(co), f"{what}: contact sets differ"
    assert bonded_set(cg) == bonded_set(co), f"{what}: bond sets differ"
    pg, po = g.particles(), o.particles()
    assert_rows_close(pg["pos"], po["pos"], rtol, f"{what} pos")
    assert_rows_close(pg["vel"], po["vel"], rtol, f"{what} vel")
    assert_rows_close(pg["force"], po["force"], rtol, f"{what} force", atol_frac=rtol)
    assert_rows_close(pg["moment"], po["moment"], rtol, f"{what} moment", atol_frac=rtol)
    assert_rows_close(pg["omega"], po["omega"], rtol, f"{what} omega", atol_frac=rtol)
    assert_rows_close(pg["quat"], po["quat"], rtol, f"{what} quat")
    assert_rows_close(cg["force"], co["force"], rtol, f"{what} contact force", atol_frac=rtol)
    assert_rows_close(cg["shear"], co["shear"], rtol, f"{what} shear", atol_frac=rtol)
    assert_rows_close(cg["point"], co["point"], rtol, f"{what} point")
    return cg


# ---- broad phase ---------------------------------------------------------------------

@pytest.mark.parametrize("side", [3, 10, 26])
def test_broadphase_lattice_bitexact(gpu, side):
    sc = scenes.bonded_cube(side, steps=0)
    g, o = both(sc.cfg, sc.particles)
    a = compare_broadphase(g, o)
    assert a["cp_count"] > 0


def test_broadphase_hash_collisions_bitexact(gpu):
    """A wide domain so Morton codes exceed H and buckets collide (non-power
    of two H, so neighbour buckets may coincide too)."""
    cfg, p = random_cloud(4000, (3.9, 3.9, 3.9), 0.004, 0.006, seed=3,
                          cfg_kw=dict(domain_max=[4.0, 4.0, 4.0]))
    g, o = both(cfg, p)
    H = g.derived()["hash_table_size"]
    assert H & (H - 1) != 0, "want a non power-of-two table"
    a = compare_broadphase(g, o)
    assert a["morton"].max() > H


def test_broadphase_outside_domain_bitexact(gpu):
    """Particles below domain_min (cells <= 0) and on exact cell boundaries."""
    cfg, p = random_cloud(500, (0.2, 0.2, 0.2), 0.005, 0.01, seed=9)
    g0, _ = both(cfg, p)
    cs = g0.derived()["cell_size"]
    g0.close()
    pos = p.pos.copy()
    pos[:50] -= 0.5
    pos[50:100] = np.asarray(cfg.domain_min) + np.round(pos[50:100] / cs) * cs
    q = ParticleInput.from_arrays(np.cbrt(p.volume / (4 / 3 * np.pi)), pos, p.vel, 2500.0)
    g, o = both(cfg, q)
    compare_broadphase(g, o)


# ---- contacts --------------------------------------------------------------------------

@pytest.mark.parametrize("side", [3, 10, 26])
def test_init_bonds_bitexact(gpu, side):
    sc = scenes.bonded_cube(side, steps=0)
    g, o = both(sc.cfg, sc.particles)
    g.initialize()
    o.initialize()
    cg, co = g.contacts(), o.contacts()
    assert pair_set(cg) == pair_set(co)
    assert bonded_set(cg) == bonded_set(co)
    assert len(cg["i"]) == 3 * side * side * (side - 1)


def test_one_step_from_identical_state_cube(gpu):
    """Run the oracle into the impact, copy its state to the GPU, step both."""
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    g, o = both(sc.cfg, sc.particles)
    o.initialize()
    o.simulate(160)  # past first wall contact at ~100 steps
    for _ in range(3):
        p, c = o.particles(), o.contacts()
        g.set_particles(pos=p["pos"], vel=p["vel"], omega=p["omega"], quat=p["quat"],
                        wall_shear=p["wall_shear"])
        g.set_contacts(c)
        g.simulate(1)
        o.simulate(1)
        compare_state(g, o, RTOL_STEP, "cube one step")
        o.simulate(40)


def test_one_step_from_identical_state_granular(gpu):
    """Overlapping random cloud: Hertz contacts created, ended and sliding."""
    cfg, p = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=5, v=0.5,
                          cfg_kw=dict(pp_coefficient_friction=0.3))
    g, o = both(cfg, p)
    o.simulate(5)
    for _ in range(3):
        pp, c = o.particles(), o.contacts()
        g.set_particles(pos=pp["pos"], vel=pp["vel"], omega=pp["omega"], quat=pp["quat"],
                        wall_shear=pp["wall_shear"])
        g.set_contacts(c)
        g.simulate(1)
        o.simulate(1)
        cg = compare_state(g, o, RTOL_STEP, "granular one step")
        assert len(cg["i"]) > 100
        o.simulate(10)
    s = o.stats()
    assert s["contacts_created"] > 0 and s["contacts_ended"] > 0


def test_step_enumeration_visits_cp_list(gpu):
    """The step's own fused pair enumeration (8 lanes per particle over its
    octant buckets, repeated buckets skipped, entries above i by binary
    search) visits exactly the distinct pairs of the reference's cp_list, on
    a lattice, on a random cloud, and with colliding hash buckets."""
    sc = scenes.bonded_cube(10, steps=0)
    cloud = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=5, v=0.5)
    wide = random_cloud(4000, (3.9, 3.9, 3.9), 0.004, 0.006, seed=3,
                        cfg_kw=dict(domain_max=[4.0, 4.0, 4.0]))
    for cfg, p in ((sc.cfg, sc.particles), cloud, wide):
        g = GlobalData(cfg, p)
        g.simulate(3)
        bp = g.debug_broadphase()
        distinct = np.unique(bp["cp"], axis=0)
        pairs, chk = g.debug_step_enumeration()
        assert pairs == len(distinct), (pairs, len(distinct), bp["cp_count"])
        assert chk == enumeration_checksum(distinct)
        assert g.stats()["error"] == 0
        g.close()


def test_global_damping_one_step_and_horizon(gpu):
    """apply_body_force!'s damping term -d·|F|·sign(v) (src/kernels.jl:436-441)
    with a nonzero coefficient: one step from an identical state of a granular
    cloud whose grains have velocity or spin components that are exactly zero
    (sign(0) = 0) as well as moving and spinning ones; then a bonded cube's
    impact with damping over a 200-step horizon.  (A horizon on the granular
    cloud is not a parity test: sign(v) of a velocity component passing
    through zero turns rounding differences into O(1) force differences, and
    the dense cloud's collisions amplify them.)"""
    cfg, p = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=15, v=0.5,
                          cfg_kw=dict(global_damping=0.3, pp_coefficient_friction=0.3))
    rng = np.random.default_rng(15)
    g, o = both(cfg, p)
    o.simulate(5)
    pp = o.particles()
    vel, omega = pp["vel"].copy(), rng.normal(0, 50.0, (p.n, 3))
    for k in range(0, p.n, 7):
        vel[k, k % 3] = 0.0
        omega[k, (k + 1) % 3] = 0.0
    vel[::11] = 0.0
    omega[::13] = 0.0
    o.set_particles(vel=vel, omega=omega)
    copy_state(o, g)
    g.simulate(1)
    o.simulate(1)
    compare_state(g, o, RTOL_STEP, "damping one step")
    g.close()
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    cfg = sc.cfg.replace(global_damping=0.2)
    g, o = both(cfg, sc.particles)
    g.initialize()
    o.initialize()
    for _ in range(4):
        g.simulate(50)
        o.simulate(50)
        compare_state(g, o, RTOL_HORIZON, "damped cube horizon")
    assert np.count_nonzero(np.any(o.particles()["wall_shear"] != 0, axis=1)) > 0


def test_full_size_cube_mid_impact(gpu):
    """The 17,576-sphere bonded cube at 20 m/s in its fragmentation (the GPU
    runs the first 3,800 steps; the oracle joins from the GPU's state): one
    step from that identical state — wall contacts, Hertz contacts between
    fragments and bonds breaking — then a 200-step horizon."""
    sc = scenes.c2()
    g, o = both(sc.cfg, sc.particles, threads=host_threads())
    g.initialize()
    g.simulate(3800)
    copy_state(g, o)
    g.simulate(1)
    o.simulate(1)
    cg = compare_state(g, o, RTOL_STEP, "c2 one step")
    pg = g.particles()
    assert np.count_nonzero(np.any(pg["wall_shear"] != 0, axis=1)) > 100
    assert np.count_nonzero(cg["bonded"] == 0) > 1000  # Hertz contacts between fragments
    b0 = o.stats()["bonds_broken"]
    for _ in range(4):
        g.simulate(50)
        o.simulate(50)
        compare_state(g, o, RTOL_HORIZON, "c2 horizon")
    assert o.stats()["bonds_broken"] > b0  # bonds broke inside the compared horizon
    assert g.stats()["error"] == 0


@pytest.mark.parametrize("precision,rtol", [("fp64", RTOL_STEP), ("fp32", RTOL_FP32)])
def test_polydisperse_bed_one_step(gpu, precision, rtol):
    """100,000 spheres with the 2,000,000-sphere pour's radii (lognormal,
    median 1 mm, σ 0.25, clipped to [0.5, 2] mm) pre-compacted into touching
    columns on the floor: one step from an identical state with about one
    Hertz contact per sphere, FP64 (rtol 1e-9) and the FP32 force mode
    (1e-3 against the FP64 oracle)."""
    f = 2.0 * (100_000 / 2_000_000) ** (1.0 / 3.0)
    sc = scenes.granular_bed(100_000, box=(0.4 * f, 0.4 * f, 1.2), seed=21)
    g, o = both(sc.cfg, sc.particles, precision=precision, threads=host_threads())
    o.simulate(20)
    copy_state(o, g)
    g.simulate(1)
    o.simulate(1)
    cg, co = g.contacts(), o.contacts()
    assert len(co["i"]) > 80_000
    if precision == "fp64":
        compare_state(g, o, rtol, "bed one step")
    else:
        assert pair_set(cg) == pair_set(co)
        assert_rows_close(cg["force"], co["force"], rtol, "bed fp32 contact force", atol_frac=rtol)
        pg, po = g.particles(), o.particles()
        assert_rows_close(pg["force"], po["force"], rtol, "bed fp32 force", atol_frac=rtol)
        assert_rows_close(pg["pos"], po["pos"], 1e-9, "bed fp32 pos")


def _boundary_pairs(npair, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.004, 0.006, 2 * npair)
    side = int(np.ceil(npair ** (1.0 / 3.0)))
    ijk = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:npair]
    centres = (ijk + 0.5) * 0.05
    dirs = rng.standard_normal((npair, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    return r, centres, dirs


def _place(r, centres, dirs, rel):
    """Pair k's spheres at separation (r_a + r_b)(1 + rel[k]) along dirs[k]."""
    sep = (r[0::2] + r[1::2]) * (1.0 + rel)
    pos = np.empty((2 * len(centres), 3))
    pos[0::2] = centres - dirs * (sep / 2)[:, None]
    pos[1::2] = centres + dirs * (sep / 2)[:, None]
    return pos


def test_touching_decisions_at_the_boundary(gpu):
    """Pairs placed at separations (rᵢ + rⱼ)(1 + δ), |δ| from 1e-6 down to
    1e-14 either side of touching: the contacts the neighbour-list step
    creates, and then keeps or ends, equal the oracle's (the FP32 screens
    decide only pairs whose outcome they can prove).  An overlap of exactly
    zero is left out: the reference's Hertz-Mindlin formulas divide 0 by 0
    there (a new contact with zero overlap has zero normal and shear force,
    and the sliding test 0 >= μ·0 takes the ratio branch), so every
    implementation of them gives NaN."""
    npair = 512
    r, centres, dirs = _boundary_pairs(npair, seed=5)
    deltas = np.array([-1e-6, -1e-8, -1e-10, -1e-12, -1e-13, -1e-14, 1e-14, 1e-13, 1e-12, 1e-10,
                       1e-8, 1e-6, 3e-3])
    cfg = DEMConfig(domain_min=[-0.05] * 3, domain_max=[0.5] * 3, max_coordinate_number=8,
                    wall_distance=10.0, gravity=[0.0, 0.0, 0.0], dt=1e-9,
                    particle_elastic_modulus=1e8)
    pos0 = _place(r, centres, dirs, np.full(npair, 2e-3))  # apart, on the neighbour lists
    p = ParticleInput.from_arrays(r, pos0, np.zeros_like(pos0), 2500.0)
    for lanes in (4, 1):  # both layouts of the list step
        g, o = both(cfg, p)
        g.set_launch_shape(list_lanes=lanes)
        g.simulate(3)  # full searches (a new handle searches at both buffer parities), a list step
        searches = g.stats()["full_searches"]
        created = 0
        for shift in range(3):
            rel = deltas[(np.arange(npair) + 5 * shift) % len(deltas)]
            copy_state(g, o)
            pos = _place(r, centres, dirs, rel)
            g.set_particles(pos=pos)
            o.set_particles(pos=pos)
            g.simulate(1)
            o.simulate(1)
            assert g.stats()["full_searches"] == searches, "the steps under test are list steps"
            cg, co = g.contacts(), o.contacts()
            assert pair_set(cg) == pair_set(co), f"lanes {lanes} shift {shift}"
            assert np.isfinite(g.particles()["pos"]).all()
            created += len(co["i"])
        assert 0 < created < 3 * npair
        g.close()


def test_list_layouts_bit_identical(gpu):
    """The neighbour-list update with one lane per particle and with four
    give the same results bit for bit: a compacted polydisperse bed, a dense
    granular cloud whose contacts form and end every step, and a bonded cube
    that fragments at the wall (its lattice coordinates take the exact FP64
    fallbacks of the cell tests when a Hertz contact between fragments ends;
    the four-lane path shares that cp_list test between a particle's lanes,
    the one-lane path runs it alone)."""
    f = 2.0 * (30_000 / 2_000_000) ** (1.0 / 3.0)
    bed = scenes.granular_bed(30_000, box=(0.4 * f, 0.4 * f, 1.2), seed=23)
    ccfg, cp = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=15, v=0.5)
    cloud = SimpleNamespace(cfg=ccfg, particles=cp, bonded=False)
    cube = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    for name, sc, steps in (("bed", bed, 200), ("cloud", cloud, 200), ("cube", cube, 2000)):
        outs = []
        for lanes in (1, 4):
            g = GlobalData(sc.cfg, sc.particles)
            g.set_launch_shape(list_lanes=lanes)
            if sc.bonded:
                g.initialize()
            g.simulate(steps)
            outs.append((g.particles(), g.contacts(), g.stats()))
            g.close()
        for k in outs[0][0]:
            np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k], err_msg=k)
        for k in outs[0][1]:
            np.testing.assert_array_equal(outs[0][1][k], outs[1][1][k], err_msg=k)
        s1, s4 = outs[0][2], outs[1][2]
        assert (s1["contacts_created"], s1["contacts_ended"]) == \
            (s4["contacts_created"], s4["contacts_ended"])
        if name != "bed":
            # contacts ended: the four-lane path's shared cp_list membership
            # test ran and matched the one-lane path's own
            assert s4["contacts_ended"] > 0, name


def run_layouts(cfg, p, steps, bonded, knob, values=(1, 4), precision="fp64", tables=None):
    """Runs the scene once per value of a launch-shape knob; returns each run's
    particles, contacts and stats."""
    outs = []
    for v in values:
        g = GlobalData(cfg, p, precision=precision, tables=tables)
        g.set_launch_shape(**{knob: v})
        if bonded:
            g.initialize()
        g.simulate(steps)
        outs.append((g.particles(), g.contacts(), g.stats()))
        g.close()
    return outs


def assert_runs_identical(outs, what):
    (p0, c0, s0), rest = outs[0], outs[1:]
    for p1, c1, s1 in rest:
        for k in p0:
            np.testing.assert_array_equal(p0[k], p1[k], err_msg=f"{what} {k}")
        for k in c0:
            np.testing.assert_array_equal(c0[k], c1[k], err_msg=f"{what} contacts {k}")
        for k in ("bonds_broken", "contacts_created", "contacts_ended", "warn_gap",
                  "warn_damping", "error"):
            assert s0.get(k) == s1.get(k), (what, k)


def test_profiled_steps_equal_graph_steps(gpu):
    """dem_step_profiled (the step's kernels with CUDA events between them)
    steps exactly as dem_step does, on both contact buffers, and reports a
    positive device time for each phase."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    a, b = GlobalData(sc.cfg, sc.particles), GlobalData(sc.cfg, sc.particles)
    for g in (a, b):
        g.initialize()
    a.simulate(60)
    for s in range(60):
        if s % 3 == 0:  # both parities of the contact buffers
            ph = b.simulate_profiled()
            assert set(ph) == {"contacts", "force", "integrate"}
            assert all(v > 0 for v in ph.values()), ph
        else:
            b.simulate(1)
    pa, pb = a.particles(), b.particles()
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
    assert pair_set(a.contacts()) == pair_set(b.contacts())
    assert a.stats()["steps_done"] == b.stats()["steps_done"] == 60
    a.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_integrate_layouts_bit_identical(gpu, precision):
    """The integrator with one thread per particle and split over four warps
    per 32 particles (one per force component, one for the walls and the
    quaternion) gives the same results bit for bit: a bonded cube's wall
    impact (wall contacts, spin, bonds breaking), a damped cube, and a
    polydisperse cloud under gravity with damping thrown at the floor."""
    cube = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    outs = run_layouts(cube.cfg, cube.particles, 1000, True, "integrate_lanes",
                       precision=precision)  # bonds start to break near step 900
    assert_runs_identical(outs, f"cube {precision}")
    assert outs[0][2]["bonds_broken"] > 0
    assert np.count_nonzero(np.any(outs[0][0]["wall_shear"] != 0, axis=1)) > 0
    damped = cube.cfg.replace(global_damping=0.2)
    assert_runs_identical(run_layouts(damped, cube.particles, 150, True, "integrate_lanes",
                                      precision=precision), f"damped cube {precision}")
    # a wall restitution above 1 gives negative wall damping, which is
    # counted once per wall contact and step, whatever the layout
    cfg, p = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=15, v=0.5,
                          cfg_kw=dict(global_damping=0.3, pp_coefficient_friction=0.3,
                                      pw_coefficient_restitution=1.2))
    p.vel[:, 2] -= 1.0
    outs = run_layouts(cfg, p, 150, False, "integrate_lanes", precision=precision)
    assert_runs_identical(outs, f"cloud {precision}")
    assert outs[0][2]["warn_damping"] > 0


def test_short_horizon_cube(gpu):
    sc = scenes.bonded_cube(10, speed=10.0, steps=0, seed=1)
    g, o = both(sc.cfg, sc.particles)
    g.initialize()
    o.initialize()
    for _ in range(4):
        g.simulate(50)
        o.simulate(50)
        compare_state(g, o, RTOL_HORIZON, "cube horizon")
    assert g.stats()["error"] == 0


def test_short_horizon_fast_impact_breaks_bonds(gpu):
    """A fast impact that breaks bonds: broken-bond counts and bond sets match."""
    sc = scenes.bonded_cube(6, speed=30.0, steps=0, seed=2)
    cfg = sc.cfg.replace(bond_tensile_strength=2e5, bond_shear_strength=2e5)
    g, o = both(cfg, sc.particles)
    g.initialize()
    o.initialize()
    for _ in range(8):
        g.simulate(50)
        o.simulate(50)
        compare_state(g, o, RTOL_HORIZON, "fast impact")
    assert o.stats()["bonds_broken"] > 0
    assert g.stats()["bonds_broken"] == o.stats()["bonds_broken"]


def test_deterministic_rerun(gpu):
    cfg, p = random_cloud(2000, (0.04, 0.04, 0.04), 0.0008, 0.0015, seed=8, v=0.3)
    outs = []
    for _ in range(2):
        g = GlobalData(cfg, p)
        g.simulate(100)
        outs.append((g.particles(), g.contacts()))
        g.close()
    for k in outs[0][0]:
        np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k])
    for k in outs[0][1]:
        np.testing.assert_array_equal(outs[0][1][k], outs[1][1][k])


def test_fp32_force_mode_error(gpu):
    cfg, p = random_cloud(3000, (0.05, 0.05, 0.05), 0.0008, 0.0015, seed=5, v=0.5)
    g, o = both(cfg, p, precision="fp32")
    o.simulate(5)
    pp, c = o.particles(), o.contacts()
    g.set_particles(pos=pp["pos"], vel=pp["vel"], omega=pp["omega"], quat=pp["quat"],
                    wall_shear=pp["wall_shear"])
    g.set_contacts(c)
    g.simulate(1)
    o.simulate(1)
    cg, co = g.contacts(), o.contacts()
    assert pair_set(cg) == pair_set(co)
    assert_rows_close(cg["force"], co["force"], RTOL_FP32, "fp32 contact force", atol_frac=RTOL_FP32)
    pg, po = g.particles(), o.particles()
    assert_rows_close(pg["force"], po["force"], RTOL_FP32, "fp32 force", atol_frac=RTOL_FP32)


def test_fp32_force_mode_bonded(gpu):
    sc = scenes.bonded_cube(8, speed=10.0, steps=0, seed=4)
    g, o = both(sc.cfg, sc.particles, precision="fp32")
    g.initialize()
    o.initialize()
    g.simulate(200)
    o.simulate(200)
    cg, co = g.contacts(), o.contacts()
    assert bonded_set(cg) == bonded_set(co)
    pg, po = g.particles(), o.particles()
    assert_rows_close(pg["pos"], po["pos"], 1e-6, "fp32 pos")
    assert_rows_close(pg["force"], po["force"], RTOL_FP32, "fp32 force", atol_frac=RTOL_FP32)


def kinetic_energy(st, mass):
    return 0.5 * float(np.sum(mass * np.sum(st["vel"] ** 2, axis=1)))


def test_fp32_force_mode_impact_errors(gpu):
    """FP32 force mode on a fast impact that breaks bonds, against the FP64
    oracle: per-result errors stated in the assertions (force 1e-3 relative,
    kinetic energy 1e-4 relative, broken-bond count within 1% of the bonds;
    the breakage decision itself is the FP64 test)."""
    sc = scenes.bonded_cube(6, speed=30.0, steps=0, seed=2)
    cfg = sc.cfg.replace(bond_tensile_strength=2e5, bond_shear_strength=2e5)
    g, o = both(cfg, sc.particles, precision="fp32")
    g.initialize()
    o.initialize()
    nb0 = o.stats()["bonded"]
    for _ in range(4):
        g.simulate(50)
        o.simulate(50)
    pg, po = g.particles(), o.particles()
    m = sc.particles.mass
    ke_g, ke_o = kinetic_energy(pg, m), kinetic_energy(po, m)
    assert abs(ke_g - ke_o) <= 1e-4 * ke_o, (ke_g, ke_o)
    bg, bo = g.stats()["bonds_broken"], o.stats()["bonds_broken"]
    assert bo > 0
    assert abs(bg - bo) <= max(1, 0.01 * nb0), (bg, bo)
    assert_rows_close(pg["pos"], po["pos"], 1e-6, "fp32 impact pos")


def test_precision_switch_midrun(gpu):
    """FP64 -> FP32 -> FP64 force modes in one run: the stored bond forces are
    re-encoded at each switch (FP32 mode keeps them as FP32 hi/lo pairs), so
    the run stays within the FP32 tolerance of the FP64 oracle throughout."""
    sc = scenes.bonded_cube(6, speed=30.0, steps=0, seed=7)
    g, o = both(sc.cfg, sc.particles)
    g.initialize()
    o.initialize()
    for prec in ("fp64", "fp32", "fp64", "fp32"):
        g.set_precision(prec)
        g.simulate(40)
        o.simulate(40)
        cg, co = g.contacts(), o.contacts()
        assert bonded_set(cg) == bonded_set(co), prec
        assert_rows_close(cg["force"], co["force"], RTOL_FP32, f"{prec} contact force",
                          atol_frac=RTOL_FP32)
        assert_rows_close(cg["torque_i"], co["torque_i"], RTOL_FP32, f"{prec} torque",
                          atol_frac=RTOL_FP32)
        pg, po = g.particles(), o.particles()
        assert_rows_close(pg["pos"], po["pos"], 1e-6, f"{prec} pos")


# ---- edge cases ----------------------------------------------------------------------------

def test_single_particle_on_wall(gpu):
    cfg = DEMConfig(domain_min=[-1, -1, -1], domain_max=[1, 1, 1], wall_distance=0.0,
                    dt=1e-6, max_coordinate_number=4)
    p = ParticleInput.from_arrays(np.array([0.01]), np.array([[0.0, 0.0, 0.0095]]),
                                  np.array([[0.1, 0.0, -0.5]]), 2500.0)
    g, o = both(cfg, p)
    for _ in range(5):
        g.simulate(20)
        o.simulate(20)
        pg, po = g.particles(), o.particles()
        assert_rows_close(pg["pos"], po["pos"], RTOL_HORIZON, "pos")
        assert_rows_close(pg["vel"], po["vel"], RTOL_HORIZON, "vel")
        assert_rows_close(pg["wall_shear"], po["wall_shear"], RTOL_HORIZON, "wall shear",
                          atol_frac=RTOL_HORIZON)


def test_empty_scene(gpu):
    cfg = DEMConfig(domain_min=[-1, -1, -1], domain_max=[1, 1, 1])
    p = ParticleInput.from_arrays(np.zeros(0), np.zeros((0, 3)), np.zeros((0, 3)), 2500.0)
    g = GlobalData(cfg, p)
    g.initialize()
    g.simulate(3)
    g.sync()
    assert len(g.contacts()["i"]) == 0


def test_capacity_overflow_reports_error(gpu):
    sc = scenes.bonded_cube(5, steps=0)
    cfg = sc.cfg.replace(max_coordinate_number=1)
    g = GlobalData(cfg, sc.particles)
    with pytest.raises(DemError) as e:
        g.initialize()
    assert e.value.code == DEM_ERR_CAPACITY


def test_integer_pipe_conversions_match_hardware(gpu):
    """The FP64<->FP32 conversions done with integer instructions round
    exactly as the hardware conversions (ties, range edges, subnormal and
    overflowing results included); the Newton-Raphson FP64 reciprocal is
    within 2 ulp of the correctly rounded one; the integer-pipe halving is
    bit-identical to x * 0.5 (zeros, subnormals, exponent edges, infinities);
    where the integrator skips the quaternion increment of a spinless
    particle or the spin update of a torque-free one, the skipped FMA chains
    would have returned their input bit for bit, and the identity
    orientation normalises to itself (rsqrt(1) is exactly 1)."""
    import ctypes
    bad = (ctypes.c_int64 * 4)()
    for seed in (1, 2, 3):
        assert gpu.dem_selftest_conversions(1 << 22, seed, bad) == 0
        assert tuple(bad) == (0, 0, 0, 0), (seed, tuple(bad))
