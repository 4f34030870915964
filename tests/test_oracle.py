"""CPU tests of the oracle: pinned against the reference's own functions
(golden vectors) and against analytic known answers."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from taichi_dem_julia_port_gb300 import scenes
from taichi_dem_julia_port_gb300.config import DEMConfig
from taichi_dem_julia_port_gb300.scenes import ParticleInput

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ref_golden():
    return json.loads((GOLDEN / "reference_functions.json").read_text())


def test_morton_readme_kat(oracle_lib, ref_golden):
    # README.md:23 — cartesian3morton([2,3,4]) == morton3d32(1,2,3) + 1 == 54
    kat = ref_golden["readme_kat"]
    assert O.morton1(*kat["cartesian3morton"]) == kat["value"] == 54


def test_morton_matches_reference_dem_py(oracle_lib, ref_golden):
    for x, y, z, expect in ref_golden["morton"]:
        assert O.morton1(x, y, z) == expect, (x, y, z)


def test_quaternion_matrix_matches_reference(oracle_lib, ref_golden):
    for rec in ref_golden["quat2rot"]:
        R = O.quat_to_matrix(rec["q"])
        np.testing.assert_allclose(R.ravel(), rec["R"], rtol=0, atol=1e-14)


# ---- physics pinned to the reference's dem.py ----------------------------------
# tests/golden/reference_physics.json holds the outputs of dem.py's own
# DEMSolver.resolve (EBPM dem.py:1405-1528, Hertz-Mindlin dem.py:1529-1606),
# resolve_wall/evaluate_wall (dem.py:1609-1743), apply_body_force
# (dem.py:1280-1305) and update (dem.py:1309-1354), executed from the
# reference's source (tests/golden/make_physics_golden.py).  dem.py and
# src/kernels.jl state the same formulas; they differ only in the association
# of a few sums (the Rodrigues term, the position update, the quaternion
# increments), in normalize (v/|v| against inv(|v|)·v) and in the 3x3 inverse
# (adjugate/determinant against column cross products), so the oracle, which
# follows kernels.jl, agrees with them to rounding: measured at most 1.8e-14
# of each vector's magnitude.  The stated bound is 1e-12.  Discrete outcomes
# (bond broken or not, wall contact or not) must be identical, including
# strengths placed a relative 1e-9 below and above the stress a case reaches.
PHYS_RTOL = 1e-12


@pytest.fixture(scope="module")
def phys_golden():
    return json.loads((GOLDEN / "reference_physics.json").read_text())


def _cfg_of(p: dict) -> DEMConfig:
    return DEMConfig(
        particle_elastic_modulus=p["E"], particle_poisson_ratio=p["nu"],
        wall_elastic_modulus=p["wall_E"], wall_poisson_ratio=p["wall_nu"],
        pp_coefficient_friction=p["mu"], pp_coefficient_restitution=p["e"],
        pw_coefficient_friction=p["pw_mu"], pw_coefficient_restitution=p["pw_e"],
        bond_radius_ratio=p["bond_ratio"], bond_elastic_modulus=p["bond_E"],
        bond_poisson_ratio=p["bond_nu"], bond_compressive_strength=p["sc"],
        bond_tensile_strength=p["st"], bond_shear_strength=p["ss"], dt=p["dt"],
        gravity=list(p["gravity"]), global_damping=p["global_damping"],
        wall_normal=list(p["wall_n"]), wall_distance=p["wall_d"], tolerance=1e-12)


def _close(got, want, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = float(np.abs(want).max())
    err = float(np.abs(got - want).max())
    assert err <= PHYS_RTOL * scale, f"{what}: |d| {err:.3e} > {PHYS_RTOL:g}·{scale:.3e}"


def test_bond_forces_match_reference_dem_py(oracle_lib, phys_golden):
    """EBPM: increments k1..k6, accumulated force and moments, particle forces
    and moments, for random frames and the degenerate ones (bond along ±x)."""
    n_intact = 0
    for c in phys_golden["bond"]:
        if c["out"]["bonded"] == 0:
            continue
        o = O.eval_pair(_cfg_of(c["params"]), c["gi"], c["gj"], c["state"], True)
        assert o["kind"] == 2
        for k in ("fi", "fj", "mi", "mj", "k", "F", "ti", "tj"):
            _close(o[k], c["out"][k], f"bond {k}")
        n_intact += 1
    assert n_intact >= 60


def test_bond_breakage_decisions_match_reference_dem_py(oracle_lib, phys_golden):
    """σc, σt, τ against strengths a relative 1e-9 below (breaks) and above
    (holds) the stress each case reaches; a broken bond applies no force."""
    modes = set()
    for c in phys_golden["bond"]:
        o = O.eval_pair(_cfg_of(c["params"]), c["gi"], c["gj"], c["state"], True)
        broken = c["out"]["bonded"] == 0
        assert (o["kind"] == 1) == broken, c.get("threshold")
        assert c["out"]["active"] == (0 if broken else 1)
        if broken:
            assert not np.any(c["out"]["fi"]) and not np.any(o["fi"])
        if "threshold" in c:
            t = c["threshold"]
            assert broken == (t["rel"] < 1.0)
            modes.add(t["mode"])
    assert modes == {"sc", "st", "ss"}


def test_hertz_forces_match_reference_dem_py(oracle_lib, phys_golden):
    """Hertz-Mindlin: new and carried shear histories, sliding and sticking,
    spinning and spinless grains, degenerate and near-degenerate frames."""
    sliding = 0
    for c in phys_golden["hertz"]:
        o = O.eval_pair(_cfg_of(c["params"]), c["gi"], c["gj"], c["state"], False)
        assert o["kind"] == 2
        for k in ("fi", "fj", "mi", "mj", "k", "F", "s"):
            _close(o[k], c["out"][k], f"hertz {k}")
        F = np.asarray(c["out"]["F"])
        sliding += abs(np.hypot(F[1], F[2]) - c["params"]["mu"] * F[0]) <= 1e-9 * abs(F[0])
    assert 20 <= sliding <= len(phys_golden["hertz"]) - 20


def test_wall_forces_match_reference_dem_py(oracle_lib, phys_golden):
    """Particle-wall Hertz-Mindlin on both sides of the plane, axis-aligned
    and oblique normals, carried or new shear history, and non-touching cases."""
    touching = 0
    for c in phys_golden["wall"]:
        o = O.eval_wall(_cfg_of(c["params"]), c["g"], c["s_in"])
        assert o["touch"] == c["out"]["touch"]
        if not o["touch"]:
            assert not np.any(o["f"]) and not np.any(c["out"]["f"])
            continue
        touching += 1
        for k in ("f", "m", "k", "F", "s"):
            _close(o[k], c["out"][k], f"wall {k}")
    assert touching >= 80


def test_body_force_and_update_match_reference_dem_py(oracle_lib, phys_golden):
    """Gravity, global damping (including sign(0) = 0 on zero velocity and
    spin components) and the integrator: position, velocity, quaternion and
    spin after one update."""
    dampings = set()
    for c in phys_golden["update"]:
        o = O.eval_update(_cfg_of(c["params"]), c["grains"], c["F"], c["T"])
        dampings.add(c["params"]["global_damping"])
        for i, ref in enumerate(c["out"]):
            np.testing.assert_array_equal(o["F"][i], ref["F"])
            np.testing.assert_array_equal(o["T"][i], ref["T"])
            for k in ("k", "v", "q", "w"):
                _close(o[k][i], ref[k], f"update {k}")
    assert len(dampings) >= 3 and 0.0 in dampings


def test_frame_maps_normal_to_x(oracle_lib):
    rng = np.random.default_rng(0)
    for _ in range(100):
        a = rng.standard_normal(3)
        a /= np.linalg.norm(a)
        R = O.frame_to_x(a)
        np.testing.assert_allclose(R @ a, [1, 0, 0], atol=1e-12)
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    # the degenerate branch (s < tolerance) of src/kernels.jl:151-155
    np.testing.assert_array_equal(O.frame_to_x([1.0, 0, 0]), np.eye(3))
    np.testing.assert_array_equal(O.frame_to_x([-1.0, 0, 0]), np.diag([-1.0, 1.0, -1.0]))


def test_norm_scaled_branch(oracle_lib):
    assert O.jl_norm([0.0, 0.0, 0.0]) == 0.0
    assert O.jl_norm([3.0, 4.0, 12.0]) == 13.0
    assert O.jl_norm([1e300, 1e300, 0.0]) == pytest.approx(math.sqrt(2) * 1e300)
    assert O.jl_norm([1e-300, 0.0, 0.0]) == 1e-300


def test_oracle_regression_vectors(oracle_lib):
    g = json.loads((GOLDEN / "oracle_regression.json").read_text())["cube3_150"]
    sc = scenes.bonded_cube(3, speed=10.0, steps=0, seed=7)
    o = O.OracleScene(sc.cfg, sc.particles)
    o.initialize()
    o.simulate(150)
    p, c = o.particles(), o.contacts()
    np.testing.assert_array_equal(p["pos"], np.array(g["pos"]))
    np.testing.assert_array_equal(p["vel"], np.array(g["vel"]))
    np.testing.assert_array_equal(np.stack([c["i"], c["j"]], 1), np.array(g["pairs"]).reshape(-1, 2))


def _two_spheres(r=0.01, overlap=1e-5, v=0.0, E=1e8, e=0.9, mu=0.5, gravity=0.0):
    cfg = DEMConfig(domain_min=[-1, -1, -1], domain_max=[1, 1, 1], particle_elastic_modulus=E,
                    particle_poisson_ratio=0.3, pp_coefficient_restitution=e,
                    pp_coefficient_friction=mu, wall_distance=100.0,
                    gravity=[0.0, 0.0, gravity], dt=1e-7, max_coordinate_number=8)
    pos = np.array([[0.0, 0.0, 0.0], [2 * r - overlap, 0.0, 0.0]])
    vel = np.array([[v, 0, 0], [-v, 0, 0]])
    return cfg, ParticleInput.from_arrays(np.array([r, r]), pos, vel, 2500.0)


def test_hertz_normal_force_kat(oracle_lib):
    """Two resting spheres overlapping by δ: Fn = 4/3 Y* sqrt(R* δ) δ."""
    cfg, p = _two_spheres(overlap=2e-5)
    o = O.OracleScene(cfg, p)
    o.simulate(1)
    st = o.static()
    r = st["radius"][0]
    delta = 2 * r - (p.pos[1, 0] - p.pos[0, 0])
    nu, E = 0.3, 1e8
    Ys = 1.0 / (2 * (1 - nu * nu) / E)
    Rs = r / 2
    Fn = 4.0 / 3.0 * Ys * math.sqrt(Rs * delta) * delta
    f = o.particles()["force"]
    assert f[0, 0] == pytest.approx(-Fn, rel=1e-12)
    assert f[1, 0] == pytest.approx(Fn, rel=1e-12)
    assert abs(f[0, 1]) < 1e-12 * Fn and abs(f[0, 2]) < 1e-12 * Fn
    c = o.contacts()
    assert len(c["i"]) == 1 and c["bonded"][0] == 0


def _bond_pair(gap=0.0, pull=0.0, r=0.01, E=1e8, st=1e6, ss=1e6):
    cfg = DEMConfig(domain_min=[-1, -1, -1], domain_max=[1, 1, 1], bond_elastic_modulus=E,
                    bond_tensile_strength=st, bond_shear_strength=ss, wall_distance=100.0,
                    gravity=[0.0, 0.0, 0.0], dt=1e-6, max_coordinate_number=8)
    pos = np.array([[0.0, 0.0, 0.0], [2 * r + gap, 0.0, 0.0]])
    vel = np.array([[-pull, 0, 0], [pull, 0, 0]])
    return cfg, ParticleInput.from_arrays(np.array([r, r]), pos, vel, 2500.0)


def test_bond_axial_stiffness_kat(oracle_lib):
    """One step of separating velocity v: ΔFx = k1·(dᵢ-dⱼ), k1 = E·A/L."""
    v = 0.01
    cfg, p = _bond_pair(pull=v)
    o = O.OracleScene(cfg, p)
    o.initialize()
    assert o.stats()["bonded"] == 1
    o.simulate(1)
    c = o.contacts()
    r = o.static()["radius"][0]
    rb = 0.5 * r
    A = math.pi * rb * rb
    L = p.pos[1, 0] - p.pos[0, 0]
    k1 = 1e8 * A / L
    expect = k1 * (-v * cfg.dt - v * cfg.dt)  # dᵢ - dⱼ along the bond axis
    assert c["force"][0, 0] == pytest.approx(expect, rel=1e-12)


def test_bond_breaks_at_tensile_strength(oracle_lib):
    """A pair pulled apart breaks once σt = F/A reaches the tensile strength."""
    v = 1.0
    cfg, p = _bond_pair(pull=v, st=1e3, ss=1e12)
    o = O.OracleScene(cfg, p)
    o.initialize()
    r = o.static()["radius"][0]
    A = math.pi * (0.5 * r) ** 2
    L = p.pos[1, 0] - p.pos[0, 0]
    k1 = 1e8 * A / L
    per_step = k1 * 2 * v * cfg.dt / A  # σt growth per step
    n_expect = math.ceil(1e3 / per_step)
    for s in range(1, n_expect + 3):
        o.simulate(1)
        if o.stats()["bonded"] == 0:
            break
    assert o.stats()["bonds_broken"] == 1
    assert abs(s - n_expect) <= 1


def test_serial_and_parallel_modes_identical(oracle_lib):
    sc = scenes.bonded_cube(6, speed=10.0, steps=0, seed=5)
    outs = []
    for t in (1, 4):
        o = O.OracleScene(sc.cfg, sc.particles, threads=t)
        o.initialize()
        o.simulate(300)
        outs.append((o.particles(), o.contacts()))
    for k in outs[0][0]:
        np.testing.assert_array_equal(outs[0][0][k], outs[1][0][k])
    for k in outs[0][1]:
        np.testing.assert_array_equal(outs[0][1][k], outs[1][1][k])


def test_lattice_bond_count(oracle_lib):
    for side in (3, 10):
        sc = scenes.bonded_cube(side, steps=0)
        o = O.OracleScene(sc.cfg, sc.particles)
        o.initialize()
        assert o.stats()["bonded"] == 3 * side * side * (side - 1)


def test_cp_list_multiset_covers_touching_pairs(oracle_lib):
    """Every touching pair is in cp_list (cell = 4 r_max > 2·(rᵢ+rⱼ))."""
    rng = np.random.default_rng(11)
    n = 3000
    r = rng.uniform(0.5e-3, 2e-3, n)
    pos = rng.uniform(0, 0.05, (n, 3))
    cfg = DEMConfig(domain_min=[-0.01] * 3, domain_max=[0.06] * 3, max_coordinate_number=64)
    o = O.OracleScene(cfg, ParticleInput.from_arrays(r, pos, np.zeros((n, 3)), 2500.0))
    bp = o.debug_broadphase()
    pairs = {tuple(x) for x in bp["cp"].tolist()}
    r = o.static()["radius"]
    from scipy.spatial import cKDTree
    tree = cKDTree(pos)
    for i, j in tree.query_pairs(2 * r.max()):
        a, b = min(i, j), max(i, j)
        if np.linalg.norm(pos[a] - pos[b]) < r[a] + r[b]:
            assert (a, b) in pairs


def test_capacity_error(oracle_lib):
    sc = scenes.bonded_cube(4, steps=0)
    cfg = sc.cfg.replace(max_coordinate_number=1)
    o = O.OracleScene(cfg, sc.particles)
    with pytest.raises(RuntimeError):
        o.initialize()


def test_reference_scenes_fixture(oracle_lib):
    """The packed reference scenes equal a fresh read of the reference's files
    (when the reference checkout is present) and run on the oracle."""
    from taichi_dem_julia_port_gb300 import DEMConfig, load_particles
    from tests import reference_scenes as rs
    ref = rs.reference_checkout()
    for name, cfg_rel in (("carom", "cfg/1.toml"), ("cube_911", "cfg/2.toml")):
        cfg, p, src = rs.load(name)
        assert src.startswith(cfg_rel)
        if ref is not None:
            cfg2 = DEMConfig.from_toml(ref / cfg_rel)
            p2 = load_particles((ref / cfg_rel).parent / cfg2.init_particles)
            assert cfg2.to_toml() == cfg.to_toml()
            for k in ("id", "gid", "volume", "mass", "pos", "vel"):
                np.testing.assert_array_equal(getattr(p2, k), getattr(p, k), err_msg=k)
    cfg, p, _ = rs.load("cube_911")
    o = O.OracleScene(cfg, p)
    o.initialize()
    st = o.stats()
    assert st["bonded"] > 2000 and st["bonded"] == st["contacts"]
    o.simulate(20)
    assert o.stats()["error"] == 0
