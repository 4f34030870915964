"""CPU tests of the host side: config, p4p/p4c files, scenes and the C ABI
surface of libdem_sm100a.so (loaded, no GPU call)."""
import ctypes
import io
import re
from pathlib import Path

import numpy as np
import pytest

from taichi_dem_julia_port_gb300 import _abi, p4io, scenes
from taichi_dem_julia_port_gb300.config import DEMConfig

ROOT = Path(__file__).resolve().parents[1]
from tests.reference_scenes import reference_checkout  # noqa: E402

_REF = reference_checkout()
REF_CFG = _REF / "cfg" if _REF is not None else Path("reference-checkout-absent")


def header_functions():
    src = (ROOT / "include" / "dem_gb300.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(dem_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_header_function(dem_lib_path):
    lib = ctypes.CDLL(str(dem_lib_path))
    names = header_functions()
    assert len(names) >= 19
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_abi.ENTRY_POINTS), set(names) ^ set(_abi.ENTRY_POINTS)
    assert _abi.load_library().dem_version().decode().startswith("dem_gb300")


def test_config_struct_matches_header():
    src = (ROOT / "include" / "dem_gb300.h").read_text()
    body = src[src.index("typedef struct DemConfigC {"):src.index("} DemConfigC;")]
    fields = re.findall(r"(?:double|int64_t)\s+(\w+)", body)
    assert fields == [f for f, _ in _abi.DemConfigC._fields_]
    assert len(fields) == 32  # + init_particles = the 33 keys of DEMConfig


@pytest.mark.parametrize("name", ["DemStats", "DemLaunchShape", "DemParticleState"])
def test_result_structs_match_header(name, tmp_path):
    """The ctypes mirrors of the header's result structs: same fields in the
    same order, and the same size as the C compiler gives them."""
    import shutil
    import subprocess
    src = (ROOT / "include" / "dem_gb300.h").read_text()
    body = src[src.index(f"typedef struct {name} {{"):src.index(f"}} {name};")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"(?:double|int64_t|int32_t|int)\s*\*?\s*(\w+)\s*[;,\[]", body)
    mirror = getattr(_abi, name)
    assert fields == [f for f, _ in mirror._fields_]
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    prog = tmp_path / "size.c"
    prog.write_text(f'#include "dem_gb300.h"\n#include <stdio.h>\n'
                    f'int main(void) {{ printf("%zu", sizeof({name})); return 0; }}\n')
    exe = tmp_path / "size"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(prog), "-o", str(exe)], check=True)
    assert int(subprocess.run([str(exe)], capture_output=True, text=True).stdout) == \
        ctypes.sizeof(mirror)


def test_config_defaults_and_roundtrip(tmp_path):
    c = DEMConfig()
    assert c.dt == 2.63e-5 and c.max_coordinate_number == 64 and c.tolerance == 1e-12
    assert c.total_steps == int(0.5 / 2.63e-5)
    t = tmp_path / "c.toml"
    t.write_text(c.replace(dt=1e-6, domain_min=[1.0, 2.0, 3.0]).to_toml())
    d = DEMConfig.from_toml(t)
    assert d.dt == 1e-6 and d.domain_min == [1.0, 2.0, 3.0]
    cc = d.to_c()
    assert cc.dt == 1e-6 and list(cc.domain_min) == [1.0, 2.0, 3.0]
    with pytest.raises(ValueError):
        DEMConfig.from_dict({"no_such_key": 1})


@pytest.mark.skipif(not REF_CFG.exists(), reason="reference checkout not present")
def test_reference_config_files_parse():
    for f in sorted(REF_CFG.glob("*.toml")):
        c = DEMConfig.from_toml(f)
        assert c.dt > 0 and len(c.domain_min) == 3


def test_jl_float_format():
    assert p4io.jl_float(0.5) == "0.5"
    assert p4io.jl_float(1e-5) == "1.0e-5"
    assert p4io.jl_float(2.0) == "2.0"
    assert p4io.jl_float(1e6) == "1.0e6"
    assert p4io.jl_float(123456.0) == "123456.0"
    for x in (0.1, 1 / 3, -2.5e-7, 6.02e23, 3.0):
        assert float(p4io.jl_float(x)) == x


def test_p4p_p4c_roundtrip_and_compare(tmp_path):
    rng = np.random.default_rng(0)
    n = 20
    ids = np.arange(1, n + 1)
    pos, vel = rng.standard_normal((n, 3)), rng.standard_normal((n, 3))
    vol, mass = rng.uniform(1, 2, n), rng.uniform(1, 2, n)
    f1, f2 = tmp_path / "a.p4p", tmp_path / "b.p4p"
    for f, p in ((f1, pos), (f2, pos * (1 + 1e-12))):
        with open(f, "w") as fh:
            p4io.write_p4p(fh, 0.0, ids, np.zeros(n), vol, mass, p, vel)
            p4io.write_p4p(fh, 1e-3, ids, np.zeros(n), vol, mass, p, vel)
    recs = p4io.read_p4p(f1)
    assert len(recs) == 2 and np.array_equal(recs[0].pos, pos)
    p4io.compare_p4p(f1, f2)
    with open(f2, "w") as fh:
        p4io.write_p4p(fh, 0.0, ids, np.zeros(n), vol, mass, pos * 1.001, vel)
        p4io.write_p4p(fh, 1e-3, ids, np.zeros(n), vol, mass, pos, vel)
    with pytest.raises(AssertionError):
        p4io.compare_p4p(f1, f2)
    ci, cj = np.array([0, 2, 1]), np.array([1, 5, 3])
    pt, fo = rng.standard_normal((3, 3)), rng.standard_normal((3, 3))
    c1, c2 = tmp_path / "a.p4c", tmp_path / "b.p4c"
    with open(c1, "w") as fh:
        p4io.write_p4c(fh, 0.0, ci, cj, pt, fo, [1, 0, 1])
    order = [2, 0, 1]
    with open(c2, "w") as fh:
        p4io.write_p4c(fh, 0.0, ci[order], cj[order], pt[order], fo[order], np.array([1, 0, 1])[order])
    p4io.compare_p4c(c1, c2)  # compared as sorted pairs
    r = p4io.read_p4c(c1)[0]
    assert list(zip(r.i, r.j)) == [(1, 2), (2, 4), (3, 6)]
    with pytest.raises(RuntimeError):
        p4io.write_p4c(io.StringIO(), 0.0, [0, 0], [1, 1], pt[:2], fo[:2], [0, 0])


def test_bonded_cube_scene():
    sc = scenes.bonded_cube(4, steps=0)
    assert sc.n == 64
    r = np.cbrt(sc.particles.volume / (4 / 3 * np.pi))
    assert np.all((r > 0.0095 - 1e-12) & (r < 0.0105 + 1e-12))
    wall_z = -sc.cfg.wall_distance
    assert np.isclose(np.min(sc.particles.pos[:, 2] - r) - wall_z, 1e-3)
    assert np.all(sc.particles.vel[:, 2] == -10.0)


def test_granular_pour_no_overlap():
    sc = scenes.granular_pour(8000, box=(0.1, 0.1, 0.1), seed=1)
    from scipy.spatial import cKDTree
    p = sc.particles.pos
    r = np.cbrt(sc.particles.volume / (4 / 3 * np.pi))
    pairs = cKDTree(p).query_pairs(2 * r.max())
    for i, j in pairs:
        assert np.linalg.norm(p[i] - p[j]) >= r[i] + r[j]
    assert np.all(p > 0) and np.all(p < 0.1)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(FileNotFoundError):
        _abi.load_library(tmp_path / "libdem_sm100a.so")


def test_serving_sizing_and_requests():
    from taichi_dem_julia_port_gb300.serving import ArenaSizing, poisson_requests
    s = ArenaSizing.from_budget(160e9)
    assert 160e9 * 0.95 < s.bytes <= 160e9
    assert s.max_contacts == s.max_particles * s.contacts_per_particle
    a, b = poisson_requests(50, seed=9), poisson_requests(50, seed=9)
    assert [(r.arrival_s, r.steps, r.n_hint) for r in a] == [(r.arrival_s, r.steps, r.n_hint) for r in b]
    gaps = np.diff([0.0] + [r.arrival_s for r in a])
    assert 0.005 < gaps.mean() < 0.05  # mean 1/50 s
    assert all(1_000 <= r.steps <= 50_000 for r in a)
    assert all(900 <= r.n_hint <= 1_000_000 for r in a)
    sc = a[1].scene()
    assert not sc.bonded and abs(sc.n - a[1].n_hint) == 0


def test_server_policy_argument():
    from taichi_dem_julia_port_gb300.serving import ArenaSizing, Server
    with pytest.raises(ValueError):
        Server(ArenaSizing(1000, 1000, 4096, 2, 16, 8), policy="lifo")


class _DriftingHandle:
    """A stand-in for a stepping handle whose step cost falls as the run goes
    on (as when scenes settle), by more than the difference between shapes:
    the default shape is truly the fastest, but a candidate timed late in
    the descent looks faster than the baseline timed first."""

    def __init__(self):
        self.shape = {"force_block": 256, "force_grid": 152 * 16, "integrate_block": 256,
                      "force_blocks_per_sm": 0, "dependent_launch": 0,
                      "detect_blocks_per_sm": 4}
        self.default = dict(self.shape)
        self.t = 0

    def launch_shape(self):
        return dict(self.shape)

    def set_launch_shape(self, **shape):
        self.shape = dict(self.shape, **shape)

    def step(self, n):
        self.t += n

    def step_timed(self, n):
        cost = 1.0 if self.shape == self.default else 1.02
        total = sum(cost * (1.0 - 0.004 * min(self.t + k, 150)) for k in range(n))
        self.t += n
        return total


def test_autotune_confirms_its_choice():
    """The descent picks a shape that only looked faster because the run
    moved on; timing it against the starting shape on one stretch of the run
    reverts to the starting shape."""
    from taichi_dem_julia_port_gb300.autotune import autotune
    unconfirmed = _DriftingHandle()
    assert autotune(unconfirmed, steps=2, confirm_rounds=0).shape != unconfirmed.default
    h = _DriftingHandle()
    r = autotune(h, steps=2, confirm_rounds=2)
    assert r.shape == h.default
    assert h.shape == h.default
    chosen = [c for c, _ in r.trials if not c.get("baseline") and not c.get("confirm")]
    assert chosen, "the descent timed candidates"


def test_corrupt_p4p_is_rejected_with_its_line(tmp_path):
    """Malformed p4p input raises ValueError naming the file and line, before
    anything reaches the library."""
    from taichi_dem_julia_port_gb300.executor import load_particles
    good = ("TIMESTEP PARTICLES\n0.0 2\nID  GROUP  VOLUME  MASS  PX  PY  PZ  VX  VY  VZ\n"
            "1 0 4.1e-6 0.01 0.0 0.0 0.0 0.0 0.0 0.0\n"
            "2 0 4.1e-6 0.01 0.02 0.0 0.0 0.0 0.0 0.0\n")
    f = tmp_path / "good.p4p"
    f.write_text(good)
    assert load_particles(f).n == 2
    cases = {
        "header": ("PARTICLES\n" + good.split("\n", 1)[1], ":1:"),
        "count": (good.replace("0.0 2\n", "0.0 two\n"), ":2:"),
        "truncated": ("".join(good.splitlines(True)[:4]),
                      "announces 2 particles, the file has 1"),
        "columns": (good.replace("2 0 4.1e-6 0.01 0.02 0.0 0.0 0.0 0.0 0.0",
                                 "2 0 4.1e-6 0.01 0.02"), ":5: expected 10 columns"),
        "value": (good.replace("0.02 0.0 0.0", "0.02 x 0.0"), ":5:"),
    }
    for name, (text, msg) in cases.items():
        f = tmp_path / f"{name}.p4p"
        f.write_text(text)
        with pytest.raises(ValueError) as e:
            load_particles(f)
        assert msg in str(e.value), (name, str(e.value))


def test_bench_byte_model_for_the_cube_window():
    """bench.py's algorithmic bytes per kernel (every field once per unit)
    for the 17,576-sphere cube's timed window (48,096 contacts, 41,427 of
    them bonds): the figures its roofline divides by the phase times."""
    import bench
    alg = bench.algorithmic_bytes(17576, 48096, 41427)
    assert alg == {"force": 14570456, "integrate": 10175040, "contacts": 2182024}
    # a settling pour without contacts writes neither spin nor quaternion
    assert bench.algorithmic_bytes(1000, 0, 0, settling=True)["integrate"] == 1000 * (360 - 56)
    assert bench.algorithmic_bytes(1000, 0, 0)["force"] == 0


def test_first_bad_grain_named_in_a_large_scene(dem_lib_path):
    """Scene set-up checks every grain on the host before any device call,
    over several threads for large scenes (200,000 grains here), and names the
    first bad grain whichever thread finds it."""
    from taichi_dem_julia_port_gb300 import GlobalData
    from taichi_dem_julia_port_gb300.scenes import ParticleInput
    n = 200_000
    rng = np.random.default_rng(3)
    r = np.full(n, 1e-3)
    pos = rng.uniform(0.0, 0.2, (n, 3))
    cfg = DEMConfig(domain_min=[-0.01] * 3, domain_max=[0.21] * 3)
    for bad in ([150_001, 190_000], [7, 150_001], [199_999]):
        p = ParticleInput.from_arrays(r, pos.copy(), np.zeros((n, 3)), 2500.0)
        for k, i in enumerate(bad):
            if k % 2:
                p.volume[i] = -1.0
            else:
                p.pos[i, 2] = np.nan
        with pytest.raises(_abi.DemError) as e:
            GlobalData(cfg, p, lib=_abi.load_library(dem_lib_path))
        assert e.value.code == _abi.DEM_ERR_INVALID
        assert f"grain {bad[0]}:" in str(e.value), str(e.value)
