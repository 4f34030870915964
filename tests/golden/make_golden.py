"""Generates the golden vectors under tests/golden/ (run in a checkout where the
reference repository is available; the GPU machine never runs this script).

1. Reference-generated: `morton3d32` (dem.py:758-777) and `quat2RotMatrix`
   (dem.py:317-344) are pure-Python arithmetic inside Taichi decorators.  They
   are taken from the reference's own dem.py with `ast`, stripped of the
   decorators and executed here on seeded inputs.  The Morton vectors follow
   README.md:23: cartesian3morton(ijk) == morton3d32(ijk - 1) + 1.
2. Oracle-generated regression vectors for small scenes (the CPU oracle's own
   outputs, to detect unintended changes of the oracle).

    python tests/golden/make_golden.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import ast
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def _extract(src: str, name: str) -> ast.FunctionDef:
    for node in ast.walk(ast.parse(src)):
        if isinstance(node, ast.FunctionDef) and node.name == name:
            node.decorator_list = []
            for a in node.args.args:
                a.annotation = None
            node.returns = None
            return node
    raise KeyError(name)


def reference_functions(dem_py: Path) -> dict:
    src = dem_py.read_text()
    mod = ast.Module(body=[_extract(src, "morton3d32"), _extract(src, "quat2RotMatrix")],
                     type_ignores=[])
    ns = {"Zero3x3": lambda: np.zeros((3, 3))}
    exec(compile(ast.fix_missing_locations(mod), str(dem_py), "exec"), ns)
    return ns


def morton_vectors(ns, rng) -> list:
    cells = [(2, 3, 4), (1, 1, 1), (1024, 1024, 1024), (1025, 1, 1), (0, 0, 0), (-1, 5, 9)]
    for x in range(1, 9):
        for y in range(1, 9):
            for z in range(1, 9):
                cells.append((x, y, z))
    cells += [tuple(int(v) for v in rng.integers(1, 1025, size=3)) for _ in range(2000)]
    cells += [tuple(int(v) for v in rng.integers(-2000, 3000, size=3)) for _ in range(200)]
    out = []
    for (x, y, z) in cells:
        out.append([x, y, z, int(ns["morton3d32"](x - 1, y - 1, z - 1)) + 1])
    return out


def quat_vectors(ns, rng) -> list:
    out = []
    for _ in range(200):
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        R = np.asarray(ns["quat2RotMatrix"](list(q)), dtype=np.float64)
        out.append({"q": q.tolist(), "R": R.ravel().tolist()})
    return out


def oracle_vectors() -> dict:
    """Small-scene regression vectors from the CPU oracle."""
    from oracle.oracle import OracleScene
    from taichi_dem_julia_port_gb300 import scenes

    res = {}
    sc = scenes.bonded_cube(3, speed=10.0, steps=0, seed=7)
    o = OracleScene(sc.cfg, sc.particles)
    o.initialize()
    o.simulate(150)
    p, c = o.particles(), o.contacts()
    res["cube3_150"] = {"pos": p["pos"].tolist(), "vel": p["vel"].tolist(),
                        "force": p["force"].tolist(), "pairs": np.stack([c["i"], c["j"]], 1).tolist(),
                        "bonded": c["bonded"].tolist(), "stats": o.stats()}
    return res


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $DEM_REFERENCE, else ../reference)")
    args = ap.parse_args()
    if args.reference is None:
        from tests.reference_scenes import reference_checkout
        found = reference_checkout()
        if found is None:
            ap.error("no reference checkout: give --reference PATH or set DEM_REFERENCE")
        args.reference = str(found)
    rng = np.random.default_rng(20231203)
    ns = reference_functions(Path(args.reference) / "dem.py")
    golden = {
        "source": "dem.py morton3d32 / quat2RotMatrix executed from the reference source",
        "readme_kat": {"cartesian3morton": [2, 3, 4], "value": 54},
        "morton": morton_vectors(ns, rng),
        "quat2rot": quat_vectors(ns, rng),
    }
    (HERE / "reference_functions.json").write_text(json.dumps(golden))
    (HERE / "oracle_regression.json").write_text(json.dumps(oracle_vectors()))
    print("wrote", HERE / "reference_functions.json", HERE / "oracle_regression.json")


if __name__ == "__main__":
    main()
