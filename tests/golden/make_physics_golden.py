"""Generates tests/golden/reference_physics.json: golden vectors for the contact
forces, wall forces and time integration, computed by the reference's own
dem.py methods executed from its source.

The methods are taken from class DEMSolver in the reference's dem.py with
`ast` (decorators and annotations removed) and run on the CPU against the
numpy stand-in for Taichi in tests/golden/taichi_standin.py:

    resolve           dem.py:1357-1606  bonded (EBPM) and Hertz-Mindlin pairs
    evaluate_wall     dem.py:1609-1712  particle-wall Hertz-Mindlin
    resolve_wall      dem.py:1715-1743  the wall contact's begin/end rule
    apply_body_force  dem.py:1280-1305  gravity and global damping
    update            dem.py:1309-1354  translation, Euler's equations, quaternion
    quat2RotMatrix    dem.py:317-344

The contact-slot bookkeeping that `resolve` calls (dem.py:1188-1205) is
replaced by two small methods here: one slot per pair, found or appended.

Each case stores its inputs (material, surface and wall constants, dt, grain
state, carried contact state) and dem.py's outputs.  tests/test_oracle.py
runs the same inputs through the oracle's resolve_one / resolve_wall /
body_and_update and compares.  The bond cases include strengths set just
below and just above the stress that the case reaches, so that the breakage
decisions are pinned, not only the arithmetic.

    python tests/golden/make_physics_golden.py [--reference PATH]
(PATH is the reference checkout; without the option, $DEM_REFERENCE or a
directory `reference` beside this repository.)
"""
from __future__ import annotations

import argparse
import ast
import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import taichi_standin as S  # noqa: E402

METHODS = ["resolve", "evaluate_wall", "resolve_wall", "apply_body_force", "update"]
TOL = 1e-12  # dem.py DoublePrecisionTolerance, src/config.jl `tolerance` default


def _strip(fn: ast.FunctionDef) -> ast.FunctionDef:
    fn.decorator_list = []
    for a in fn.args.args:
        a.annotation = None
    fn.returns = None
    return fn


def load_reference(dem_py: Path):
    """Returns (RefSolver class, namespace) built from dem.py's source."""
    tree = ast.parse(dem_py.read_text())
    funcs = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.ClassDef) and node.name == "DEMSolver":
            for item in node.body:
                if isinstance(item, ast.FunctionDef) and item.name in METHODS:
                    funcs[item.name] = _strip(item)
        if isinstance(node, ast.FunctionDef) and node.name == "quat2RotMatrix":
            funcs["quat2RotMatrix"] = _strip(node)
    missing = set(METHODS + ["quat2RotMatrix"]) - set(funcs)
    if missing:
        raise KeyError(f"not found in {dem_py}: {sorted(missing)}")
    ns = {
        "ti": S.ti, "tm": S.tm, "Vector3": S.Vector3, "Vector4": S.Vector4,
        "DEMMatrix": S.DEMMatrix, "Zero3x3": S.Zero3x3, "Matrix3x3": S.DEMMatrix,
        "Contact": S.record_type(S.CONTACT), "DoublePrecisionTolerance": TOL,
        "set_max_coordinate_number": 16, "Integer": int, "Real": float,
    }
    mod = ast.Module(body=list(funcs.values()), type_ignores=[])
    exec(compile(ast.fix_missing_locations(mod), str(dem_py), "exec"), ns)

    class RefSolver:
        """Holds the fields that the extracted methods read through `self`."""

        def __init__(self, n, params):
            self.config = S.SimpleNamespace(
                dt=params["dt"], gravity=S.vec(params["gravity"]),
                global_damping=params["global_damping"])
            ns["config"] = self.config  # apply_body_force reads the module-level `config`
            self.gf = S.Field(S.GRAIN, n)
            self.cf = S.Field(S.CONTACT, n)
            self.cfn = [0] * n
            self.mf = S.Field(S.MATERIAL, 2)
            self.surf = S.Field(S.SURFACE, (2, 2))
            self.wf = S.Field(S.WALL, 1)
            self.wcf = S.Field(S.CONTACT, (n, 1))
            m = params
            self.mf[0] = S.make_record(S.MATERIAL, density=0.0, elasticModulus=m["E"],
                                       poissonRatio=m["nu"])
            self.mf[1] = S.make_record(S.MATERIAL, density=0.0, elasticModulus=m["wall_E"],
                                       poissonRatio=m["wall_nu"])
            self.surf[0, 0] = S.make_record(
                S.SURFACE, coefficientFriction=m["mu"], coefficientRestitution=m["e"],
                radius_ratio=m["bond_ratio"], elasticModulus=m["bond_E"],
                poissonRatio=m["bond_nu"], compressiveStrength=m["sc"],
                tensileStrength=m["st"], shearStrength=m["ss"])
            pw = S.make_record(S.SURFACE, coefficientFriction=m["pw_mu"],
                               coefficientRestitution=m["pw_e"])
            self.surf[0, 1] = pw
            self.surf[1, 0] = pw
            self.wf[0] = S.make_record(S.WALL, normal=m["wall_n"], distance=m["wall_d"],
                                       materialType=1)

        # one contact slot per particle pair (stands in for dem.py:1188-1205)
        def append_contact_offset(self, i):
            off = self.cfn[i]
            self.cfn[i] += 1
            return off if off < 1 else -1

        def search_active_contact_offset(self, i, j):
            if self.cfn[i] and self.cf[i].j == j and self.cf[i].isActive:
                return i
            return -1

    for name in METHODS:
        setattr(RefSolver, name, ns[name])
    return RefSolver, ns


# ---- case generation --------------------------------------------------------

def rand_params(rng) -> dict:
    lu = lambda a, b: float(math.exp(rng.uniform(math.log(a), math.log(b))))  # noqa: E731
    n = rng.standard_normal(3)
    return {
        "E": lu(1e7, 1e10), "nu": float(rng.uniform(0.15, 0.35)),
        "wall_E": lu(1e8, 2e11), "wall_nu": float(rng.uniform(0.2, 0.3)),
        "mu": float(rng.uniform(0.1, 0.9)), "e": float(rng.uniform(0.3, 0.95)),
        "pw_mu": float(rng.uniform(0.1, 0.9)), "pw_e": float(rng.uniform(0.3, 0.95)),
        "bond_ratio": float(rng.uniform(0.3, 0.7)), "bond_E": lu(1e7, 1e10),
        "bond_nu": float(rng.uniform(0.15, 0.35)),
        "sc": 1e300, "st": 1e300, "ss": 1e300,
        "dt": lu(1e-7, 1e-5), "gravity": (rng.standard_normal(3) * 5).tolist(),
        "global_damping": 0.0,
        "wall_n": (n / np.linalg.norm(n)).tolist(), "wall_d": float(rng.uniform(-0.1, 0.1)),
    }


def rand_grain(rng, pos, r=None, spin=True) -> dict:
    r = float(rng.uniform(5e-4, 2e-2)) if r is None else r
    rho = float(rng.uniform(1000, 8000))
    m = rho * 4.0 / 3.0 * math.pi * r ** 3
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    return {"r": r, "m": m, "k": list(map(float, pos)),
            "v": (rng.uniform(-5, 5, 3)).tolist(),
            "w": (rng.uniform(-200, 200, 3) if spin else np.zeros(3)).tolist(),
            "q": q.tolist(), "I": 0.4 * m * r * r}


def unit(rng, kind):
    if kind == "x+":
        return np.array([1.0, 0.0, 0.0])
    if kind == "x-":
        return np.array([-1.0, 0.0, 0.0])
    if kind == "near_x":  # s just above the tolerance
        d = np.array([1.0, 3e-12, 0.0])
        return d / np.linalg.norm(d)
    d = rng.standard_normal(3)
    return d / np.linalg.norm(d)


def set_grain(solver, idx, g):
    solver.gf[idx] = S.make_record(
        S.GRAIN, mass=g["m"], radius=g["r"], contactRadius=g["r"], position=g["k"],
        velocity=g["v"], quaternion=g["q"], omega=g["w"], inertia=np.eye(3) * g["I"])


def run_pair(Ref, params, gi, gj, state, bonded):
    sol = Ref(2, params)
    set_grain(sol, 0, gi)
    set_grain(sol, 1, gj)
    if state is not None:
        sol.cfn[0] = 1
        sol.cf[0] = S.make_record(
            S.CONTACT, i=0, j=1, isActive=1, isBonded=int(bonded), force_a=state[0:3],
            moment_a=state[3:6], moment_b=state[6:9], shear_displacement=state[9:12])
    sol.resolve(0, 1)
    c = sol.cf[0]
    return {
        "fi": sol.gf[0].force.tolist(), "fj": sol.gf[1].force.tolist(),
        "mi": sol.gf[0].moment.tolist(), "mj": sol.gf[1].moment.tolist(),
        "active": int(c.isActive), "bonded": int(c.isBonded),
        "k": c.position.tolist(), "F": c.force_a.tolist(), "ti": c.moment_a.tolist(),
        "tj": c.moment_b.tolist(), "s": c.shear_displacement.tolist(),
    }


def bond_stresses(params, gi, gj, out):
    """The three stresses that dem.py:1487-1493 tests, from the case's output
    state (only used to place strengths around them)."""
    rb = params["bond_ratio"] * min(gi["r"], gj["r"])
    A = math.pi * rb ** 2
    I = rb ** 4 * math.pi / 4.0
    F, ta, tb = out["F"], out["ti"], out["tj"]
    sa = -F[0] / A - rb / I * math.sqrt(ta[1] ** 2 + ta[2] ** 2)
    sb = -F[0] / A - rb / I * math.sqrt(tb[1] ** 2 + tb[2] ** 2)
    tau = abs(ta[0]) * rb / 2.0 / I + 4.0 / 3.0 / A * math.sqrt(F[1] ** 2 + F[2] ** 2)
    return {"sc": -min(sa, sb), "st": max(sa, sb), "ss": tau}


def bond_cases(Ref, rng, count, with_thresholds):
    cases = []
    kinds = ["rand"] * 6 + ["x+", "x-", "near_x"]
    for n in range(count):
        p = rand_params(rng)
        d = unit(rng, kinds[len(cases) % len(kinds)])
        gi = rand_grain(rng, rng.uniform(-0.1, 0.1, 3))
        rj = float(rng.uniform(5e-4, 2e-2))
        L = (gi["r"] + rj) * float(rng.uniform(0.95, 1.05))
        gj = rand_grain(rng, np.array(gi["k"]) + L * d, r=rj)
        rb = p["bond_ratio"] * min(gi["r"], rj)
        A, I = math.pi * rb * rb, rb ** 4 * math.pi / 4
        fs, ms = p["bond_E"] * A * 1e-4, p["bond_E"] * I / L * 1e-3
        state = np.concatenate([rng.standard_normal(3) * fs, rng.standard_normal(6) * ms,
                                np.zeros(3)]).tolist()
        case = {"params": p, "gi": gi, "gj": gj, "state": state, "bonded": 1}
        case["out"] = run_pair(Ref, p, gi, gj, state, True)
        cases.append(case)
        if n >= with_thresholds:
            continue
        # strengths placed a relative 1e-9 below / above each positive stress
        sig = bond_stresses(p, gi, gj, case["out"])
        for mode, val in sig.items():
            if not (val > 0 and math.isfinite(val)):
                continue
            for rel in (1.0 - 1e-9, 1.0 + 1e-9):
                q = dict(p)
                q[mode] = val * rel
                cc = {"params": q, "gi": gi, "gj": gj, "state": state, "bonded": 1,
                      "threshold": {"mode": mode, "rel": rel}}
                cc["out"] = run_pair(Ref, q, gi, gj, state, True)
                cases.append(cc)
    return cases


def hertz_cases(Ref, rng, count):
    cases = []
    kinds = ["rand"] * 6 + ["x+", "x-", "near_x"]
    for n in range(count):
        p = rand_params(rng)
        d = unit(rng, kinds[n % len(kinds)])
        gi = rand_grain(rng, rng.uniform(-0.1, 0.1, 3), spin=n % 5 != 0)
        rj = float(rng.uniform(5e-4, 2e-2))
        delta = (gi["r"] + rj) * float(10 ** rng.uniform(-4, -1.7))
        gj = rand_grain(rng, np.array(gi["k"]) + (gi["r"] + rj - delta) * d, r=rj,
                        spin=n % 5 != 0)
        existing = n % 3 != 0
        if existing:
            mag = delta * (10 ** rng.uniform(-4, 0))  # large histories slide
            s = np.concatenate([[0.0], rng.standard_normal(2) * mag]).tolist()
            state = [0.0] * 9 + s
        else:
            state = None
        out = run_pair(Ref, p, gi, gj, state, False)
        cases.append({"params": p, "gi": gi, "gj": gj,
                      "state": state if state is not None else [0.0] * 12,
                      "bonded": 0, "new": int(not existing), "out": out})
    return cases


def wall_cases(Ref, rng, count):
    cases = []
    for n in range(count):
        p = rand_params(rng)
        kind = n % 6
        if kind == 1:
            p["wall_n"] = [1.0, 0.0, 0.0]
        elif kind == 2:
            p["wall_n"] = [0.0, 0.0, -1.0]
        elif kind == 3:
            p["wall_n"] = [-1.0, 0.0, 0.0]
        nrm = np.array(p["wall_n"])
        g = rand_grain(rng, np.zeros(3), spin=n % 4 != 0)
        frac = float(rng.uniform(0.9, 0.9999)) if n % 7 else float(rng.uniform(1.0001, 1.2))
        side = 1.0 if n % 2 else -1.0
        base = rng.uniform(-0.1, 0.1, 3)
        base = base - (base @ nrm - p["wall_d"]) * nrm  # a point on the plane
        g["k"] = (base + side * frac * g["r"] * nrm).tolist()
        existing = n % 3 != 0
        s_in = (np.concatenate([[0.0], rng.standard_normal(2)]) * g["r"] *
                10 ** rng.uniform(-5, -1)).tolist() if existing else [0.0, 0.0, 0.0]
        sol = Ref(1, p)
        set_grain(sol, 0, g)
        if existing:
            sol.wcf[0, 0] = S.make_record(S.CONTACT, isActive=1, materialType_i=0,
                                          materialType_j=1, shear_displacement=s_in)
        sol.resolve_wall()
        wc = sol.wcf[0, 0]
        out = {"touch": int(wc.isActive), "f": sol.gf[0].force.tolist(),
               "m": sol.gf[0].moment.tolist(), "k": wc.position.tolist(),
               "F": wc.force_a.tolist(), "s": wc.shear_displacement.tolist()}
        cases.append({"params": p, "g": g, "s_in": s_in, "existing": int(existing), "out": out})
    return cases


def update_cases(Ref, rng, batches, n):
    cases = []
    for b in range(batches):
        p = rand_params(rng)
        p["global_damping"] = [0.0, 0.05, 0.3, 0.9][b % 4]
        grains, F, T = [], [], []
        for i in range(n):
            g = rand_grain(rng, rng.uniform(-0.1, 0.1, 3), spin=i % 4 != 0)
            f = rng.standard_normal(3) * g["m"] * 1e3
            t = rng.standard_normal(3) * g["I"] * 1e4
            if i % 5 == 0:  # zero components: sign(0) in the damping term
                g["v"][i % 3] = 0.0
                f[(i + 1) % 3] = 0.0
                t[i % 3] = 0.0
            if i % 7 == 0:
                g["q"] = [1.0, 0.0, 0.0, 0.0]
            grains.append(g)
            F.append(f.tolist())
            T.append(t.tolist())
        sol = Ref(n, p)
        for i, g in enumerate(grains):
            set_grain(sol, i, g)
            sol.gf[i].force = S.vec(F[i])
            sol.gf[i].moment = S.vec(T[i])
        sol.apply_body_force()
        ft = [sol.gf[i].force.tolist() for i in range(n)]
        mt = [sol.gf[i].moment.tolist() for i in range(n)]
        sol.update()
        out = [{"k": sol.gf[i].position.tolist(), "v": sol.gf[i].velocity.tolist(),
                "q": sol.gf[i].quaternion.tolist(), "w": sol.gf[i].omega.tolist(),
                "F": ft[i], "T": mt[i]} for i in range(n)]
        cases.append({"params": p, "grains": grains, "F": F, "T": T, "out": out})
    return cases


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $DEM_REFERENCE, else ../reference)")
    args = ap.parse_args()
    if args.reference is None:
        sys.path.insert(0, str(HERE.parents[1]))
        from tests.reference_scenes import reference_checkout
        found = reference_checkout()
        if found is None:
            ap.error("no reference checkout: give --reference PATH or set DEM_REFERENCE")
        args.reference = str(found)
    Ref, _ = load_reference(Path(args.reference) / "dem.py")
    rng = np.random.default_rng(20261204)
    golden = {
        "source": "dem.py DEMSolver.resolve / evaluate_wall / resolve_wall / "
                  "apply_body_force / update executed from the reference source",
        "tolerance": TOL,
        "bond": bond_cases(Ref, rng, 60, 14),
        "hertz": hertz_cases(Ref, rng, 180),
        "wall": wall_cases(Ref, rng, 120),
        "update": update_cases(Ref, rng, 8, 24),
    }
    path = HERE / "reference_physics.json"
    path.write_text(json.dumps(golden, separators=(",", ":")))
    print("wrote", path, {k: len(v) for k, v in golden.items() if isinstance(v, list)})


if __name__ == "__main__":
    main()
