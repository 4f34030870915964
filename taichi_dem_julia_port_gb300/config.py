"""`DEMConfig` — the 33 keys of the reference's config (src/config.jl:3-45).

Same names, defaults and meaning; `from_toml` reads the same TOML files
(src/executor.jl:182).  Keys absent from a file take the defaults below.
"""
from __future__ import annotations

import dataclasses
import tomllib
from dataclasses import dataclass, field
from pathlib import Path

from ._abi import DemConfigC


def _v3(*x):
    return field(default_factory=lambda: list(x))


@dataclass
class DEMConfig:
    domain_min: list = _v3(-200.0, -200.0, -30.0)
    domain_max: list = _v3(200.0, 200.0, 90.0)
    init_particles: str = "../Resources/bunny.p4p"
    particle_contact_radius_multiplier: float = 1.1
    neighboring_search_safety_factor: float = 1.01
    particle_elastic_modulus: float = 7e10
    particle_poisson_ratio: float = 0.25
    wall_normal: list = _v3(0.0, 0.0, -1.0)
    wall_distance: float = 25.0
    wall_density: float = 7800.0
    wall_elastic_modulus: float = 2e11
    wall_poisson_ratio: float = 0.25

    bond_radius_ratio: float = 0.5
    bond_elastic_modulus: float = 28e9
    bond_poisson_ratio: float = 0.2
    bond_compressive_strength: float = 3e8
    bond_tensile_strength: float = 6e7
    bond_shear_strength: float = 6e7

    pp_coefficient_friction: float = 0.3
    pp_coefficient_restitution: float = 0.9
    pp_coefficient_rolling_resistance: float = 0.01

    pw_coefficient_friction: float = 0.35
    pw_coefficient_restitution: float = 0.7
    pw_coefficient_rolling_resistance: float = 0.01

    max_coordinate_number: int = 64
    collision_pair_init_capacity_factor: int = 128

    tolerance: float = 1e-12
    max_particle_count: int = 1000000000

    gravity: list = _v3(0.0, 0.0, -9.81)
    global_damping: float = 0.0
    dt: float = 2.63e-5
    target_time: float = 0.5
    saving_interval_time: float = 0.05

    # ---- construction -------------------------------------------------------
    @classmethod
    def from_dict(cls, d: dict) -> "DEMConfig":
        names = {f.name for f in dataclasses.fields(cls)}
        unknown = set(d) - names
        if unknown:
            raise ValueError(f"unknown DEMConfig keys: {sorted(unknown)}")
        cfg = cls()
        for k, v in d.items():
            f = next(f for f in dataclasses.fields(cls) if f.name == k)
            if f.type in ("list", list):
                v = [float(x) for x in v]
                if len(v) != 3:
                    raise ValueError(f"{k} must have 3 components")
            elif f.type in ("int", int):
                v = int(v)
            elif f.type in ("float", float):
                v = float(v)
            setattr(cfg, k, v)
        return cfg

    @classmethod
    def from_toml(cls, path: str | Path) -> "DEMConfig":
        with open(path, "rb") as fh:
            return cls.from_dict(tomllib.load(fh))

    def to_toml(self) -> str:
        lines = []
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, str):
                lines.append(f'{f.name} = "{v}"')
            elif isinstance(v, list):
                lines.append(f"{f.name} = [{', '.join(repr(float(x)) for x in v)}]")
            else:
                lines.append(f"{f.name} = {v!r}")
        return "\n".join(lines) + "\n"

    def replace(self, **kw) -> "DEMConfig":
        return dataclasses.replace(self, **kw)

    # ---- C ABI --------------------------------------------------------------
    def to_c(self) -> DemConfigC:
        c = DemConfigC()
        for name, _ in DemConfigC._fields_:
            v = getattr(self, name)
            if isinstance(v, list):
                getattr(c, name)[:] = [float(x) for x in v]
            else:
                setattr(c, name, v)
        return c

    # ---- derived (src/executor.jl:262-263) -----------------------------------
    @property
    def total_steps(self) -> int:
        return int(self.target_time / self.dt)

    @property
    def save_per_steps(self) -> int:
        return int(self.saving_interval_time / self.dt)
