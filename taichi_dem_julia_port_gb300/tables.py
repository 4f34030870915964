"""Material, surface and wall tables of a scene (the reference's
GlobalData.materials / surfaces / walls and Grain.mid; src/types.jl:9-27,
58-62, src/executor.jl:1-29).

The reference's kernels read the tables per contact (surfaces[midᵢ, midⱼ],
materials[midᵢ], materials[midⱼ]; src/kernels.jl:175-177, 255-263) and loop
over the walls per particle (src/kernels.jl:317-426).  Its `solve` fills them
with one particle material, one wall material and one wall
(src/executor.jl:282-315): `Tables.standard` builds exactly that.  Indices
here are 0-based (the reference's mid - 1).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi

MAX_MATERIALS = 8
MAX_WALLS = 8


@dataclass
class Material:
    """Material (src/types.jl:9-13)."""
    density: float
    elastic_modulus: float
    poisson_ratio: float


@dataclass
class Surface:
    """Surface (src/types.jl:17-27): Hertz-Mindlin friction and restitution,
    the declared (unused) rolling resistance, and the EBPM bond's radius
    ratio, modulus, Poisson ratio and strengths."""
    friction: float
    restitution: float
    rolling_resistance: float = 0.0
    bond_radius_ratio: float = 0.0
    bond_elastic_modulus: float = 0.0
    bond_poisson_ratio: float = 0.0
    bond_compressive_strength: float = 0.0
    bond_tensile_strength: float = 0.0
    bond_shear_strength: float = 0.0


@dataclass
class Wall:
    """Wall (src/types.jl:58-62): the plane normal·x = distance."""
    normal: list
    distance: float
    material: int


@dataclass
class Tables:
    materials: list
    surfaces: list           # n x n: surfaces[a][b] for materials a, b
    walls: list
    grain_material: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))

    @classmethod
    def standard(cls, cfg, particles) -> "Tables":
        """The tables `solve` builds (src/executor.jl:282-315): material 0 the
        particles' (density of the last grain, the config's modulus and
        Poisson ratio), material 1 the wall's, the particle-particle and
        particle-wall surfaces, and the config's one wall."""
        n = particles.n
        rho = float(particles.mass[-1] / particles.volume[-1]) if n else 0.0
        pp = Surface(cfg.pp_coefficient_friction, cfg.pp_coefficient_restitution,
                     cfg.pp_coefficient_rolling_resistance, cfg.bond_radius_ratio,
                     cfg.bond_elastic_modulus, cfg.bond_poisson_ratio,
                     cfg.bond_compressive_strength, cfg.bond_tensile_strength,
                     cfg.bond_shear_strength)
        pw = Surface(cfg.pw_coefficient_friction, cfg.pw_coefficient_restitution,
                     cfg.pw_coefficient_rolling_resistance)
        return cls(materials=[Material(rho, cfg.particle_elastic_modulus, cfg.particle_poisson_ratio),
                              Material(cfg.wall_density, cfg.wall_elastic_modulus,
                                       cfg.wall_poisson_ratio)],
                   surfaces=[[pp, pw], [pw, Surface(0.0, 0.0)]],
                   walls=[Wall(list(cfg.wall_normal), cfg.wall_distance, 1)],
                   grain_material=np.zeros(n, np.int32))

    def to_c(self):
        """(DemTables, keep-alive list) for dem_create_tables / the oracle."""
        nm = len(self.materials)
        if not 1 <= nm <= MAX_MATERIALS or not 0 <= len(self.walls) <= MAX_WALLS:
            raise ValueError("1-8 materials and 0-8 walls")
        if len(self.surfaces) != nm or any(len(row) != nm for row in self.surfaces):
            raise ValueError("surfaces must be an n x n table")
        mats = (_abi.DemMaterial * nm)(*[_abi.DemMaterial(m.density, m.elastic_modulus,
                                                          m.poisson_ratio) for m in self.materials])
        surfs = (_abi.DemSurface * (nm * nm))(*[
            _abi.DemSurface(s.friction, s.restitution, s.rolling_resistance, s.bond_radius_ratio,
                            s.bond_elastic_modulus, s.bond_poisson_ratio,
                            s.bond_compressive_strength, s.bond_tensile_strength,
                            s.bond_shear_strength)
            for row in self.surfaces for s in row])
        nw = len(self.walls)
        walls = (_abi.DemWall * max(nw, 1))(*[
            _abi.DemWall((C.c_double * 3)(*[float(x) for x in w.normal]), w.distance, w.material)
            for w in self.walls])
        gm = np.ascontiguousarray(self.grain_material, np.int32)
        t = _abi.DemTables(nm, C.cast(mats, C.POINTER(_abi.DemMaterial)),
                           C.cast(surfs, C.POINTER(_abi.DemSurface)), nw,
                           C.cast(walls, C.POINTER(_abi.DemWall)),
                           gm.ctypes.data_as(C.POINTER(C.c_int32)))
        return t, [mats, surfs, walls, gm]
