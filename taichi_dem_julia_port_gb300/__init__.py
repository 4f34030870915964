"""GB300 (sm_103a) DEM time step with the surface of the reference package
DEMPort (lucifer1004/taichi_dem_julia_port).

    from taichi_dem_julia_port_gb300 import DEMConfig, GlobalData, solve

The step itself lives in libdem_sm100a.so (hand-written CUDA, C ABI in
include/dem_gb300.h); this package is its host front end.
"""
from .arena import Arena
from .config import DEMConfig
from .executor import (GlobalData, StateBuffers, initialize, load_particles, save_single, simulate,
                       solve)
from .p4io import compare_p4c, compare_p4p, read_p4c, read_p4p
from .scenes import ParticleInput, bonded_cube, granular_pour
from .tables import Material, Surface, Tables, Wall

DEMConfigDefault = DEMConfig

__all__ = [
    "Arena", "DEMConfig", "DEMConfigDefault", "GlobalData", "StateBuffers", "initialize",
    "simulate", "solve",
    "load_particles", "save_single", "read_p4p", "read_p4c", "compare_p4p", "compare_p4c",
    "ParticleInput", "bonded_cube", "granular_pour", "Material", "Surface", "Wall", "Tables",
]
