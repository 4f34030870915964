"""ctypes view of include/dem_gb300.h and the loader of libdem_sm100a.so.

The structures here mirror the header field for field; `ENTRY_POINTS` lists
every function the header declares with its ctypes signature.  The loader never
falls back to another implementation: a missing library is an error.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

DEM_OK = 0
DEM_ERR_INVALID = 1
DEM_ERR_CUDA = 2
DEM_ERR_CAPACITY = 3
DEM_ERR_TIMEOUT = 4
DEM_ERR_NO_DEVICE = 5
DEM_ERR_RANGE = 6

DEM_FP64 = 0
DEM_FP32_FORCE = 1

_D3 = C.c_double * 3


class DemConfigC(C.Structure):
    _fields_ = [
        ("domain_min", _D3),
        ("domain_max", _D3),
        ("particle_contact_radius_multiplier", C.c_double),
        ("neighboring_search_safety_factor", C.c_double),
        ("particle_elastic_modulus", C.c_double),
        ("particle_poisson_ratio", C.c_double),
        ("wall_normal", _D3),
        ("wall_distance", C.c_double),
        ("wall_density", C.c_double),
        ("wall_elastic_modulus", C.c_double),
        ("wall_poisson_ratio", C.c_double),
        ("bond_radius_ratio", C.c_double),
        ("bond_elastic_modulus", C.c_double),
        ("bond_poisson_ratio", C.c_double),
        ("bond_compressive_strength", C.c_double),
        ("bond_tensile_strength", C.c_double),
        ("bond_shear_strength", C.c_double),
        ("pp_coefficient_friction", C.c_double),
        ("pp_coefficient_restitution", C.c_double),
        ("pp_coefficient_rolling_resistance", C.c_double),
        ("pw_coefficient_friction", C.c_double),
        ("pw_coefficient_restitution", C.c_double),
        ("pw_coefficient_rolling_resistance", C.c_double),
        ("max_coordinate_number", C.c_int64),
        ("collision_pair_init_capacity_factor", C.c_int64),
        ("tolerance", C.c_double),
        ("max_particle_count", C.c_int64),
        ("gravity", _D3),
        ("global_damping", C.c_double),
        ("dt", C.c_double),
        ("target_time", C.c_double),
        ("saving_interval_time", C.c_double),
    ]


_PD = C.POINTER(C.c_double)
_PI32 = C.POINTER(C.c_int32)
_PU32 = C.POINTER(C.c_uint32)
_PU8 = C.POINTER(C.c_uint8)


class DemParticlesIn(C.Structure):
    _fields_ = [("n", C.c_int64), ("id", _PI32), ("gid", _PI32), ("volume", _PD),
                ("mass", _PD), ("pos", _PD), ("vel", _PD)]


class DemParticleState(C.Structure):
    # double* fields held as addresses (c_void_p: built from integers, which
    # keeps the per-step state exchange cheap)
    _fields_ = [("n", C.c_int64), ("pos", C.c_void_p), ("vel", C.c_void_p),
                ("omega", C.c_void_p), ("quat", C.c_void_p), ("force", C.c_void_p),
                ("moment", C.c_void_p), ("wall_shear", C.c_void_p)]


class DemParticleStatic(C.Structure):
    _fields_ = [("n", C.c_int64), ("radius", _PD), ("radius0", _PD), ("mass", _PD),
                ("inertia", _PD)]


class DemContacts(C.Structure):
    _fields_ = [("i", _PI32), ("j", _PI32), ("bonded", _PU8), ("point", _PD), ("force", _PD),
                ("torque_i", _PD), ("torque_j", _PD), ("shear", _PD)]


class DemDerived(C.Structure):
    _fields_ = [("cell_size", C.c_double), ("r_max", C.c_double), ("hash_table_size", C.c_int64),
                ("total_steps", C.c_int64), ("save_per_steps", C.c_int64),
                ("material_density", C.c_double), ("contact_capacity", C.c_int64)]


class DemMaterial(C.Structure):
    _fields_ = [("density", C.c_double), ("elastic_modulus", C.c_double),
                ("poisson_ratio", C.c_double)]


class DemSurface(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "friction", "restitution", "rolling_resistance", "bond_radius_ratio",
        "bond_elastic_modulus", "bond_poisson_ratio", "bond_compressive_strength",
        "bond_tensile_strength", "bond_shear_strength")]


class DemWall(C.Structure):
    _fields_ = [("normal", _D3), ("distance", C.c_double), ("material", C.c_int64)]


class DemTables(C.Structure):
    _fields_ = [("n_materials", C.c_int64), ("materials", C.POINTER(DemMaterial)),
                ("surfaces", C.POINTER(DemSurface)), ("n_walls", C.c_int64),
                ("walls", C.POINTER(DemWall)), ("grain_material", C.POINTER(C.c_int32))]


class DemStats(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("steps_done", C.c_int64), ("contacts", C.c_int64),
                ("bonded", C.c_int64), ("bonds_broken", C.c_int64), ("contacts_ended", C.c_int64),
                ("contacts_created", C.c_int64), ("warn_gap", C.c_int64),
                ("warn_damping", C.c_int64), ("error", C.c_int32), ("precision", C.c_int32),
                ("full_searches", C.c_int64), ("exchanges_direct", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class DemLaunchShape(C.Structure):
    _fields_ = [("force_block", C.c_int32), ("force_grid", C.c_int32),
                ("compact_block", C.c_int32), ("compact_grid", C.c_int32),
                ("integrate_block", C.c_int32), ("detect_blocks_per_sm", C.c_int32),
                ("force_blocks_per_sm", C.c_int32), ("dependent_launch", C.c_int32),
                ("list_lanes", C.c_int32), ("integrate_lanes", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


DEM_SCENE_FREE = 0
DEM_SCENE_FROZEN = 1
DEM_SCENE_STEP = 2
DEM_SCENE_INIT = 3


class DemArenaConfig(C.Structure):
    _fields_ = [("max_particles", C.c_int64), ("max_contacts", C.c_int64),
                ("max_buckets", C.c_int64), ("max_scenes", C.c_int32),
                ("max_coordinate_number", C.c_int32), ("precision", C.c_int32),
                ("pad", C.c_int32), ("cell_factor", C.c_double)]


class DemSceneInfo(C.Structure):
    _fields_ = [("mode", C.c_int32), ("pad", C.c_int32), ("n", C.c_int64),
                ("first_slot", C.c_int64), ("steps_done", C.c_int64),
                ("steps_target", C.c_int64), ("buckets", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


_H = C.c_void_p
_PH = C.POINTER(C.c_void_p)

# name -> (restype, argtypes); every function of include/dem_gb300.h
ENTRY_POINTS = {
    "dem_set_device": (C.c_int, [C.c_int]),
    "dem_create": (C.c_int, [C.POINTER(DemConfigC), C.POINTER(DemParticlesIn), _PH]),
    "dem_create_tables": (C.c_int, [C.POINTER(DemConfigC), C.POINTER(DemParticlesIn),
                                    C.POINTER(DemTables), _PH]),
    "dem_get_wall_shear": (C.c_int, [_H, C.c_int32, C.c_void_p]),
    "dem_set_wall_shear": (C.c_int, [_H, C.c_int32, C.c_void_p]),
    "dem_destroy": (C.c_int, [_H]),
    "dem_init_bonds": (C.c_int, [_H]),
    "dem_step": (C.c_int, [_H, C.c_int64]),
    "dem_step_timed": (C.c_int, [_H, C.c_int64, C.POINTER(C.c_float)]),
    "dem_step_profiled": (C.c_int, [_H, C.POINTER(C.c_float), C.c_int]),
    "dem_sync": (C.c_int, [_H]),
    "dem_set_precision": (C.c_int, [_H, C.c_int]),
    "dem_set_launch_shape": (C.c_int, [_H, C.POINTER(DemLaunchShape)]),
    "dem_get_launch_shape": (C.c_int, [_H, C.POINTER(DemLaunchShape)]),
    "dem_set_skin_factor": (C.c_int, [_H, C.c_int32, C.c_double]),
    "dem_get_particles": (C.c_int, [_H, C.POINTER(DemParticleState)]),
    "dem_set_particles": (C.c_int, [_H, C.POINTER(DemParticleState)]),
    "dem_set_particles_async": (C.c_int, [_H, C.POINTER(DemParticleState)]),
    "dem_step_exchange": (C.c_int, [_H, C.POINTER(DemParticleState), C.c_int64,
                                     C.POINTER(DemParticleState)]),
    "dem_host_alloc": (C.c_int, [C.c_int64, C.POINTER(C.c_void_p)]),
    "dem_host_free": (C.c_int, [C.c_void_p]),
    "dem_get_static": (C.c_int, [_H, C.POINTER(DemParticleStatic)]),
    "dem_get_derived": (C.c_int, [_H, C.POINTER(DemDerived)]),
    "dem_get_contacts": (C.c_int, [_H, C.POINTER(DemContacts), C.c_int64, C.POINTER(C.c_int64)]),
    "dem_get_io_contacts": (C.c_int, [_H, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "dem_scene_get_io_contacts": (C.c_int, [_H, C.c_int32, C.c_void_p, C.c_int64,
                                            C.POINTER(C.c_int64)]),
    "dem_set_contacts": (C.c_int, [_H, C.POINTER(DemContacts), C.c_int64]),
    "dem_get_stats": (C.c_int, [_H, C.POINTER(DemStats)]),
    "dem_debug_broadphase": (C.c_int, [_H, _PI32, _PU32, _PU32, _PU32, _PU32, _PI32, C.c_int64,
                                       C.POINTER(C.c_int64)]),
    "dem_arena_create": (C.c_int, [C.POINTER(DemArenaConfig), _PH]),
    "dem_arena_add": (C.c_int, [_H, C.POINTER(DemConfigC), C.POINTER(DemParticlesIn), C.c_int,
                                C.c_int64, C.POINTER(C.c_int32)]),
    "dem_arena_remove": (C.c_int, [_H, C.c_int32]),
    "dem_arena_set_cell_factor": (C.c_int, [_H, C.c_int32, C.c_double]),
    "dem_arena_scene_info": (C.c_int, [_H, C.c_int32, C.POINTER(DemSceneInfo)]),
    "dem_scene_get_particles": (C.c_int, [_H, C.c_int32, C.POINTER(DemParticleState)]),
    "dem_scene_get_contacts": (C.c_int, [_H, C.c_int32, C.POINTER(DemContacts), C.c_int64,
                                         C.POINTER(C.c_int64)]),
    "dem_scene_get_stats": (C.c_int, [_H, C.c_int32, C.POINTER(DemStats)]),
    "dem_scene_get_derived": (C.c_int, [_H, C.c_int32, C.POINTER(DemDerived)]),
    "dem_bucket_sort_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                          C.POINTER(C.c_double), C.c_double, C.c_int64,
                                          C.c_void_p, C.c_void_p, C.c_void_p]),
    "dem_selftest_conversions": (C.c_int, [C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "dem_selftest_wait_timeout": (C.c_int, [C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_int)]),
    "dem_debug_step_enumeration": (C.c_int, [_H, C.POINTER(C.c_int64), C.POINTER(C.c_uint64)]),
    "dem_strerror": (C.c_char_p, [C.c_int]),
    "dem_version": (C.c_char_p, []),
}

# DemIOContact: one p4c line (i, j 0-based; bonded; 𝐤; 𝐅ᵢ), 64 bytes
IO_CONTACT_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("bonded", "<i4"), ("pad", "<i4"),
                             ("point", "<f8", (3,)), ("force", "<f8", (3,))])
assert IO_CONTACT_DTYPE.itemsize == 64

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libdem_sm100a.so"


class DemError(RuntimeError):
    def __init__(self, code: int, where: str, message: str = ""):
        self.code = code
        super().__init__(f"{where}: DEM error {code}: {message}")


_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libdem_sm100a.so (built in-tree by taichi_dem_julia_port_gb300.build).

    Raises FileNotFoundError when the library has not been built: there is no
    fallback implementation."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing; build it with `python -m taichi_dem_julia_port_gb300.build` "
            "(the DEM step runs only through this CUDA library)")
    lib = C.CDLL(str(p))
    for name, (res, args) in ENTRY_POINTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(lib, rc: int, where: str) -> None:
    if rc != DEM_OK:
        raise DemError(rc, where, lib.dem_strerror(rc).decode())


def ptr(a: np.ndarray | None, ctype):
    """Pointer to a contiguous numpy array's data (None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))
