"""Many independent scenes stepped together in one device arena.

The reference steps one scene per process (`solve`, src/executor.jl:174-394).
An `Arena` holds many scenes in shared particle slots, contact buffers and
bucket table (dem_arena_* in include/dem_gb300.h); every `step` advances each
scene in Step mode by one `simulate!` inside the same kernels.  Scenes can be
added and removed between steps without changing the captured step graph,
which is what batched runs (a fixed set of scenes) and the serving loop (scenes
arriving and leaving) use.  A scene's results are bit-for-bit those of the same
scene run alone (`GlobalData`).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import check, ptr
from .config import DEMConfig
from .executor import (PRECISIONS, _f64, get_launch_shape, read_contacts, read_particles,
                       set_launch_shape)
from .scenes import ParticleInput

MODES = {_abi.DEM_SCENE_FREE: "free", _abi.DEM_SCENE_FROZEN: "frozen",
         _abi.DEM_SCENE_STEP: "step", _abi.DEM_SCENE_INIT: "init"}


def buckets_for(n: int) -> int:
    """Bucket-table entries a scene of n particles takes: the power of two of
    at least 2n, and at least 1024 (mirrors dem_arena_add)."""
    H = 1024
    while H < 2 * n:
        H <<= 1
    return H


@dataclass
class _SceneRec:
    cfg: DEMConfig
    particles: ParticleInput
    cfg_c: object


class Arena:
    """Device arena of independent scenes (dem_arena_create)."""

    def __init__(self, max_particles: int, max_scenes: int = 256,
                 max_contacts: int | None = None, max_buckets: int | None = None,
                 max_coordinate_number: int = 16, precision: str = "fp64",
                 cell_factor: float = 0.0, lib=None):
        self.lib = lib or _abi.load_library()
        if max_contacts is None:
            max_contacts = max_particles * max_coordinate_number
        if max_buckets is None:
            max_buckets = 4 * max_particles + 1024 * max_scenes
        self.max_particles, self.max_scenes = int(max_particles), int(max_scenes)
        self.max_contacts, self.max_buckets = int(max_contacts), int(max_buckets)
        self.precision = precision
        ac = _abi.DemArenaConfig(self.max_particles, self.max_contacts, self.max_buckets,
                                 self.max_scenes, int(max_coordinate_number),
                                 PRECISIONS[precision], 0, float(cell_factor))
        h = C.c_void_p()
        check(self.lib, self.lib.dem_arena_create(C.byref(ac), C.byref(h)), "dem_arena_create")
        self.h = h
        self._scenes: dict[int, _SceneRec] = {}

    # ---- lifetime -------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.dem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- scenes ---------------------------------------------------------------
    def add(self, cfg: DEMConfig, particles: ParticleInput, init_bonds: bool = True,
            steps: int = 0) -> int:
        """Adds a scene; bonds are created on the next step when init_bonds
        (`initialize!`), and the scene freezes after `steps` steps (0 = never).
        Raises DemError(DEM_ERR_CAPACITY) when the arena has no room."""
        n = particles.n
        cfg_c = cfg.to_c()
        ids = np.ascontiguousarray(particles.id, dtype=np.int32)
        gid = np.ascontiguousarray(particles.gid, dtype=np.int32)
        vol, mass = _f64(particles.volume), _f64(particles.mass)
        pos, vel = _f64(particles.pos, (n, 3)), _f64(particles.vel, (n, 3))
        pin = _abi.DemParticlesIn(n, ptr(ids, C.c_int32), ptr(gid, C.c_int32),
                                  ptr(vol, C.c_double), ptr(mass, C.c_double),
                                  ptr(pos, C.c_double), ptr(vel, C.c_double))
        sid = C.c_int32()
        check(self.lib, self.lib.dem_arena_add(self.h, C.byref(cfg_c), C.byref(pin),
                                               int(bool(init_bonds)), int(steps), C.byref(sid)),
              "dem_arena_add")
        self._scenes[sid.value] = _SceneRec(cfg, particles, cfg_c)
        return sid.value

    def remove(self, scene: int) -> None:
        check(self.lib, self.lib.dem_arena_remove(self.h, int(scene)), "dem_arena_remove")
        self._scenes.pop(scene, None)

    def scenes(self) -> list[int]:
        return sorted(self._scenes)

    def info(self, scene: int) -> dict:
        si = _abi.DemSceneInfo()
        check(self.lib, self.lib.dem_arena_scene_info(self.h, int(scene), C.byref(si)),
              "dem_arena_scene_info")
        d = si.as_dict()
        d["mode"] = MODES[d["mode"]]
        return d

    def set_cell_factor(self, cell_factor: float, scene: int = -1) -> None:
        """Search-cell factor of one scene or all (-1); results do not change."""
        check(self.lib, self.lib.dem_arena_set_cell_factor(self.h, int(scene),
                                                           float(cell_factor)),
              "dem_arena_set_cell_factor")

    def launch_shape(self) -> dict:
        return get_launch_shape(self.lib, self.h)

    def set_launch_shape(self, **shape) -> None:
        set_launch_shape(self.lib, self.h, shape)

    def set_skin_factor(self, skin_factor: float, scene: int = -1) -> None:
        """Neighbour-list skin of one scene or all (-1), as a fraction of the
        largest the search allows (0 = full pair search every step); results do
        not change."""
        check(self.lib, self.lib.dem_set_skin_factor(self.h, int(scene), float(skin_factor)),
              "dem_set_skin_factor")

    # ---- the step -------------------------------------------------------------
    def step(self, nsteps: int = 1) -> None:
        """`simulate!` × nsteps for every scene in Step mode (asynchronous)."""
        check(self.lib, self.lib.dem_step(self.h, int(nsteps)), "dem_step")

    def step_timed(self, nsteps: int) -> float:
        ms = C.c_float()
        check(self.lib, self.lib.dem_step_timed(self.h, int(nsteps), C.byref(ms)),
              "dem_step_timed")
        return float(ms.value)

    def step_profiled(self) -> dict:
        """One step with CUDA events between its kernels; device milliseconds per phase."""
        from .executor import GlobalData
        ms = (C.c_float * len(GlobalData.PHASES))()
        check(self.lib, self.lib.dem_step_profiled(self.h, ms, len(ms)), "dem_step_profiled")
        return dict(zip(GlobalData.PHASES, [float(x) for x in ms]))

    def sync(self) -> None:
        check(self.lib, self.lib.dem_sync(self.h), "dem_sync")

    # ---- per-scene state ------------------------------------------------------
    def particles(self, scene: int, forces: bool = True, out: dict | None = None) -> dict:
        """A scene's particle state; `out` may hold preallocated (e.g. pinned) arrays."""
        n = self._scenes[scene].particles.n
        return read_particles(
            self.lib, lambda st: self.lib.dem_scene_get_particles(self.h, int(scene), st), n,
            forces, "dem_scene_get_particles", out)

    def contacts(self, scene: int) -> dict:
        return read_contacts(
            self.lib,
            lambda cs, cap, cnt: self.lib.dem_scene_get_contacts(self.h, int(scene), cs, cap, cnt),
            "dem_scene_get_contacts")

    def stats(self, scene: int) -> dict:
        s = _abi.DemStats()
        check(self.lib, self.lib.dem_scene_get_stats(self.h, int(scene), C.byref(s)),
              "dem_scene_get_stats")
        return s.as_dict()

    def derived(self, scene: int) -> dict:
        d = _abi.DemDerived()
        check(self.lib, self.lib.dem_scene_get_derived(self.h, int(scene), C.byref(d)),
              "dem_scene_get_derived")
        return {k: getattr(d, k) for k, _ in d._fields_}
