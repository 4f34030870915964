"""TEST INFRASTRUCTURE ONLY — Python view of the CPU oracle (liboracle.so).

The oracle is the FP64 CPU restatement of the reference DEM step
(oracle/dem_oracle.cpp).  Tests, the smoke check and bench.py's CPU-baseline
legs use it as the checker / CPU baseline; the product package never imports
it.  Its methods mirror taichi_dem_julia_port_gb300.GlobalData so that parity
tests read the same on both sides.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from taichi_dem_julia_port_gb300 import _abi
from taichi_dem_julia_port_gb300._abi import ptr

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        from oracle.build import build
        build()
    lib = C.CDLL(str(LIB))
    H = C.c_void_p
    sig = {
        "oracle_create": (H, [C.POINTER(_abi.DemConfigC), C.POINTER(_abi.DemParticlesIn), C.c_int]),
        "oracle_destroy": (None, [H]),
        "oracle_create_tables": (H, [C.POINTER(_abi.DemConfigC), C.POINTER(_abi.DemParticlesIn),
                                     C.POINTER(_abi.DemTables), C.c_int]),
        "oracle_get_wall_shear": (C.c_int, [H, C.c_int, C.POINTER(C.c_double)]),
        "oracle_set_wall_shear": (C.c_int, [H, C.c_int, C.POINTER(C.c_double)]),
        "oracle_set_threads": (None, [H, C.c_int]),
        "oracle_max_threads": (C.c_int, []),
        "oracle_init_bonds": (C.c_int, [H]),
        "oracle_step": (C.c_int, [H, C.c_int64]),
        "oracle_get_derived": (C.c_int, [H, C.POINTER(_abi.DemDerived)]),
        "oracle_get_static": (C.c_int, [H, C.POINTER(_abi.DemParticleStatic)]),
        "oracle_get_particles": (C.c_int, [H, C.POINTER(_abi.DemParticleState)]),
        "oracle_set_particles": (C.c_int, [H, C.POINTER(_abi.DemParticleState)]),
        "oracle_get_contacts": (C.c_int, [H, C.POINTER(_abi.DemContacts), C.c_int64,
                                          C.POINTER(C.c_int64)]),
        "oracle_set_contacts": (C.c_int, [H, C.POINTER(_abi.DemContacts), C.c_int64]),
        "oracle_get_stats": (C.c_int, [H, C.POINTER(_abi.DemStats)]),
        "oracle_broadphase": (C.c_int, [H, C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.c_int64,
                                        C.POINTER(C.c_int64)]),
        "oracle_morton1": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32]),
        "oracle_quat_to_matrix": (None, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "oracle_frame_to_x": (None, [C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double)]),
        "oracle_jl_norm": (C.c_double, [C.POINTER(C.c_double)]),
        "oracle_eval_pair": (C.c_int, [C.POINTER(_abi.DemConfigC), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                       C.POINTER(C.c_double)]),
        "oracle_eval_wall": (C.c_int, [C.POINTER(_abi.DemConfigC), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "oracle_eval_update": (C.c_int, [C.POINTER(_abi.DemConfigC), C.c_int64,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _chk(rc: int, where: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{where}: oracle error {rc}")


class OracleScene:
    """One scene on the CPU oracle; `threads` = 1 is the serial mode."""

    def __init__(self, cfg, particles, threads: int = 1, tables=None):
        self.lib = load()
        self.n = particles.n
        self._cfg = cfg.to_c()
        self._keep = [np.ascontiguousarray(particles.id, np.int32),
                      np.ascontiguousarray(particles.gid, np.int32),
                      np.ascontiguousarray(particles.volume, np.float64),
                      np.ascontiguousarray(particles.mass, np.float64),
                      np.ascontiguousarray(particles.pos, np.float64).reshape(-1, 3),
                      np.ascontiguousarray(particles.vel, np.float64).reshape(-1, 3)]
        ids, gid, vol, mass, pos, vel = self._keep
        pin = _abi.DemParticlesIn(self.n, ptr(ids, C.c_int32), ptr(gid, C.c_int32),
                                  ptr(vol, C.c_double), ptr(mass, C.c_double),
                                  ptr(pos, C.c_double), ptr(vel, C.c_double))
        if tables is not None:
            tc, self._tables_keep = tables.to_c()
            self.h = self.lib.oracle_create_tables(C.byref(self._cfg), C.byref(pin), C.byref(tc),
                                                   int(threads))
        else:
            self.h = self.lib.oracle_create(C.byref(self._cfg), C.byref(pin), int(threads))
        if not self.h:
            raise RuntimeError("oracle_create failed")

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, t: int) -> None:
        self.lib.oracle_set_threads(self.h, int(t))

    def initialize(self) -> None:
        _chk(self.lib.oracle_init_bonds(self.h), "oracle_init_bonds")

    def simulate(self, nsteps: int = 1) -> None:
        _chk(self.lib.oracle_step(self.h, int(nsteps)), "oracle_step")

    def derived(self) -> dict:
        d = _abi.DemDerived()
        self.lib.oracle_get_derived(self.h, C.byref(d))
        return {k: getattr(d, k) for k, _ in d._fields_}

    def static(self) -> dict:
        n = self.n
        out = {k: np.empty(n) for k in ("radius", "radius0", "mass", "inertia")}
        st = _abi.DemParticleStatic(n, *(ptr(out[k], C.c_double) for k in
                                         ("radius", "radius0", "mass", "inertia")))
        self.lib.oracle_get_static(self.h, C.byref(st))
        return out

    def particles(self, forces: bool = True) -> dict:
        n = self.n
        out = {k: np.empty((n, 3)) for k in ("pos", "vel", "omega", "wall_shear", "force",
                                              "moment")}
        out["quat"] = np.empty((n, 4))
        st = _abi.DemParticleState(n, *(out[k].ctypes.data for k in
                                        ("pos", "vel", "omega", "quat", "force", "moment",
                                         "wall_shear")))
        self.lib.oracle_get_particles(self.h, C.byref(st))
        return out

    def set_particles(self, pos=None, vel=None, omega=None, quat=None, wall_shear=None):
        n = self.n
        def f(a, k):
            return None if a is None else np.ascontiguousarray(a, np.float64).reshape(n, k)
        arrs = [f(pos, 3), f(vel, 3), f(omega, 3), f(quat, 4), None, None, f(wall_shear, 3)]
        st = _abi.DemParticleState(n, *(None if a is None else a.ctypes.data for a in arrs))
        self.lib.oracle_set_particles(self.h, C.byref(st))

    def wall_shear(self, wall: int) -> np.ndarray:
        out = np.empty((self.n, 3))
        _chk(self.lib.oracle_get_wall_shear(self.h, int(wall), ptr(out, C.c_double)),
             "oracle_get_wall_shear")
        return out

    def set_wall_shear(self, wall: int, shear) -> None:
        a = np.ascontiguousarray(shear, np.float64).reshape(self.n, 3)
        _chk(self.lib.oracle_set_wall_shear(self.h, int(wall), ptr(a, C.c_double)),
             "oracle_set_wall_shear")

    def contacts(self) -> dict:
        cnt = C.c_int64()
        self.lib.oracle_get_contacts(self.h, None, 0, C.byref(cnt))
        m = cnt.value
        out = {"i": np.empty(m, np.int32), "j": np.empty(m, np.int32),
               "bonded": np.empty(m, np.uint8)}
        for k in ("point", "force", "torque_i", "torque_j", "shear"):
            out[k] = np.empty((m, 3))
        cs = _abi.DemContacts(ptr(out["i"], C.c_int32), ptr(out["j"], C.c_int32),
                              ptr(out["bonded"], C.c_uint8),
                              *(ptr(out[k], C.c_double) for k in
                                ("point", "force", "torque_i", "torque_j", "shear")))
        _chk(self.lib.oracle_get_contacts(self.h, C.byref(cs), m, C.byref(cnt)),
             "oracle_get_contacts")
        return out

    def set_contacts(self, c: dict) -> None:
        m = len(c["i"])
        arr = {"i": np.ascontiguousarray(c["i"], np.int32),
               "j": np.ascontiguousarray(c["j"], np.int32),
               "bonded": np.ascontiguousarray(c.get("bonded", np.zeros(m)), np.uint8)}
        for k in ("point", "force", "torque_i", "torque_j", "shear"):
            arr[k] = np.ascontiguousarray(c[k], np.float64).reshape(m, 3) if k in c else np.zeros((m, 3))
        cs = _abi.DemContacts(ptr(arr["i"], C.c_int32), ptr(arr["j"], C.c_int32),
                              ptr(arr["bonded"], C.c_uint8),
                              *(ptr(arr[k], C.c_double) for k in
                                ("point", "force", "torque_i", "torque_j", "shear")))
        _chk(self.lib.oracle_set_contacts(self.h, C.byref(cs), m), "oracle_set_contacts")

    def stats(self) -> dict:
        s = _abi.DemStats()
        self.lib.oracle_get_stats(self.h, C.byref(s))
        return s.as_dict()

    def debug_broadphase(self, with_pairs: bool = True) -> dict:
        n = self.n
        H = self.derived()["hash_table_size"]
        out = {"cell": np.empty((n, 3), np.int32), "morton": np.empty(n, np.uint32),
               "bucket": np.empty(n, np.uint32), "bucket_count": np.empty(H, np.uint32),
               "sorted": np.empty(n, np.uint32)}
        cnt = C.c_int64()
        args = [ptr(out["cell"], C.c_int32), ptr(out["morton"], C.c_uint32),
                ptr(out["bucket"], C.c_uint32), ptr(out["bucket_count"], C.c_uint32),
                ptr(out["sorted"], C.c_uint32)]
        self.lib.oracle_broadphase(self.h, *args, None, 0, C.byref(cnt))
        if with_pairs:
            cp = np.empty((max(cnt.value, 1), 2), np.int32)
            _chk(self.lib.oracle_broadphase(self.h, *args, ptr(cp, C.c_int32), cnt.value,
                                            C.byref(cnt)), "oracle_broadphase")
            out["cp"] = cp[:cnt.value]
        out["cp_count"] = cnt.value
        return out


def morton1(x: int, y: int, z: int) -> int:
    return int(load().oracle_morton1(x, y, z))


def quat_to_matrix(q) -> np.ndarray:
    q = np.ascontiguousarray(q, np.float64)
    R = np.empty(9)
    load().oracle_quat_to_matrix(ptr(q, C.c_double), ptr(R, C.c_double))
    return R.reshape(3, 3)


def frame_to_x(a, tol: float = 1e-12) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float64)
    R = np.empty(9)
    load().oracle_frame_to_x(ptr(a, C.c_double), tol, ptr(R, C.c_double))
    return R.reshape(3, 3)


def jl_norm(a) -> float:
    a = np.ascontiguousarray(a, np.float64)
    return float(load().oracle_jl_norm(ptr(a, C.c_double)))


def _d(a) -> np.ndarray:
    return np.ascontiguousarray(a, np.float64)


def grain_record(g: dict) -> np.ndarray:
    """16-double grain record of the oracle_eval_* helpers: r, m, k, v, w, q, I."""
    return _d([g["r"], g["m"], *g["k"], *g["v"], *g["w"], *g["q"], g["I"]])


def eval_pair(cfg, gi: dict, gj: dict, state, bonded: bool) -> dict:
    """One contact through the oracle's resolve_one (grain 0 = i, grain 1 = j)."""
    c = cfg.to_c()
    a, b, st = grain_record(gi), grain_record(gj), _d(state)
    out = np.empty(28)
    _chk(load().oracle_eval_pair(C.byref(c), ptr(a, C.c_double), ptr(b, C.c_double),
                                 ptr(st, C.c_double), int(bool(bonded)), ptr(out, C.c_double)),
         "oracle_eval_pair")
    v = out[1:].reshape(9, 3)
    return {"kind": int(out[0]), "fi": v[0], "fj": v[1], "mi": v[2], "mj": v[3], "k": v[4],
            "F": v[5], "ti": v[6], "tj": v[7], "s": v[8]}


def eval_wall(cfg, g: dict, s_in) -> dict:
    """One particle against the configured wall through the oracle's resolve_wall."""
    c = cfg.to_c()
    a, s = grain_record(g), _d(s_in)
    out = np.empty(16)
    _chk(load().oracle_eval_wall(C.byref(c), ptr(a, C.c_double), ptr(s, C.c_double),
                                 ptr(out, C.c_double)), "oracle_eval_wall")
    v = out[1:].reshape(5, 3)
    return {"touch": int(out[0]), "f": v[0], "m": v[1], "k": v[2], "F": v[3], "s": v[4]}


def eval_update(cfg, grains: list, F, T) -> dict:
    """apply_body_force! + update! for the given grains and contact sums."""
    c = cfg.to_c()
    n = len(grains)
    g = _d(np.concatenate([grain_record(x) for x in grains]))
    f, t = _d(F).reshape(-1), _d(T).reshape(-1)
    out = np.empty((n, 19))
    _chk(load().oracle_eval_update(C.byref(c), n, ptr(g, C.c_double), ptr(f, C.c_double),
                                   ptr(t, C.c_double), ptr(out, C.c_double)), "oracle_eval_update")
    return {"k": out[:, 0:3], "v": out[:, 3:6], "q": out[:, 6:10], "w": out[:, 10:13],
            "F": out[:, 13:16], "T": out[:, 16:19]}


def host_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
