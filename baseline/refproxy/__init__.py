"""Reference-structured GPU proxy of the DEMPort step (a labelled stand-in).

The reference's own GPU path (Julia + CUDA.jl) cannot run on GB300 here, so
`refproxy.cu` restates it in plain CUDA C++ with the reference's structure:
AoS 272-byte grains and 136-byte contacts, nextpow2(n)^2-bit BitTables, the
same kernel decomposition (about 25 launches per step) and the three
device->host reads per step of src/executor.jl:31-172.  It is timed beside
the library on the same GPU; it is not part of the library and shares no code
with it.  Its results are checked against the CPU oracle by the tests.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
LIB_PATH = HERE / "librefproxy.so"
SRC = HERE / "refproxy.cu"
MAX_PARTICLES = 1 << 16   # the BitTables' limit (nextpow2(n)^2 bits each)


def build(force: bool = False) -> Path:
    """Compile librefproxy.so for sm_103a (nvcc), if stale."""
    hdr = ROOT / "include" / "dem_gb300.h"
    if (not force and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime > max(SRC.stat().st_mtime, hdr.stat().st_mtime)):
        return LIB_PATH
    from taichi_dem_julia_port_gb300.build import nvcc_path
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc_path(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
           "-std=c++17", "-Xcompiler", "-fPIC", f"-I{ROOT / 'include'}", "-shared",
           "-cudart", "static", str(SRC), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_LIB = None


def load():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH.name} is not built: call baseline.refproxy.build()")
        lib = C.CDLL(str(LIB_PATH))
        vp = C.c_void_p
        for name, args in {
            "rp_create": [vp, vp, C.POINTER(vp)],
            "rp_init_bonds": [vp],
            "rp_step": [vp, C.c_int64],
            "rp_step_timed": [vp, C.c_int64, C.POINTER(C.c_float)],
            "rp_get_state": [vp, vp, vp],
            "rp_get_contacts": [vp, vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)],
            "rp_destroy": [vp],
        }.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _LIB = lib
    return _LIB


def _check(rc: int, where: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{where} failed with status {rc}")


class RefProxy:
    """One scene on the reference-structured proxy (`solve`'s set-up)."""

    def __init__(self, cfg, particles):
        from taichi_dem_julia_port_gb300 import _abi
        if particles.n > MAX_PARTICLES:
            raise ValueError(f"the proxy's BitTables take at most {MAX_PARTICLES} particles")
        self.lib = load()
        self.n = particles.n
        self._cfg = cfg.to_c()
        keep = [np.ascontiguousarray(particles.id, np.int32),
                np.ascontiguousarray(particles.gid, np.int32),
                np.ascontiguousarray(particles.volume, np.float64),
                np.ascontiguousarray(particles.mass, np.float64),
                np.ascontiguousarray(particles.pos, np.float64).reshape(self.n, 3),
                np.ascontiguousarray(particles.vel, np.float64).reshape(self.n, 3)]
        pin = _abi.DemParticlesIn(self.n, *(a.ctypes.data_as(C.POINTER(
            C.c_int32 if a.dtype == np.int32 else C.c_double)) for a in keep))
        h = C.c_void_p()
        _check(self.lib.rp_create(C.byref(self._cfg), C.byref(pin), C.byref(h)), "rp_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.rp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self) -> None:
        _check(self.lib.rp_init_bonds(self.h), "rp_init_bonds")

    def simulate(self, nsteps: int = 1) -> None:
        _check(self.lib.rp_step(self.h, int(nsteps)), "rp_step")

    def simulate_timed(self, nsteps: int) -> float:
        """Milliseconds for `nsteps` steps (CUDA events on the proxy's stream)."""
        ms = C.c_float()
        _check(self.lib.rp_step_timed(self.h, int(nsteps), C.byref(ms)), "rp_step_timed")
        return float(ms.value)

    def particles(self) -> dict:
        pos, vel = np.empty((self.n, 3)), np.empty((self.n, 3))
        _check(self.lib.rp_get_state(self.h, pos.ctypes.data, vel.ctypes.data), "rp_get_state")
        return {"pos": pos, "vel": vel}

    def contacts(self) -> dict:
        cnt = C.c_int64()
        _check(self.lib.rp_get_contacts(self.h, None, None, None, 0, C.byref(cnt)),
               "rp_get_contacts")
        m = cnt.value
        out = {"i": np.empty(m, np.int32), "j": np.empty(m, np.int32),
               "bonded": np.empty(m, np.uint8)}
        _check(self.lib.rp_get_contacts(self.h, out["i"].ctypes.data, out["j"].ctypes.data,
                                        out["bonded"].ctypes.data, m, C.byref(cnt)),
               "rp_get_contacts")
        return out
