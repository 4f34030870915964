"""Host front end mirroring DEMPort's executor (src/executor.jl).

`GlobalData` owns one scene's device state through libdem_sm100a.so (the
reference's `GlobalData`, src/executor.jl:1-29); `initialize` and `simulate`
are `initialize!` / `simulate!` (src/executor.jl:155-172); `solve` is the
reference's driver (src/executor.jl:174-394): TOML config, p4p input, step
loop, p4p/p4c output every `saving_interval_time`.

Every step runs on the GPU; there is no CPU path in this package.
"""
from __future__ import annotations

import ctypes as C
import logging
import time
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import check, ptr
from .config import DEMConfig
from .p4io import read_p4p, write_p4c, write_p4p
from .scenes import ParticleInput

log = logging.getLogger("taichi_dem_julia_port_gb300")

PRECISIONS = {"fp64": _abi.DEM_FP64, "fp32": _abi.DEM_FP32_FORCE,
              "fp32_force": _abi.DEM_FP32_FORCE}


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape is not None and a.shape != shape else a


_PARTICLE_FIELDS = {"pos": 3, "vel": 3, "omega": 3, "quat": 4, "force": 3, "moment": 3,
                    "wall_shear": 3}


def read_particles(lib, call, n: int, forces: bool, where: str, out: dict | None = None) -> dict:
    """Particle state through a dem_*get_particles call taking a DemParticleState*.

    `out` may hold preallocated C-contiguous float64 (n, k) arrays for any of
    the fields (page-locked ones are copied into directly by DMA); the fields
    it holds are the ones read, others are allocated as needed."""
    if out is None:
        out = {k: np.empty((n, c)) for k, c in _PARTICLE_FIELDS.items()
               if forces or k not in ("force", "moment")}
    else:
        for k, a in out.items():
            c = _PARTICLE_FIELDS[k]
            if (not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.shape != (n, c)
                    or not a.flags.c_contiguous or not a.flags.writeable):
                raise ValueError(f"out[{k!r}] must be a writeable C-contiguous float64 "
                                 f"array of shape ({n}, {c})")
    st = _abi.DemParticleState(n, *(out[k].ctypes.data if k in out else None for k in
                                    _PARTICLE_FIELDS))
    check(lib, call(C.byref(st)), where)
    return out


_CONTACT_VECS = ("point", "force", "torque_i", "torque_j", "shear")


def read_contacts(lib, call, where: str) -> dict:
    """Active contacts sorted by (i, j) through a dem_*get_contacts call taking
    (DemContacts*, cap, int64_t* count)."""
    cnt = C.c_int64()
    check(lib, call(None, 0, C.byref(cnt)), where)
    m = cnt.value
    out = {"i": np.empty(m, np.int32), "j": np.empty(m, np.int32),
           "bonded": np.empty(m, np.uint8)}
    for k in _CONTACT_VECS:
        out[k] = np.empty((m, 3))
    cs = _abi.DemContacts(ptr(out["i"], C.c_int32), ptr(out["j"], C.c_int32),
                          ptr(out["bonded"], C.c_uint8),
                          *(ptr(out[k], C.c_double) for k in _CONTACT_VECS))
    check(lib, call(C.byref(cs), m, C.byref(cnt)), where)
    return out


def get_launch_shape(lib, h) -> dict:
    sh = _abi.DemLaunchShape()
    check(lib, lib.dem_get_launch_shape(h, C.byref(sh)), "dem_get_launch_shape")
    return sh.as_dict()


def set_launch_shape(lib, h, shape: dict) -> None:
    """Updates the given fields of the launch shape (results do not change)."""
    cur = get_launch_shape(lib, h)
    cur.update(shape)
    sh = _abi.DemLaunchShape(**cur)
    check(lib, lib.dem_set_launch_shape(h, C.byref(sh)), "dem_set_launch_shape")


class StateBuffers:
    """Page-locked particle state arrays bound to one handle, for a host loop
    that writes the state, steps and reads it back every step.  The arrays
    (`pos`, `vel`, `omega`, `quat`, `wall_shear`, and with forces=True
    `force`, `moment`) are numpy views of page-locked memory that the
    library's kernels read and write in place; `upload()` is asynchronous
    (the arrays must stay unchanged until the next `download()` or other
    synchronising call), `download()` returns when the arrays hold the device
    state.  `step(1)` does both around a step and moves most of the state
    while the step runs (dem_step_exchange)."""

    def __init__(self, g: "GlobalData", forces: bool = False):
        self._g = g
        self._lib = g.lib
        n = g.n
        names = [k for k in _PARTICLE_FIELDS if forces or k not in ("force", "moment")]
        total = sum(n * _PARTICLE_FIELDS[k] for k in names)
        base = C.c_void_p()
        check(self._lib, self._lib.dem_host_alloc(8 * max(total, 1), C.byref(base)),
              "dem_host_alloc")
        self._base = base
        flat = np.ctypeslib.as_array(C.cast(base, C.POINTER(C.c_double)), shape=(max(total, 1),))
        self.arrays = {}
        off = 0
        for k in names:
            c = _PARTICLE_FIELDS[k]
            self.arrays[k] = flat[off:off + n * c].reshape(n, c)
            off += n * c
        addr = {k: a.ctypes.data for k, a in self.arrays.items()}
        self._in = _abi.DemParticleState(n, addr["pos"], addr["vel"], addr["omega"], addr["quat"],
                                         None, None, addr["wall_shear"])
        self._out = _abi.DemParticleState(n, *(addr.get(k) for k in _PARTICLE_FIELDS))
        self.download()

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def upload(self) -> None:
        """The arrays' state to the device (dem_set_particles_async)."""
        check(self._lib, self._lib.dem_set_particles_async(self._g.h, C.byref(self._in)),
              "dem_set_particles_async")

    def step(self, nsteps: int = 1) -> None:
        """upload(), nsteps steps and download() in one call (dem_step_exchange)."""
        check(self._lib, self._lib.dem_step_exchange(self._g.h, C.byref(self._in), int(nsteps),
                                                     C.byref(self._out)), "dem_step_exchange")

    def download(self) -> None:
        """The device state into the arrays (dem_get_particles)."""
        check(self._lib, self._lib.dem_get_particles(self._g.h, C.byref(self._out)),
              "dem_get_particles")

    def close(self) -> None:
        if getattr(self, "_base", None):
            if getattr(self._g, "h", None):
                self._lib.dem_sync(self._g.h)  # no kernel may still read the arrays
            self._lib.dem_host_free(self._base)
            self._base = None
            self.arrays = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GlobalData:
    """Device state of one scene (particles, broad phase, contacts)."""

    def __init__(self, cfg: DEMConfig, particles: ParticleInput, precision: str = "fp64",
                 lib=None, tables=None):
        self.lib = lib or _abi.load_library()
        self.cfg = cfg
        self.n = particles.n
        self._cfg_c = cfg.to_c()
        ids = np.ascontiguousarray(particles.id, dtype=np.int32)
        gid = np.ascontiguousarray(particles.gid, dtype=np.int32)
        vol = _f64(particles.volume)
        mass = _f64(particles.mass)
        pos = _f64(particles.pos, (self.n, 3))
        vel = _f64(particles.vel, (self.n, 3))
        self.ids, self.gid, self.volume, self.mass = ids, gid, vol, mass
        pin = _abi.DemParticlesIn(self.n, ptr(ids, C.c_int32), ptr(gid, C.c_int32),
                                  ptr(vol, C.c_double), ptr(mass, C.c_double),
                                  ptr(pos, C.c_double), ptr(vel, C.c_double))
        h = C.c_void_p()
        self.tables = tables
        if tables is not None:  # the scene's own material, surface and wall tables
            tc, self._tables_keep = tables.to_c()
            check(self.lib, self.lib.dem_create_tables(C.byref(self._cfg_c), C.byref(pin),
                                                       C.byref(tc), C.byref(h)),
                  "dem_create_tables")
        else:
            check(self.lib, self.lib.dem_create(C.byref(self._cfg_c), C.byref(pin), C.byref(h)),
                  "dem_create")
        self.h = h
        self.set_precision(precision)

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

    # ---- the step -------------------------------------------------------------
    def set_precision(self, precision: str) -> None:
        check(self.lib, self.lib.dem_set_precision(self.h, PRECISIONS[precision]),
              "dem_set_precision")
        self.precision = precision

    def launch_shape(self) -> dict:
        return get_launch_shape(self.lib, self.h)

    def set_launch_shape(self, **shape) -> None:
        set_launch_shape(self.lib, self.h, shape)

    def set_skin_factor(self, skin_factor: float) -> None:
        """Neighbour-list skin as a fraction of the largest the search allows
        (0 = full pair search every step); results do not change."""
        check(self.lib, self.lib.dem_set_skin_factor(self.h, 0, float(skin_factor)),
              "dem_set_skin_factor")

    def initialize(self) -> None:
        """`initialize!`: broad phase + init_bonds! (bond every cp_list pair
        closer than r₀ᵢ + r₀ⱼ)."""
        check(self.lib, self.lib.dem_init_bonds(self.h), "dem_init_bonds")

    def simulate(self, nsteps: int = 1) -> None:
        """`simulate!` × nsteps (asynchronous; errors surface at sync())."""
        check(self.lib, self.lib.dem_step(self.h, int(nsteps)), "dem_step")

    def simulate_timed(self, nsteps: int) -> float:
        """Runs nsteps and returns their device time in milliseconds."""
        ms = C.c_float()
        check(self.lib, self.lib.dem_step_timed(self.h, int(nsteps), C.byref(ms)),
              "dem_step_timed")
        return float(ms.value)

    PHASES = ("contacts", "force", "integrate")

    def simulate_profiled(self) -> dict:
        """One step with CUDA events between its kernels; device milliseconds per phase."""
        ms = (C.c_float * len(self.PHASES))()
        check(self.lib, self.lib.dem_step_profiled(self.h, ms, len(ms)), "dem_step_profiled")
        return dict(zip(self.PHASES, [float(x) for x in ms]))

    def sync(self) -> None:
        check(self.lib, self.lib.dem_sync(self.h), "dem_sync")

    # ---- state ----------------------------------------------------------------
    def particles(self, forces: bool = True, out: dict | None = None) -> dict:
        """Particle state; `out` may hold preallocated (e.g. pinned) arrays."""
        return read_particles(self.lib, lambda st: self.lib.dem_get_particles(self.h, st),
                              self.n, forces, "dem_get_particles", out)

    def state_buffers(self, forces: bool = False) -> StateBuffers:
        """Page-locked state arrays bound to this handle (see StateBuffers)."""
        return StateBuffers(self, forces)

    def set_particles(self, pos=None, vel=None, omega=None, quat=None, wall_shear=None) -> None:
        n = self.n
        # C-contiguous float64 (n, k) copies only where the input is not one already
        arrs = [None if v is None else _f64(v, (n, k))
                for v, k in ((pos, 3), (vel, 3), (omega, 3), (quat, 4), (wall_shear, 3))]
        st = _abi.DemParticleState(n, *(None if a is None else a.ctypes.data for a in arrs[:4]),
                                   None, None, None if arrs[4] is None else arrs[4].ctypes.data)
        check(self.lib, self.lib.dem_set_particles(self.h, C.byref(st)), "dem_set_particles")

    def static(self) -> dict:
        n = self.n
        out = {k: np.empty(n) for k in ("radius", "radius0", "mass", "inertia")}
        st = _abi.DemParticleStatic(n, *(ptr(out[k], C.c_double) for k in
                                         ("radius", "radius0", "mass", "inertia")))
        check(self.lib, self.lib.dem_get_static(self.h, C.byref(st)), "dem_get_static")
        return out

    def derived(self) -> dict:
        d = _abi.DemDerived()
        check(self.lib, self.lib.dem_get_derived(self.h, C.byref(d)), "dem_get_derived")
        return {k: getattr(d, k) for k, _ in d._fields_}

    def contacts(self) -> dict:
        """Active contacts sorted by (i, j) (0-based indices)."""
        return read_contacts(
            self.lib, lambda cs, cap, cnt: self.lib.dem_get_contacts(self.h, cs, cap, cnt),
            "dem_get_contacts")

    def wall_shear(self, wall: int) -> np.ndarray:
        """Shear history of wall `wall`'s contacts, (n, 3) (zero where a grain
        does not touch it); wall 0's is also particles()["wall_shear"]."""
        out = np.empty((self.n, 3))
        check(self.lib, self.lib.dem_get_wall_shear(self.h, int(wall), out.ctypes.data),
              "dem_get_wall_shear")
        return out

    def set_wall_shear(self, wall: int, shear) -> None:
        a = _f64(shear, (self.n, 3))
        check(self.lib, self.lib.dem_set_wall_shear(self.h, int(wall), a.ctypes.data),
              "dem_set_wall_shear")

    def io_contacts(self) -> np.ndarray:
        """The active contacts as p4c records (a structured array of
        _abi.IO_CONTACT_DTYPE: i, j 0-based, bonded, point, force), sorted by
        (i, j), compacted on the device (dem_get_io_contacts)."""
        cnt = C.c_int64()
        check(self.lib, self.lib.dem_get_io_contacts(self.h, None, 0, C.byref(cnt)),
              "dem_get_io_contacts")
        out = np.empty(cnt.value, dtype=_abi.IO_CONTACT_DTYPE)
        if cnt.value:
            check(self.lib, self.lib.dem_get_io_contacts(self.h, out.ctypes.data, cnt.value,
                                                         C.byref(cnt)), "dem_get_io_contacts")
        return out

    def set_contacts(self, c: dict) -> None:
        m = len(c["i"])
        arr = {"i": np.ascontiguousarray(c["i"], np.int32),
               "j": np.ascontiguousarray(c["j"], np.int32),
               "bonded": np.ascontiguousarray(c.get("bonded", np.zeros(m)), np.uint8)}
        for k in ("point", "force", "torque_i", "torque_j", "shear"):
            arr[k] = _f64(c[k], (m, 3)) if k in c else np.zeros((m, 3))
        cs = _abi.DemContacts(ptr(arr["i"], C.c_int32), ptr(arr["j"], C.c_int32),
                              ptr(arr["bonded"], C.c_uint8),
                              *(ptr(arr[k], C.c_double) for k in
                                ("point", "force", "torque_i", "torque_j", "shear")))
        check(self.lib, self.lib.dem_set_contacts(self.h, C.byref(cs), m), "dem_set_contacts")

    def stats(self) -> dict:
        s = _abi.DemStats()
        check(self.lib, self.lib.dem_get_stats(self.h, C.byref(s)), "dem_get_stats")
        return s.as_dict()

    def debug_broadphase(self, with_pairs: bool = True) -> dict:
        """The reference broad phase on the current positions: cell ijk, Morton
        code, 1-based bucket (hashcode), bucket counts, sorted particle order
        and the cp_list pairs (0-based)."""
        n = self.n
        H = self.derived()["hash_table_size"]
        out = {"cell": np.empty((n, 3), np.int32), "morton": np.empty(n, np.uint32),
               "bucket": np.empty(n, np.uint32), "bucket_count": np.empty(H, np.uint32),
               "sorted": np.empty(n, np.uint32)}
        cnt = C.c_int64()
        args = [ptr(out["cell"], C.c_int32), ptr(out["morton"], C.c_uint32),
                ptr(out["bucket"], C.c_uint32), ptr(out["bucket_count"], C.c_uint32),
                ptr(out["sorted"], C.c_uint32)]
        check(self.lib, self.lib.dem_debug_broadphase(self.h, *args, None, 0, C.byref(cnt)),
              "dem_debug_broadphase")
        if with_pairs:
            cp = np.empty((max(cnt.value, 1), 2), np.int32)
            check(self.lib, self.lib.dem_debug_broadphase(self.h, *args, ptr(cp, C.c_int32),
                                                          cnt.value, C.byref(cnt)),
                  "dem_debug_broadphase")
            out["cp"] = cp[:cnt.value]
        out["cp_count"] = cnt.value
        return out

    def debug_step_enumeration(self) -> tuple[int, int]:
        """One step with the full pair search forced; returns the candidate
        pairs its fused enumeration visited and their 64-bit checksum
        (`dem_debug_step_enumeration`)."""
        pairs, chk = C.c_int64(), C.c_uint64()
        check(self.lib, self.lib.dem_debug_step_enumeration(self.h, C.byref(pairs), C.byref(chk)),
              "dem_debug_step_enumeration")
        return int(pairs.value), int(chk.value)


def enumeration_checksum(pairs: np.ndarray) -> int:
    """Wrapping 64-bit sum of the pair mix that dem_debug_step_enumeration
    uses, over an (m, 2) array of pairs (i, j)."""
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    z = (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)
    with np.errstate(over="ignore"):
        z ^= z >> np.uint64(33)
        z *= np.uint64(0xff51afd7ed558ccd)
        z ^= z >> np.uint64(33)
        z *= np.uint64(0xc4ceb9fe1a85ec53)
        z ^= z >> np.uint64(33)
        return int(np.sum(z, dtype=np.uint64))


def initialize(g: GlobalData) -> None:
    """`initialize!(global_data, ...)` (src/executor.jl:155-160)."""
    g.initialize()


def simulate(g: GlobalData, nsteps: int = 1) -> None:
    """`simulate!(global_data, ...)` (src/executor.jl:162-172)."""
    g.simulate(nsteps)


def load_particles(p4p_path: str | Path) -> ParticleInput:
    """The grains of the first record of a p4p file, in file order
    (src/executor.jl:217-243).

    A malformed file raises ValueError naming the file and line: a first line
    that is not the TIMESTEP header, a second line without an integer
    particle count, fewer particle rows than that count, or a row with fewer
    than ten numbers (ID GROUP VOLUME MASS PX PY PZ VX VY VZ) or a value that
    does not parse."""
    path = Path(p4p_path)
    lines = path.read_text().split("\n")

    def bad(line_no: int, what: str) -> ValueError:
        return ValueError(f"{path}:{line_no}: {what}")

    if not lines or not lines[0].startswith("TIMESTEP"):
        raise bad(1, "expected the 'TIMESTEP PARTICLES' header")
    head = lines[1].split() if len(lines) > 1 else []
    try:
        n = int(head[1])
    except (IndexError, ValueError):
        raise bad(2, "expected '<timestep> <particle count>'") from None
    if n < 0:
        raise bad(2, f"negative particle count {n}")
    if len(lines) < 3 + n or any(not lines[3 + k].strip() for k in range(n)):
        have = sum(1 for ln in lines[3:3 + n] if ln.strip())
        raise bad(3 + have + 1, f"the header announces {n} particles, the file has {have} rows")
    rows = np.empty((n, 10), dtype=np.float64)
    for k in range(n):
        f = lines[3 + k].split()
        if len(f) < 10:
            raise bad(4 + k, f"expected 10 columns, found {len(f)}")
        try:
            rows[k] = [float(x) for x in f[:10]]
        except ValueError as e:
            raise bad(4 + k, str(e)) from None
    return ParticleInput(id=rows[:, 0].astype(np.int32), gid=rows[:, 1].astype(np.int32),
                         volume=rows[:, 2].copy(), mass=rows[:, 3].copy(),
                         pos=rows[:, 4:7].copy(), vel=rows[:, 7:10].copy())


def save_single(g: GlobalData, p4p, p4c, t: float) -> int:
    """`save_single` (src/utils.jl:30-78): appends one record to each file and
    returns the number of active contacts written.  The active contacts are
    compacted into p4c records on the device (dem_get_io_contacts)."""
    st = g.particles(forces=False)
    write_p4p(p4p, t, g.ids, g.gid, g.volume, g.mass, st["pos"], st["vel"])
    c = g.io_contacts()
    write_p4c(p4c, t, c["i"], c["j"], c["point"], c["force"], c["bonded"])
    return len(c)


def solve(cfg_filename: str | Path, no_bond: bool = False, save_snapshot: bool = False,
          save_information: bool = True, output_dir: str | Path = ".",
          precision: str = "fp64", particles: ParticleInput | None = None,
          cfg: DEMConfig | None = None) -> GlobalData:
    """The reference driver `solve` (src/executor.jl:174-394).

    `save_snapshot` needs an OpenGL stack (GLMakie) and is unavailable here;
    passing True raises.  `particles`/`cfg` may be given directly instead of
    reading `init_particles` relative to the config file."""
    if save_snapshot:
        raise NotImplementedError("snapshots need a graphics stack (GLMakie); unavailable")
    t0 = time.perf_counter()
    if cfg is None:
        cfg = DEMConfig.from_toml(cfg_filename)
    if particles is None:
        particles = load_particles(Path(cfg_filename).parent / cfg.init_particles)
    g = GlobalData(cfg, particles, precision=precision)
    d = g.derived()
    log.info("Setting: hash_table_size=%d cell_size=%g", d["hash_table_size"], d["cell_size"])
    if not no_bond:
        g.initialize()
    total_steps, save_per = cfg.total_steps, max(cfg.save_per_steps, 1)
    out = Path(output_dir)
    p4p = p4c = None
    if save_information:
        p4p = open(out / "output.p4p", "w")
        p4c = open(out / "output.p4c", "w")
        save_single(g, p4p, p4c, 0.0)
    step = 0
    try:
        while step < total_steps:
            t1 = time.perf_counter()
            k = save_per  # the reference runs whole save intervals (src/executor.jl:365-370)
            g.simulate(k)
            g.sync()
            step += k
            log.info("Solving... step=%d dt=%.3fs", step, time.perf_counter() - t1)
            if save_information:
                save_single(g, p4p, p4c, step * cfg.dt)
    finally:
        if p4p:
            p4p.close()
            p4c.close()
    log.info("Total time: %.3f s", time.perf_counter() - t0)
    return g
