"""Serving: a request loop with continuous batching over one device arena.

No counterpart in the reference, which runs one `solve` per process
(src/executor.jl:174-394).  Requests (a scene plus a step count) arrive over
time; each is admitted into the arena as soon as its particles, buckets and
contact reservation fit in the arena, which is sized once from an HBM budget.
Admitted scenes keep their state on the device and advance together: every
`step` launch moves all live scenes by one step, and a scene freezes on the
device when it reaches its own step count (dem_arena_add's steps_target), so a
chunk of launches never oversteps a scene.  Between chunks the loop collects
finished scenes (their result is read back and their slots freed) and admits
waiting requests, in arrival order, skipping ahead over requests that do not
fit yet.  A scene's result does not depend on what else shares the arena: it
is bit-for-bit the result of running it alone.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _abi
from .arena import Arena, buckets_for
from .scenes import Scene, bonded_cube, granular_pour

# device bytes per arena unit (the buffers dem_arena_create allocates)
SLOT_BYTES_BASE = 452          # particle SoA, broad phase, bookkeeping
SLOT_BYTES_PER_PARTNER = 12    # new-partner stash (4 B) + incoming list (8 B), per partner
SLOT_BYTES_PER_LIST_ENTRY = 4  # neighbour-list partner


def list_capacity(max_coordinate_number: int) -> int:
    """Neighbour-list partners per particle (dem_arena_create's rule)."""
    return min(max(int(max_coordinate_number), 16), 256)
CONTACT_BYTES = 345            # two contact buffers, force contributions, survival flag
BUCKET_BYTES = 8               # count + start


@dataclass
class ArenaSizing:
    max_particles: int
    max_contacts: int
    max_buckets: int
    max_scenes: int
    max_coordinate_number: int
    contacts_per_particle: int

    @property
    def bytes(self) -> int:
        return (self.max_particles * (SLOT_BYTES_BASE + SLOT_BYTES_PER_PARTNER *
                                      self.max_coordinate_number
                                      + SLOT_BYTES_PER_LIST_ENTRY *
                                      list_capacity(self.max_coordinate_number))
                + self.max_contacts * CONTACT_BYTES + self.max_buckets * BUCKET_BYTES)

    @classmethod
    def from_budget(cls, hbm_bytes: float, max_scenes: int = 1024, max_coordinate_number: int = 16,
                    contacts_per_particle: int = 8) -> "ArenaSizing":
        """Largest arena within `hbm_bytes`: contact capacity reserved at
        `contacts_per_particle` per slot and two bucket entries per slot plus
        1,024 per scene record."""
        per_slot = (SLOT_BYTES_BASE + SLOT_BYTES_PER_PARTNER * max_coordinate_number
                    + SLOT_BYTES_PER_LIST_ENTRY * list_capacity(max_coordinate_number)
                    + contacts_per_particle * CONTACT_BYTES + 2 * BUCKET_BYTES)
        fixed = 1024 * max_scenes * BUCKET_BYTES
        n = int(max(hbm_bytes - fixed, 0) // per_slot)
        n = min(n, 0x3FFFFFFF)
        return cls(n, min(n * contacts_per_particle, 0x7FFFFFFF), 2 * n + 1024 * max_scenes,
                   max_scenes, max_coordinate_number, contacts_per_particle)


@dataclass
class Request:
    rid: int
    arrival_s: float
    steps: int
    make_scene: Callable[[], Scene]
    n_hint: int = 0   # particle count (for admission before the scene is built)
    kind: str = ""
    _scene: Scene | None = field(default=None, repr=False)

    def scene(self) -> Scene:
        if self._scene is None:
            self._scene = self.make_scene()
        return self._scene


@dataclass
class Result:
    rid: int
    n: int
    steps: int
    arrival_s: float
    admitted_s: float
    completed_s: float
    stats: dict
    state: dict | None = None

    @property
    def latency_s(self) -> float:
        return self.completed_s - self.arrival_s


@dataclass
class _Live:
    req: Request
    scene: Scene
    sid: int
    admitted_s: float
    reserve: int


@dataclass
class ServeReport:
    results: list
    makespan_s: float
    particle_steps: int
    launches: int
    admissions_deferred: int = 0
    tune: dict | None = None
    extra: dict = field(default_factory=dict)

    @property
    def throughput(self) -> float:
        return self.particle_steps / self.makespan_s if self.makespan_s > 0 else 0.0

    def latency_percentiles(self, qs=(50, 99)) -> dict:
        lat = np.array([r.latency_s for r in self.results])
        return {f"p{q}": float(np.percentile(lat, q)) for q in qs} if lat.size else {}


# launch-shape update of a served arena (see Server)
SERVED_SHAPE = {"force_blocks_per_sm": 4}


class Server:
    """Continuous-batching loop over one arena sized from an HBM budget."""

    def __init__(self, sizing: ArenaSizing, precision: str = "fp32", chunk_steps: int = 200,
                 cell_factor: float = 0.0, keep_state: bool = True, lib=None,
                 policy: str = "fifo", max_active: int = 0, min_chunk: int = 1,
                 build_ahead: int = 4, launch_shape: dict | None = None):
        """policy "fifo": waiting requests are admitted in arrival order as
        soon as they fit.  policy "sjf": the waiting request with the least
        work (particles x steps) first, and only while the live scenes hold
        fewer than `max_active` particles (a request is always admitted into
        an empty arena): small requests then share their launches with fewer
        particles and finish sooner, at some cost in throughput.

        A chunk runs `chunk_steps` steps, or fewer when a live scene needs
        fewer to finish (so that its slots are freed promptly), but at least
        `min_chunk` (scenes freeze on the device at their step count, so a
        longer chunk never oversteps one).  While a chunk runs, the scenes of
        up to `build_ahead` waiting requests are built on the host.

        `launch_shape` updates the arena's launch shape (results do not
        change).  By default the FP32 force kernel gets the register budget
        for four blocks per SM: served scenes of up to 1e6 spheres put most
        particles in large scenes, where it shortened the device time of the
        100-request stream by 4-10 % (the many-small-scene batch prefers the
        compiler's choice, which the arena keeps otherwise)."""
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        self.policy = policy
        self.max_active = int(max_active) if max_active else 0
        self.sizing = sizing
        self.arena = Arena(sizing.max_particles, max_scenes=sizing.max_scenes,
                           max_contacts=sizing.max_contacts, max_buckets=sizing.max_buckets,
                           max_coordinate_number=sizing.max_coordinate_number,
                           precision=precision, cell_factor=cell_factor, lib=lib)
        self.arena.set_launch_shape(**(SERVED_SHAPE if launch_shape is None else launch_shape))
        self.chunk_steps = int(chunk_steps)
        self.min_chunk = max(1, min(int(min_chunk), self.chunk_steps))
        self.build_ahead = max(0, int(build_ahead))
        self.keep_state = keep_state
        self._reserved = 0

    def close(self) -> None:
        self.arena.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _try_admit(self, req: Request, now: float, live: dict) -> bool:
        if req.n_hint and (self._reserved + req.n_hint * self.sizing.contacts_per_particle
                           > self.sizing.max_contacts):
            return False
        sc = req.scene()
        reserve = sc.n * self.sizing.contacts_per_particle
        if self._reserved + reserve > self.sizing.max_contacts:
            return False
        try:
            sid = self.arena.add(sc.cfg, sc.particles, init_bonds=sc.bonded, steps=req.steps)
        except _abi.DemError as e:
            if e.code == _abi.DEM_ERR_CAPACITY:
                return False
            raise
        self._reserved += reserve
        live[sid] = _Live(req, sc, sid, now, reserve)
        return True

    def run(self, requests: list[Request], realtime: bool = True,
            on_result: Callable[[Result], None] | None = None) -> ServeReport:
        """Serves `requests` (arrival times relative to the start).  With
        realtime=False every request is treated as already arrived."""
        pending = sorted(requests, key=lambda r: r.arrival_s)
        queue: list[Request] = []
        live: dict[int, _Live] = {}
        results: list[Result] = []
        launches = 0
        deferred = 0
        work = 0
        # where the wall-clock time goes: admission (scene build, upload),
        # waiting for the device, collection of finished scenes
        spent = {"admit_s": 0.0, "device_wait_s": 0.0, "collect_s": 0.0, "chunks": 0}
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: math.inf)
        while pending or queue or live:
            now = clock()
            while pending and pending[0].arrival_s <= now:
                queue.append(pending.pop(0))
            # admission in arrival order (fifo) or by least work (sjf), skipping
            # over requests that do not fit yet
            if self.policy == "sjf":
                queue.sort(key=lambda r: (r.n_hint or 1) * r.steps)
            active = sum(lv.scene.n for lv in live.values())
            ta = time.perf_counter()
            still = []
            for req in queue:
                over = (self.policy == "sjf" and self.max_active and live
                        and active + (req.n_hint or 0) > self.max_active)
                if over or not self._try_admit(req, time.perf_counter() - t0, live):
                    still.append(req)
                    deferred += 1
                else:
                    active += req.scene().n
            queue = still
            spent["admit_s"] += time.perf_counter() - ta
            if not live:
                if queue:
                    raise RuntimeError(f"request {queue[0].rid} can never fit the arena")
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival_s - clock(), 0.05)))
                continue
            # one chunk: at most the fewest steps any live scene still needs,
            # so a finishing scene frees its slots promptly
            need = min(lv.req.steps - self.arena.info(sid)["steps_done"]
                       for sid, lv in live.items())
            k = max(self.min_chunk, min(self.chunk_steps, need))
            self.arena.step(k)  # asynchronous
            launches += k
            # host work that overlaps the chunk: arrivals join the queue and the
            # next requests' scenes are built
            now = clock()
            while pending and pending[0].arrival_s <= now:
                queue.append(pending.pop(0))
            if self.policy == "sjf":
                queue.sort(key=lambda r: (r.n_hint or 1) * r.steps)
            for req in queue[:self.build_ahead]:
                req.scene()
            tw = time.perf_counter()
            self.arena.sync()
            spent["device_wait_s"] += time.perf_counter() - tw
            spent["chunks"] += 1
            done_t = time.perf_counter() - t0
            tc = time.perf_counter()
            for sid in list(live):
                lv = live[sid]
                info = self.arena.info(sid)
                if info["mode"] != "frozen":
                    continue
                st = self.arena.stats(sid)
                state = self.arena.particles(sid, forces=False) if self.keep_state else None
                res = Result(lv.req.rid, lv.scene.n, lv.req.steps, lv.req.arrival_s,
                             lv.admitted_s, done_t, st, state)
                work += lv.scene.n * lv.req.steps
                results.append(res)
                if on_result:
                    on_result(res)
                self.arena.remove(sid)
                self._reserved -= lv.reserve
                lv.req._scene = None  # host copy no longer needed
                del live[sid]
            spent["collect_s"] += time.perf_counter() - tc
        makespan = time.perf_counter() - t0
        results.sort(key=lambda r: r.rid)
        return ServeReport(results, makespan, work, launches, deferred, extra=spent)


def log_uniform_int(rng, lo: float, hi: float) -> int:
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def poisson_requests(count: int = 200, rate: float = 50.0, seed: int = 5, nmin: int = 1_000,
                     nmax: int = 1_000_000, smin: int = 1_000, smax: int = 50_000) -> list[Request]:
    """The served workload: Poisson arrivals (mean `rate` per second), sizes
    log-uniform in [nmin, nmax] spheres, step counts uniform in [smin, smax],
    alternately bonded lattice cubes (side = round(∛n)) and unbonded pours
    (the generators of the batched workload), per-request material
    E ~ U(1e7, 1e9) Pa and friction ~ U(0.2, 0.8).  Scenes are built when
    admitted."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        n = log_uniform_int(rng, nmin, nmax)
        steps = int(rng.integers(smin, smax + 1))
        E, mu = float(rng.uniform(1e7, 1e9)), float(rng.uniform(0.2, 0.8))
        sub = int(rng.integers(0, 2**31 - 1))
        if k % 2 == 0:
            side = max(2, int(round(n ** (1.0 / 3.0))))
            make = (lambda side=side, sub=sub, E=E, mu=mu, steps=steps:
                    bonded_cube(side, speed=10.0, steps=steps, seed=sub, E=E, friction=mu))
            out.append(Request(k, t, steps, make, side ** 3, "cube"))
        else:
            f = (n / 2_000_000) ** (1.0 / 3.0) * 1.05
            make = (lambda n=n, f=f, sub=sub, E=E, mu=mu, steps=steps:
                    granular_pour(n, box=(0.4 * f, 0.4 * f, 1.2 * f), seed=sub, E=E,
                                  friction=mu, steps=steps))
            out.append(Request(k, t, steps, make, n, "pour"))
    return out


def sequential_plain(requests: list[Request], steps_per_probe: int = 20,
                     precision: str = "fp64", lib=None) -> dict:
    """The plain path scene by scene: each request alone on a single-scene
    handle, one after another in arrival order.  Each scene's step time is
    measured over `steps_per_probe` steps (after 3 untimed ones) and scaled to
    its step count; completion times follow from serving the requests in
    order, each starting at max(arrival, previous completion)."""
    from .executor import GlobalData

    busy = 0.0
    lat = []
    work = 0
    total = 0.0
    for req in sorted(requests, key=lambda r: r.arrival_s):
        sc = req.make_scene()  # built afresh: served requests drop their host copy
        g = GlobalData(sc.cfg, sc.particles, precision=precision, lib=lib)
        if sc.bonded:
            g.initialize()
        g.simulate(3)
        ms = g.simulate_timed(steps_per_probe) / steps_per_probe
        g.close()
        t = ms * 1e-3 * req.steps
        start = max(busy, req.arrival_s)
        busy = start + t
        lat.append(busy - req.arrival_s)
        work += sc.n * req.steps
        total += t
    lat = np.array(lat)
    return {"particle_steps_per_s": work / busy if busy > 0 else 0.0, "makespan_s": busy,
            "busy_s": total, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "particle_steps": work}


__all__ = ["ArenaSizing", "Request", "Result", "Server", "ServeReport", "poisson_requests",
           "sequential_plain", "buckets_for"]
