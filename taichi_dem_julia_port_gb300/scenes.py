"""Seeded synthetic scenes for the benchmark workloads.

Every scene is returned the way `solve` receives it: a DEMConfig plus the p4p
columns of its particles (ID, GROUP, VOLUME, MASS, position, velocity).  No
external data set is involved; sizes and value ranges follow the workload
definitions:

  bonded_cube(10, ...)  1,000-sphere bonded cube impact (10x10x10 lattice)
  bonded_cube(26, ...)  17,576-sphere bonded cube impact (26x26x26 lattice)
  granular_pour(n)      unbonded polydisperse pour, lognormal radii
  granular_bed(n)       the pour's spheres pre-compacted into touching columns
  mixed_batch(256)      256 independent scenes of 500-20,000 spheres, half
                        cubes and half pours, per-scene materials
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .config import DEMConfig


@dataclass
class ParticleInput:
    id: np.ndarray      # int32 (n,)
    gid: np.ndarray     # int32 (n,)
    volume: np.ndarray  # float64 (n,)
    mass: np.ndarray    # float64 (n,)
    pos: np.ndarray     # float64 (n, 3)
    vel: np.ndarray     # float64 (n, 3)

    @property
    def n(self) -> int:
        return int(self.id.shape[0])

    def copy(self) -> "ParticleInput":
        return ParticleInput(*(np.array(a, copy=True) for a in
                               (self.id, self.gid, self.volume, self.mass, self.pos, self.vel)))

    @classmethod
    def from_arrays(cls, radius, pos, vel, density, ids=None) -> "ParticleInput":
        radius = np.asarray(radius, dtype=np.float64)
        n = radius.shape[0]
        vol = 4.0 / 3.0 * math.pi * radius ** 3
        return cls(
            id=np.asarray(ids if ids is not None else np.arange(1, n + 1), dtype=np.int32),
            gid=np.zeros(n, dtype=np.int32),
            volume=vol,
            mass=density * vol,
            pos=np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3),
            vel=np.ascontiguousarray(vel, dtype=np.float64).reshape(n, 3),
        )


@dataclass
class Scene:
    name: str
    cfg: DEMConfig
    particles: ParticleInput
    steps: int
    bonded: bool

    @property
    def n(self) -> int:
        return self.particles.n


def bonded_cube(side: int = 10, speed: float = 10.0, steps: int = 10_000, seed: int = 1,
                radius: float = 0.01, jitter: float = 0.05, density: float = 2500.0,
                E: float = 1e8, friction: float = 0.5, dt: float = 1e-6) -> Scene:
    """Simple-cubic lattice of side^3 spheres, spacing 2·radius, radius
    jittered uniformly by ±jitter, moving at `speed` toward a rigid plane 1 mm
    below the lowest sphere surface.  Face neighbours satisfy
    |𝐤ᵢ-𝐤ⱼ| < 1.1(rᵢ+rⱼ) and bond at t = 0; diagonal neighbours do not."""
    rng = np.random.default_rng(seed)
    n = side ** 3
    spacing = 2.0 * radius
    iz, iy, ix = np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij")
    pos = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64) * spacing
    r = radius * (1.0 + rng.uniform(-jitter, jitter, size=n))
    vel = np.zeros((n, 3))
    vel[:, 2] = -speed
    p = ParticleInput.from_arrays(r, pos, vel, density)
    r_eff = np.cbrt(p.volume / (4.0 / 3.0 * math.pi))
    wall_z = float(np.min(pos[:, 2] - r_eff)) - 1e-3
    lo = pos.min(axis=0) - 0.1
    hi = pos.max(axis=0) + 0.1
    lo[2] = min(lo[2], wall_z - 0.1)
    cfg = DEMConfig(
        domain_min=lo.tolist(), domain_max=hi.tolist(), init_particles="<synthetic>",
        particle_elastic_modulus=E, particle_poisson_ratio=0.3,
        wall_normal=[0.0, 0.0, -1.0], wall_distance=-wall_z,
        bond_elastic_modulus=1e8, bond_tensile_strength=1e6, bond_shear_strength=1e6,
        pp_coefficient_friction=friction, pp_coefficient_restitution=0.9,
        max_coordinate_number=16, dt=dt, target_time=steps * dt,
        saving_interval_time=1000 * dt, gravity=[0.0, 0.0, -9.81],
    )
    return Scene(f"bonded_cube_{side}", cfg, p, steps, True)


def granular_pour(n: int = 2_000_000, box=(0.4, 0.4, 1.2), seed: int = 3, median: float = 1e-3,
                  sigma: float = 0.25, rmin: float = 0.5e-3, rmax: float = 2e-3,
                  density: float = 2500.0, E: float = 1e8, friction: float = 0.4,
                  dt: float = 2e-7, steps: int = 5_000) -> Scene:
    """Unbonded polydisperse spheres at rest in a box above a floor plane.

    Radii are lognormal (median, sigma) clipped to [rmin, rmax].  Positions
    are uniform without overlap, drawn as a random subset of the sites of a
    cubic lattice with spacing 2·rmax plus a uniform jitter that keeps every
    sphere inside its own site (equivalent to rejection sampling for this
    packing fraction, and O(n))."""
    rng = np.random.default_rng(seed)
    r = np.clip(median * np.exp(sigma * rng.standard_normal(n)), rmin, rmax)
    h = 2.0 * rmax * 1.001
    dims = np.maximum((np.asarray(box) / h).astype(np.int64), 1)
    sites = int(np.prod(dims))
    if sites < n:
        raise ValueError(f"box holds {sites} sites < {n} spheres")
    pick = rng.choice(sites, size=n, replace=False)
    pick.sort()
    ix = pick % dims[0]
    iy = (pick // dims[0]) % dims[1]
    iz = pick // (dims[0] * dims[1])
    slack = (h - 2.0 * r)[:, None] * 0.5
    jit = rng.uniform(-1.0, 1.0, size=(n, 3)) * slack
    pos = (np.stack([ix, iy, iz], axis=1) + 0.5) * h + jit
    vel = np.zeros((n, 3))
    p = ParticleInput.from_arrays(r, pos, vel, density)
    lo = np.array([-0.05, -0.05, -0.05])
    hi = np.asarray(box, dtype=np.float64) + 0.05
    cfg = DEMConfig(
        domain_min=lo.tolist(), domain_max=hi.tolist(), init_particles="<synthetic>",
        particle_elastic_modulus=E, particle_poisson_ratio=0.3,
        wall_normal=[0.0, 0.0, -1.0], wall_distance=0.0,
        bond_elastic_modulus=1e8, bond_tensile_strength=1e6, bond_shear_strength=1e6,
        pp_coefficient_friction=friction, pp_coefficient_restitution=0.9,
        max_coordinate_number=16, dt=dt, target_time=steps * dt,
        saving_interval_time=1000 * dt, gravity=[0.0, 0.0, -9.81],
    )
    return Scene(f"granular_pour_{n}", cfg, p, steps, False)


def granular_bed(n: int = 2_000_000, box=(0.4, 0.4, 1.2), seed: int = 3, median: float = 1e-3,
                 sigma: float = 0.25, rmin: float = 0.5e-3, rmax: float = 2e-3,
                 overlap: float = 1e-3, tilt: float = 0.25, density: float = 2500.0,
                 E: float = 1e8, friction: float = 0.4, dt: float = 2e-7,
                 steps: int = 5_000) -> Scene:
    """The pour's spheres (lognormal radii, median 1 mm, σ 0.25, clipped to
    [0.5, 2] mm) pre-compacted into a bed with contacts from the first step.

    Columns on a square grid over the box's floor; each column is a stack in
    which every sphere rests on the one below with an overlap of
    `overlap`·(rᵢ + rⱼ) and the lowest sphere overlaps the floor plane by the
    same fraction of its radius.  Each sphere's centre is displaced sideways
    by at most `tilt`·rmin from its column's axis, so consecutive spheres
    meet nearly head-on (a sphere is higher than the one below by at least
    0.94 of their radii's sum, so it touches no other sphere of its column),
    and the grid pitch 2·rmax·1.001 + 2·tilt·rmin keeps neighbouring columns
    apart.  Every sphere therefore starts with one or two contacts; gravity
    and the sideways offsets then let the columns lean, creating and ending
    contacts.  The box's floor must hold enough columns for the stacks to
    stay below its height."""
    rng = np.random.default_rng(seed)
    r = np.clip(median * np.exp(sigma * rng.standard_normal(n)), rmin, rmax)
    off_max = tilt * rmin
    h = 2.0 * rmax * 1.001 + 2.0 * off_max
    nx, ny = max(int(box[0] / h), 1), max(int(box[1] / h), 1)
    ncol = nx * ny
    col = np.arange(n) % ncol                     # round-robin: columns of equal count
    lvl = np.arange(n) // ncol
    off = rng.uniform(-1.0, 1.0, size=(n, 2)) * off_max
    pos = np.empty((n, 3))
    pos[:, 0] = (col % nx + 0.5) * h + off[:, 0]
    pos[:, 1] = (col // nx + 0.5) * h + off[:, 1]
    z = np.empty(n)
    first = lvl == 0
    z[first] = r[first] * (1.0 - overlap)
    for k in range(1, int(lvl.max()) + 1 if n else 0):
        cur = np.nonzero(lvl == k)[0]
        below = cur - ncol
        dxy2 = np.sum((pos[cur, :2] - pos[below, :2]) ** 2, axis=1)
        d = (r[cur] + r[below]) * (1.0 - overlap)
        z[cur] = z[below] + np.sqrt(d * d - dxy2)
    pos[:, 2] = z
    if n and z.max() + rmax > box[2]:
        raise ValueError(f"bed of {n} spheres is {z.max():.3f} m high, box {box[2]} m")
    p = ParticleInput.from_arrays(r, pos, np.zeros((n, 3)), density)
    lo = np.array([-0.05, -0.05, -0.05])
    hi = np.asarray(box, dtype=np.float64) + 0.05
    cfg = DEMConfig(
        domain_min=lo.tolist(), domain_max=hi.tolist(), init_particles="<synthetic>",
        particle_elastic_modulus=E, particle_poisson_ratio=0.3,
        wall_normal=[0.0, 0.0, -1.0], wall_distance=0.0,
        bond_elastic_modulus=1e8, bond_tensile_strength=1e6, bond_shear_strength=1e6,
        pp_coefficient_friction=friction, pp_coefficient_restitution=0.9,
        max_coordinate_number=16, dt=dt, target_time=steps * dt,
        saving_interval_time=1000 * dt, gravity=[0.0, 0.0, -9.81],
    )
    return Scene(f"granular_bed_{n}", cfg, p, steps, False)


def mixed_batch(count: int = 256, seed: int = 4, nmin: int = 500, nmax: int = 20_000,
                steps: int = 10_000) -> list[Scene]:
    """Independent scenes for batched stepping: sizes log-uniform in
    [nmin, nmax]; even entries are bonded lattice cubes (the 1,000-sphere cube
    impact's rules: radius 0.01 m ±5%, 10 m/s onto a plane 1 mm below,
    dt 1e-6 s; side = round(∛n), so n becomes side³), odd entries unbonded
    polydisperse pours (the 2,000,000-sphere pour's rules: lognormal radii,
    median 1 mm, σ 0.25, clipped to [0.5, 2] mm, at rest in a box of the same
    shape scaled to hold n spheres at the same density, dt 2e-7 s).  Each scene
    draws its particle elastic modulus from U(1e7, 1e9) Pa and its friction
    coefficient from U(0.2, 0.8)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), count))
    E = rng.uniform(1e7, 1e9, count)
    mu = rng.uniform(0.2, 0.8, count)
    out = []
    for k in range(count):
        sub = int(rng.integers(0, 2**31 - 1))
        if k % 2 == 0:
            side = max(2, int(round(sizes[k] ** (1.0 / 3.0))))
            sc = bonded_cube(side, speed=10.0, steps=steps, seed=sub, E=float(E[k]),
                             friction=float(mu[k]))
        else:
            n = int(round(sizes[k]))
            f = (n / 2_000_000) ** (1.0 / 3.0) * 1.05
            sc = granular_pour(n, box=(0.4 * f, 0.4 * f, 1.2 * f), seed=sub, E=float(E[k]),
                               friction=float(mu[k]), steps=steps)
        sc.name = f"{sc.name}#{k}"
        out.append(sc)
    return out


def c1(seed: int = 1) -> Scene:
    """1,000-sphere bonded cube, -10 m/s, 10,000 steps at dt = 1e-6 s."""
    return bonded_cube(10, speed=10.0, steps=10_000, seed=seed)


def c2(seed: int = 2) -> Scene:
    """17,576-sphere bonded cube, 20 m/s, 20,000 steps at dt = 1e-6 s."""
    return bonded_cube(26, speed=20.0, steps=20_000, seed=seed)


def c3(n: int = 2_000_000, seed: int = 3) -> Scene:
    """2,000,000-sphere unbonded pour, 5,000 steps at dt = 2e-7 s."""
    return granular_pour(n, seed=seed)
