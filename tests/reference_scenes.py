"""The reference repository's own example scenes (cfg/1.toml + carom.p4p,
cfg/2.toml + cube_911_particles_impact.p4p), packed by
tests/golden/make_reference_scenes.py."""
from __future__ import annotations

import os
import tomllib
from pathlib import Path

import numpy as np

from taichi_dem_julia_port_gb300.config import DEMConfig
from taichi_dem_julia_port_gb300.scenes import ParticleInput

FIXTURE = Path(__file__).resolve().parent / "golden" / "reference_scenes.npz"
NAMES = ("carom", "cube_911")


def reference_checkout() -> Path | None:
    """The reference repository's checkout when one is available: the directory
    named by $DEM_REFERENCE, else a directory `reference` beside this
    repository.  None when neither exists (tests then check only the fixtures)."""
    env = os.environ.get("DEM_REFERENCE")
    cands = [Path(env)] if env else [Path(__file__).resolve().parents[2] / "reference"]
    for c in cands:
        if (c / "src" / "kernels.jl").exists():
            return c
    return None


def load(name: str):
    z = np.load(FIXTURE)
    cfg = DEMConfig.from_dict(tomllib.loads(str(z[f"{name}/cfg_toml"])))
    p = ParticleInput(id=z[f"{name}/id"], gid=z[f"{name}/gid"], volume=z[f"{name}/volume"],
                      mass=z[f"{name}/mass"], pos=z[f"{name}/pos"], vel=z[f"{name}/vel"])
    return cfg, p, str(z[f"{name}/source"])
