"""Packs the reference repository's own example scenes into a test fixture
(run in a checkout where the reference repository is available; the GPU machine
never runs this script).

The reference ships its example inputs as TOML configs and p4p particle files
(cfg/1.toml with Resources/carom.p4p: a 16-ball carom break; cfg/2.toml with
Resources/cube_911_particles_impact.p4p: a 911-sphere bonded cube hitting a
wall at 25 m/s).  They are read here with this package's own readers
(`DEMConfig.from_toml`, `load_particles`, the code paths `solve` uses) and
stored as arrays plus the config's TOML text, so that the GPU parity tests
can run the reference's scenes without the reference repository.

    python tests/golden/make_reference_scenes.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

SCENES = {"carom": "cfg/1.toml", "cube_911": "cfg/2.toml"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $DEM_REFERENCE, else ../reference)")
    ap.add_argument("--out", default=str(HERE / "reference_scenes.npz"))
    args = ap.parse_args()
    if args.reference is None:
        from tests.reference_scenes import reference_checkout
        found = reference_checkout()
        if found is None:
            ap.error("no reference checkout: give --reference PATH or set DEM_REFERENCE")
        args.reference = str(found)
    from taichi_dem_julia_port_gb300 import DEMConfig, load_particles

    ref = Path(args.reference)
    arrays = {}
    for name, cfg_rel in SCENES.items():
        cfg_path = ref / cfg_rel
        cfg = DEMConfig.from_toml(cfg_path)
        p = load_particles((cfg_path.parent / cfg.init_particles).resolve())
        arrays[f"{name}/cfg_toml"] = np.array(cfg.to_toml())
        arrays[f"{name}/source"] = np.array(f"{cfg_rel} + {cfg.init_particles}")
        for k in ("id", "gid", "volume", "mass", "pos", "vel"):
            arrays[f"{name}/{k}"] = np.asarray(getattr(p, k))
    np.savez_compressed(args.out, **arrays)
    print(args.out)


if __name__ == "__main__":
    main()
