"""GPU parity on the reference repository's own example scenes (cfg/2.toml:
the 911-sphere bonded cube hitting a wall at 25 m/s; cfg/1.toml: the 16-ball
carom break), against the CPU oracle over their impacts: contact and bond
sets equal, positions and velocities within the short-horizon tolerance."""
import numpy as np
import pytest

from oracle.oracle import OracleScene
from taichi_dem_julia_port_gb300 import GlobalData
from tests import reference_scenes as rs
from tests.conftest import assert_rows_close
from tests.test_gpu_parity import bonded_set, pair_set

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def compare(g, o, what):
    cg, co = g.contacts(), o.contacts()
    assert pair_set(cg) == pair_set(co), f"{what}: contact sets differ"
    assert bonded_set(cg) == bonded_set(co), f"{what}: bond sets differ"
    pg, po = g.particles(), o.particles()
    assert_rows_close(pg["pos"], po["pos"], RTOL, f"{what} pos")
    assert_rows_close(pg["vel"], po["vel"], RTOL, f"{what} vel", atol_frac=RTOL)
    return cg, pg


def run_pair(name, chunks, lead=0):
    """Both paths from the scene's start; with `lead`, the GPU runs that many
    steps alone first and its state (particles and contacts) is copied into
    the oracle, which then steps alongside."""
    cfg, p, _ = rs.load(name)
    g, o = GlobalData(cfg, p), OracleScene(cfg, p)
    g.initialize()
    o.initialize()
    assert bonded_set(g.contacts()) == bonded_set(o.contacts())
    done = 0
    if lead:
        g.simulate(lead)
        st = g.particles()
        o.set_particles(**{k: st[k] for k in ("pos", "vel", "omega", "quat", "wall_shear")})
        o.set_contacts(g.contacts())
        done = lead
    for k in chunks:
        g.simulate(k)
        o.simulate(k)
        done += k
        compare(g, o, f"{name} after {done} steps")
    return g, o


def test_reference_cube_911_wall_impact(gpu):
    # the front face is 10 mm from the wall: contact near step 4,000 at dt 1e-7;
    # the GPU covers most of the approach alone, the oracle joins before impact
    g, o = run_pair("cube_911", (500, 500, 1000, 1000), lead=3600)
    assert np.abs(o.particles()["wall_shear"]).sum() > 0 or \
        np.abs(o.particles()["force"][:, 0]).max() > 0
    assert g.stats()["error"] == 0
    g.close()


def test_reference_carom_break(gpu):
    # the cue ball rolls 1.21 m to the rack, slowing from 5 m/s on the floor:
    # the break comes near step 103,500 at dt 2.56e-6; the GPU covers the
    # approach alone, the oracle joins for the break
    g, o = run_pair("carom", (1500, 1500, 1500, 1500, 2000), lead=101_500)
    v = o.particles()["vel"]
    assert (np.linalg.norm(v, axis=1) > 1e-3).sum() > 1, "the break moved more than the cue ball"
    assert g.stats()["error"] == 0
    g.close()
