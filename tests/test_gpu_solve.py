"""The `solve` drop-in end to end (src/executor.jl:174-394): the reference's
911-sphere bonded cube scene (cfg/2.toml with its p4p file, packed as a test
fixture) run through `solve` on the GPU writes output.p4p / output.p4c every
save interval, with the contacts compacted into p4c records on the device
(dem_get_io_contacts); the same files written from the CPU oracle's state
must agree under the reference's own comparison (compare_p4p / compare_p4c,
src/utils.jl:170-209: contacts as sorted pairs, rtol = sqrt(eps)) up to 1,000
steps into the wall impact, and within the parity tests' short-horizon bound
(1e-5) over the whole run."""
import numpy as np
import pytest

from oracle.oracle import OracleScene, host_threads
from taichi_dem_julia_port_gb300 import GlobalData, p4io
from taichi_dem_julia_port_gb300.executor import solve
from tests import reference_scenes as rs

pytestmark = pytest.mark.gpu


def oracle_solve(cfg, p, out_dir, no_bond=False):
    """The same loop on the CPU oracle, writing with the same p4p/p4c writers."""
    o = OracleScene(cfg, p, threads=host_threads())
    if not no_bond:
        o.initialize()
    out_dir.mkdir(parents=True, exist_ok=True)
    save_per = max(cfg.save_per_steps, 1)

    def save(fp, fc, t):
        st = o.particles(forces=False)
        p4io.write_p4p(fp, t, p.id, p.gid, p.volume, p.mass, st["pos"], st["vel"])
        c = o.contacts()
        p4io.write_p4c(fc, t, c["i"], c["j"], c["point"], c["force"], c["bonded"])

    with open(out_dir / "output.p4p", "w") as fp, open(out_dir / "output.p4c", "w") as fc:
        save(fp, fc, 0.0)
        step = 0
        while step < cfg.total_steps:
            o.simulate(save_per)
            step += save_per
            save(fp, fc, step * cfg.dt)
    return o


def test_solve_writes_the_reference_files(gpu, tmp_path):
    cfg, p, _ = rs.load("cube_911")
    # six save intervals of 1,000 steps: the approach and the start of the
    # wall impact (the front face meets the wall near step 4,000)
    cfg = cfg.replace(target_time=6 * cfg.saving_interval_time)
    (tmp_path / "gpu_solve").mkdir()
    g = solve("cfg/2.toml", cfg=cfg, particles=p, output_dir=tmp_path / "gpu_solve")
    o = oracle_solve(cfg, p, tmp_path / "oracle_solve")
    gp, op = tmp_path / "gpu_solve" / "output.p4p", tmp_path / "oracle_solve" / "output.p4p"
    gc, oc = tmp_path / "gpu_solve" / "output.p4c", tmp_path / "oracle_solve" / "output.p4c"
    recs = p4io.read_p4p(gp)
    save_per = cfg.save_per_steps  # trunc(1e-4 / 1e-7) = 999 in binary64, as in the reference
    n_rec = 1 + -(-cfg.total_steps // save_per)
    assert len(recs) == n_rec and recs[-1].timestep == (n_rec - 1) * save_per * cfg.dt
    # the reference's own tolerance (rtol = sqrt(eps)) holds through the
    # approach and the first 1,000 steps of the impact; over the whole file
    # the short-horizon bound of the parity tests (1e-5): the impact makes
    # rounding differences grow (the last record's velocities differ by ~2e-8)
    ro, rc_g, rc_o = p4io.read_p4p(op), p4io.read_p4c(gc), p4io.read_p4c(oc)
    early = sum(1 for r in recs if r.timestep <= 5.0e-4 + 1e-12)
    assert early >= 5
    p4io.compare_p4p(recs[:early], ro[:early])
    p4io.compare_p4c(rc_g[:early], rc_o[:early])
    p4io.compare_p4p(gp, op, rtol=1e-5)
    p4io.compare_p4c(gc, oc, rtol=1e-5)
    crecs = p4io.read_p4c(gc)
    assert crecs[0].bonded.all() and len(crecs[0].i) > 2000
    # the wall impact has started by the last record
    assert np.abs(o.particles()["wall_shear"]).sum() > 0
    g.close()


def test_io_contacts_equal_the_full_contact_read(gpu):
    """The device-compacted p4c records equal the active contacts read in
    full (dem_get_contacts), in FP64 and in the FP32 force mode (whose stored
    forces are hi/lo pairs decoded on the device)."""
    cfg, p, _ = rs.load("cube_911")
    for precision in ("fp64", "fp32"):
        g = GlobalData(cfg, p, precision=precision)
        g.initialize()
        g.simulate(4600)  # into the wall impact
        rec, full = g.io_contacts(), g.contacts()
        assert len(rec) == len(full["i"]) > 0
        np.testing.assert_array_equal(rec["i"], full["i"])
        np.testing.assert_array_equal(rec["j"], full["j"])
        np.testing.assert_array_equal(rec["bonded"], full["bonded"])
        np.testing.assert_array_equal(rec["point"], full["point"])
        np.testing.assert_array_equal(rec["force"], full["force"])
        g.close()
