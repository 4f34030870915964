"""dem_step_exchange through page-locked buffers (GlobalData.state_buffers):
upload, steps and read-back of the particle state in one call.  With the
integrator split over four warps per 32 particles (the layout of scenes of up
to 256 particles per SM) the last step's integrator writes the state into the
caller's buffers while it runs; with one thread per particle the state is
read after the step.  Either way the buffers end up holding the state of
uninterrupted stepping, bit for bit."""
import numpy as np
import pytest

from taichi_dem_julia_port_gb300 import GlobalData, Wall, scenes
from taichi_dem_julia_port_gb300._abi import DEM_ERR_CAPACITY, DemError
from tests.test_gpu_parity import random_cloud
from tests.test_gpu_tables import two_material_tables

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "omega", "quat", "force", "moment", "wall_shear")


def plain_run(cfg, p, steps, precision="fp64", tables=None):
    g = GlobalData(cfg, p, precision=precision, tables=tables)
    g.initialize()
    g.simulate(steps)
    out, st = g.particles(), g.stats()
    g.close()
    return out, st


def exchange_run(cfg, p, steps, per_call, lanes, precision="fp64", tables=None):
    g = GlobalData(cfg, p, precision=precision, tables=tables)
    g.set_launch_shape(integrate_lanes=lanes)
    g.initialize()
    buf = g.state_buffers(forces=True)
    done = 0
    while done < steps:
        k = min(per_call, steps - done)
        buf.step(k)
        done += k
    out = {k: getattr(buf, k).copy() for k in FIELDS}
    st = g.stats()
    buf.close()
    g.close()
    return out, st


def check_layouts(cfg, p, steps, precision="fp64", tables=None):
    want, st0 = plain_run(cfg, p, steps, precision, tables)
    for lanes, per_call in ((0, 1), (0, 7), (1, 1)):
        got, st = exchange_run(cfg, p, steps, per_call, lanes, precision, tables)
        for k in FIELDS:
            np.testing.assert_array_equal(got[k], want[k],
                                          err_msg=f"{k} lanes={lanes} per_call={per_call}")
        calls = -(-steps // per_call)
        # the split layout wrote every call's state during its last step
        assert st["exchanges_direct"] == (calls if lanes == 0 else 0), (lanes, per_call)
        assert st["error"] == 0 and st["bonds_broken"] == st0["bonds_broken"]
    return want, st0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_exchange_equals_uninterrupted_stepping(gpu, precision):
    """A bonded cube's wall impact (wall contacts, spin, bonds breaking near
    step 900), one step and seven steps per call, both integrator layouts."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    want, st0 = check_layouts(sc.cfg, sc.particles, 1000, precision)
    assert st0["bonds_broken"] > 0
    assert np.count_nonzero(np.any(want["wall_shear"] != 0, axis=1)) > 0


def test_exchange_with_tables_and_two_walls(gpu):
    """A two-material cube against the floor and an inclined wall: the
    records carry the first wall's shear history, as dem_get_particles does."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=12)
    z = sc.particles.pos[:, 2]
    gm = np.round((z - z.min()) / 0.02).astype(int) % 2
    nrm = np.array([-1.0, 0.0, -1.0]) / np.sqrt(2.0)
    t = two_material_tables(gm, [Wall(list(sc.cfg.wall_normal), sc.cfg.wall_distance, 2),
                                 Wall(nrm.tolist(), 0.0105, 2)])
    want, st0 = check_layouts(sc.cfg, sc.particles, 300, tables=t)
    assert np.count_nonzero(np.any(want["wall_shear"] != 0, axis=1)) > 0


@pytest.mark.parametrize("per_call", [1, 5])
def test_exchange_takes_the_callers_changes(gpu, per_call):
    """Values written into the buffers between calls reach the step: the
    split integrator reads the orientations and the first wall's shear
    history from the caller's arrays (the upload before the step carries the
    positions, velocities and spins), with the same results as uploading
    them with dem_set_particles."""
    sc = scenes.bonded_cube(6, speed=30.0, steps=0, seed=3)
    runs = []
    for via_buffers in (False, True):
        g = GlobalData(sc.cfg, sc.particles)
        g.initialize()
        g.simulate(300)  # into the wall impact: spin and wall shear
        st = g.particles()
        q = st["quat"] + np.array([0.01, -0.02, 0.03, 0.04])
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        om = st["omega"] + np.array([1.0, -2.0, 0.5])
        ws = 0.5 * st["wall_shear"]
        if via_buffers:
            buf = g.state_buffers(forces=True)
            buf.quat[:] = q
            buf.omega[:] = om
            buf.wall_shear[:] = ws
            for _ in range(10 // per_call):
                buf.step(per_call)
            out = {k: getattr(buf, k).copy() for k in FIELDS}
            assert g.stats()["exchanges_direct"] == 10 // per_call
            buf.close()
        else:
            g.set_particles(pos=st["pos"], vel=st["vel"], omega=om, quat=q, wall_shear=ws)
            g.simulate(10)
            out = g.particles()
        runs.append(out)
        g.close()
    assert np.count_nonzero(np.any(runs[0]["wall_shear"] != 0, axis=1)) > 0
    for k in FIELDS:
        np.testing.assert_array_equal(runs[1][k], runs[0][k], err_msg=k)


def test_exchange_into_other_buffers(gpu):
    """Input and output in different page-locked buffers: the output receives
    every value (an exchange in place leaves out the values the step did not
    change, which the buffer holds already), and the input is not written."""
    import ctypes as C
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    want, _ = plain_run(sc.cfg, sc.particles, 400)
    g = GlobalData(sc.cfg, sc.particles)
    g.initialize()
    g.simulate(399)
    src, dst = g.state_buffers(forces=True), g.state_buffers(forces=True)
    before = {k: getattr(src, k).copy() for k in FIELDS}
    for k in FIELDS:  # stale values everywhere in the output buffer
        getattr(dst, k)[:] = -7.0
    rc = g.lib.dem_step_exchange(g.h, C.byref(src._in), 1, C.byref(dst._out))
    assert rc == 0
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(dst, k), want[k], err_msg=k)
        np.testing.assert_array_equal(getattr(src, k), before[k], err_msg=k)
    assert g.stats()["exchanges_direct"] == 1
    src.close()
    dst.close()
    g.close()


def test_exchange_alternating_buffers(gpu):
    """Two buffer sets used in turn (each captured exchange graph belongs to
    one set), with a launch-shape change and a skin change in between that
    drop the captured graphs: the state stays that of uninterrupted stepping."""
    sc = scenes.bonded_cube(8, speed=30.0, steps=0, seed=2)
    steps = 240
    want, _ = plain_run(sc.cfg, sc.particles, steps)
    g = GlobalData(sc.cfg, sc.particles)
    g.initialize()
    bufs = [g.state_buffers(forces=True), g.state_buffers(forces=True)]
    cur = bufs[0]
    for s in range(steps):
        nxt = bufs[s % 2]
        if nxt is not cur:
            for k in FIELDS:
                getattr(nxt, k)[:] = getattr(cur, k)
            cur = nxt
        if s == 80:
            g.set_launch_shape(force_block=64)
        if s == 160:
            g.set_skin_factor(0.5)
        cur.step(1)
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(cur, k), want[k], err_msg=k)
    assert g.stats()["exchanges_direct"] == steps
    for b in bufs:
        b.close()
    g.close()


def test_exchange_reports_a_device_error(gpu):
    """A contact-capacity overflow in the exchanged step reaches the caller
    through the error word that the integrator copies with the state."""
    cfg, p = random_cloud(2000, (0.012, 0.012, 0.012), 0.0008, 0.0015, seed=9,
                          cfg_kw=dict(max_coordinate_number=2))
    g = GlobalData(cfg, p)
    buf = g.state_buffers()
    with pytest.raises(DemError) as e:
        buf.step(1)
    assert e.value.code == DEM_ERR_CAPACITY
    st = g.stats()
    assert st["exchanges_direct"] == 1 and st["error"] == DEM_ERR_CAPACITY
    buf.close()
    g.close()
