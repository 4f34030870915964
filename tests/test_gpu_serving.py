"""GPU: continuous batching gives every request the result it gets alone.

Requests overlap on the device (several scenes live at once) and some are
admitted only after others finish and free their slots; each served result
(final particle state) must equal, bit for bit, the same scene stepped alone
on a single-scene handle in the same precision."""
import numpy as np
import pytest

from taichi_dem_julia_port_gb300 import GlobalData, scenes
from taichi_dem_julia_port_gb300.serving import ArenaSizing, Request, Server

pytestmark = pytest.mark.gpu

KEYS = ("pos", "vel", "omega", "quat", "wall_shear")


def small_requests():
    def cube(side, seed, speed):
        def make():
            sc = scenes.bonded_cube(side, speed=speed, steps=0, seed=seed, E=3e8, friction=0.4)
            sc.cfg = sc.cfg.replace(bond_tensile_strength=3e5, bond_shear_strength=3e5)
            return sc
        return make

    def pour(n, seed):
        def make():
            sc = scenes.granular_pour(n, box=(0.03, 0.03, 0.04), seed=seed, steps=0,
                                      rmin=0.8e-3, rmax=1.2e-3, E=2e8, friction=0.6)
            sc.cfg = sc.cfg.replace(dt=1e-6)
            rng = np.random.default_rng(seed)
            sc.particles.vel = rng.normal(0, 5.0, sc.particles.vel.shape)
            return sc
        return make

    specs = [(cube(5, 1, 20.0), 60, 125), (pour(400, 2), 90, 400), (cube(6, 3, 25.0), 40, 216),
             (pour(300, 4), 120, 300), (cube(4, 5, 15.0), 75, 64), (pour(500, 6), 50, 500)]
    return [Request(k, 0.0, steps, make, n) for k, (make, steps, n) in enumerate(specs)]


def alone_state(req, precision):
    sc = req.make_scene()
    g = GlobalData(sc.cfg, sc.particles, precision=precision)
    if sc.bonded:
        g.initialize()
    g.simulate(req.steps)
    st = g.particles(forces=False)
    stats = g.stats()
    g.close()
    return st, stats


@pytest.mark.parametrize("precision,policy", [("fp32", "fifo"), ("fp64", "fifo"),
                                              ("fp32", "sjf")])
def test_served_results_equal_alone(gpu, precision, policy):
    reqs = small_requests()
    # room for about two scenes at a time: the rest wait for freed slots
    sizing = ArenaSizing(max_particles=1000, max_contacts=16000, max_buckets=16384,
                         max_scenes=4, max_coordinate_number=16, contacts_per_particle=16)
    with Server(sizing, precision=precision, chunk_steps=16, policy=policy,
                max_active=700) as srv:
        rep = srv.run(reqs, realtime=False)
    assert len(rep.results) == len(reqs)
    assert rep.admissions_deferred > 0, "the arena was meant to be too small for all at once"
    for res, req in zip(rep.results, reqs):
        ref, ref_stats = alone_state(req, precision)
        assert res.stats["steps_done"] == req.steps
        assert res.stats["bonds_broken"] == ref_stats["bonds_broken"]
        for k in KEYS:
            np.testing.assert_array_equal(res.state[k], ref[k], err_msg=f"request {req.rid} {k}")


def test_server_reports_latency_and_throughput(gpu):
    reqs = small_requests()
    for k, r in enumerate(reqs):
        r.arrival_s = 0.01 * k
    sizing = ArenaSizing.from_budget(2e8, max_scenes=8)
    with Server(sizing, precision="fp32", chunk_steps=32, keep_state=False) as srv:
        rep = srv.run(reqs, realtime=True)
    pct = rep.latency_percentiles()
    assert rep.particle_steps == sum(r.n * r.steps for r in rep.results)
    assert rep.throughput > 0 and 0 < pct["p50"] <= pct["p99"] <= rep.makespan_s
