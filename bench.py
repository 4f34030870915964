#!/usr/bin/env python
"""DEM step throughput on GB300 (one JSON line on stdout).

Workload (default): the 17,576-sphere bonded-cube impact — 26x26x26 simple
cubic lattice, radius 0.01 m ±5 %, 50,700 EBPM bonds, 20 m/s toward a rigid
plane, FP64, dt = 1e-6 s.  One "step" is one DEM time step (`simulate!`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Our arm: --advance untimed steps (default 4,000 for the 17,576-sphere cube:
the cube meets the wall after about 50 steps and its stress wave has crossed
it by about 3,000, so the timed window lies in the fragmentation, with wall
contacts, Hertz contacts between fragments and bonds breaking), W untimed
warm-up steps, then K steps each timed with CUDA
events on the library's stream, with a 256 MiB write between steps to flush
L2 (the scene itself fits in L2).  value = particle-steps/s over all ranks
(max time over ranks); `config.timed_window` gives the window's first step,
mean contact and bond counts, wall contacts, bonds broken and full pair
searches.  `e2e` repeats the metric through the C ABI with host buffers on
the same window (replayed from its first state until at least --e2e-steps
steps are timed): every step uploads the particle state from page-locked host
arrays, steps, and reads it back into them (one dem_step_exchange call per
step, through GlobalData.state_buffers).  `roofline` reports the dominant
kernel from per-phase CUDA events (dem_step_profiled) over the same window,
against its algorithmic bytes (every field once per unit; re-reads from L2
are `gather_bytes`).  `cpu_baseline` times the CPU oracle (OpenMP, all host
threads) from the window's first state.  The clock sampler polls every 20 ms;
a window shorter than five samples is followed by untimed steps of the same
load until five are in (`clocks.padding_steps`).

The default line also carries `batched` (below), `pour` (the 2,000,000-sphere
pour settling, and pre-compacted into a bed with about one contact per sphere)
and `served` (a 100-request Poisson stream with step counts scaled by 0.05,
p50/p99 completion latency, against the plain FP64 path scene by scene).

--workload c4 steps 256 independent scenes (500-20,000 spheres each, half
bonded cubes, half pours, FP32 force / FP64 state) together in one arena,
after the autotuner picks the search-cell factor and launch shape, and reports
the same metric for the plain FP64 path run scene by scene.  The default run
appends this comparison as `batched` (50 timed steps).  --workload c5 runs the
served request stream (Poisson arrivals, continuous batching within an HBM
budget) and reports aggregate particle-steps/s with p50/p99 completion latency.

For c1/c2 the line adds `reference_gpu_proxy`: the same scene on a plain CUDA
C++ restatement of the reference's GPU path with its own structure (AoS
records, BitTables, ~25 launches and 3 device-to-host reads per step;
baseline/refproxy), timed the same way, standing in for the reference's
CUDA.jl path, which cannot run on this GPU.

--impl reference times the CPU restatement of the reference step on all host
threads (the reference's own GPU path, Julia + CUDA.jl, cannot run here).
With N > 1 (torchrun) every rank steps an independent replica (the path does
not shard: one scene per GPU); the reference arm runs on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

# Algorithmic bytes: every field a kernel must move, counted once per unit
# (particle fields once per particle, contact columns once per contact), from
# the kernels' SoA field lists in dem_kernels.cu.
#
# k_force, per contact: ids, flags and the carried-state slot read (16 B); the
# entry in the partner's incoming list (counter read and written, entry
# written: 16 B); the nine force contributions written (72 B); a bond reads
# its carried F, tau_i, tau_j (72 B) and writes k, F, tau_i, tau_j (96 B); a
# Hertz contact reads s (24 B) and writes k, F, s (72 B).  Per particle, once:
# position, velocity, spin, radius, mass and the bond section constants
# (112 B).  A particle gathered again by its second and later contacts is a
# re-read served from L2: reported apart as `gather_bytes` (88 B per contact
# end beyond the first), not counted as algorithmic.
FORCE_BYTES_BOND = 16 + 16 + 72 + 72 + 96
FORCE_BYTES_HERTZ = 16 + 16 + 72 + 24 + 72
FORCE_BYTES_PER_PARTICLE = 112
GATHER_BYTES_PER_CONTACT_END = 88
# k_integrate, per particle: reads position, velocity, spin, quaternion, 1/m,
# r, 1/I, wall shear, row bounds and incoming count (164 B); writes position,
# velocity, spin, quaternion, wall shear, force and moment totals, the FP32
# position and the incoming count (196 B).  Per contact: its nine
# contributions and its incoming-list entry read (80 B).
INTEGRATE_BYTES_PER_PARTICLE = 164 + 196
INTEGRATE_BYTES_PER_CONTACT = 80
# a pour settling without contacts: every particle is torque-free and keeps
# the identity orientation, so the integrator writes neither its spin (24 B)
# nor its quaternion (32 B)
INTEGRATE_BYTES_SETTLING = INTEGRATE_BYTES_PER_PARTICLE - 3 * 8 - 4 * 8
# k_search on a neighbour-list step, per particle: path byte, current row
# bounds, list length, FP32 position, next row bounds written, four list
# partner indices (53 B; the partners' FP32 positions are re-reads); per
# surviving contact: partner and flags read, survival flag written and read,
# the next row's ids, flags and carried-state slot written (26 B).
DETECT_BYTES_PER_PARTICLE = 1 + 8 + 4 + 16 + 8 + 4 * 4
ROW_BYTES_PER_CONTACT = 8 + 2 + 16


def algorithmic_bytes(n: int, contacts: int, bonds: int, settling: bool = False) -> dict:
    """Algorithmic bytes of one step's three kernels (see the constants)."""
    hertz = contacts - bonds
    integ = INTEGRATE_BYTES_SETTLING if settling and contacts == 0 else INTEGRATE_BYTES_PER_PARTICLE
    return {"force": bonds * FORCE_BYTES_BOND + hertz * FORCE_BYTES_HERTZ
            + (n * FORCE_BYTES_PER_PARTICLE if contacts else 0),
            "integrate": n * integ + contacts * INTEGRATE_BYTES_PER_CONTACT,
            "contacts": n * DETECT_BYTES_PER_PARTICLE + contacts * ROW_BYTES_PER_CONTACT}


# k_search (contact update: full search or lists, next rows), k_force, k_integrate
KERNELS_PER_STEP = 3
# FP64-pipe instructions per unit, from ncu (sm__thread_inst_executed_pipe_fp64_pred_on.sum
# of one launch over the units it processed).  Force kernel, FP64 mode: per
# Hertz contact 151.0 (a 100,000-sphere compacted bed, every contact a Hertz
# contact: 1.503e7 per launch), per bond 116.1 (the 17,576-sphere cube in its
# fragmentation, 41,427 bonds and 6,670 Hertz contacts: 5.818e6 per launch,
# less the Hertz share); FP32 mode per bond 15.0 (the same cube before its
# impact).  Integrator per particle: 92.0 in FP64 mode (the cube in its
# fragmentation, split over four warps per 32 particles: 1.616e6 per launch;
# the one-thread form measured 84.1), 51.0 in the FP32 mode (64 scenes of the
# batched workload).  Then GB300's FP64 pipe width.
FP64_INST = {("force", "fp64", "bond"): 116.1, ("force", "fp64", "hertz"): 151.0,
             ("force", "fp32", "bond"): 15.0,
             ("integrate", "fp64"): 92.0, ("integrate", "fp32"): 51.0}
# The integrator skips the quaternion increment of a particle with exactly zero
# spin, the normalisation of a spinless identity orientation and the spin
# update of a particle with exactly zero torque: in the pour's settling phase
# (no contacts) that is every particle (ncu on a 400,000-sphere pour:
# 7,200,000 FP64 thread instructions per launch)
FP64_INST_WORKLOAD = {("c3", "integrate", "fp32"): 18.0}
FP64_LANES_PER_SM = 2
SM_COUNT = 152


def fp64_roofline(kernel: str, precision: str, n_particles: int, n_bond: int, ms: float,
                  clk: dict, peaks: dict, workload: str | None = None,
                  n_hertz: int = 0) -> dict | None:
    """The FP64-pipe roofline of the force kernel (per bond and per Hertz
    contact) or the integrator (per particle): FP64 instructions over the live
    per-phase time against the pipe's peak at the SM clock sampled during the
    timed region (else the measured maximum clock of MEASURED_PEAKS.json, else
    2,070 MHz), saying which.  None when a count per unit is not known."""
    if kernel == "force":
        pb = FP64_INST.get(("force", precision, "bond"))
        ph = FP64_INST.get(("force", precision, "hertz"))
        if (n_bond and pb is None) or (n_hertz and ph is None) or not (n_bond or n_hertz):
            return None
        inst = (pb or 0.0) * n_bond + (ph or 0.0) * n_hertz
        units = n_bond + n_hertz
        per = inst / units
    else:
        per = FP64_INST_WORKLOAD.get((workload, kernel, precision),
                                     FP64_INST.get((kernel, precision)))
        units = n_particles
    if per is None or not units or not ms:
        return None
    if clk.get("sm_mhz"):
        sm_mhz, src = clk["sm_mhz"], "the median SM clock sampled during the timed region"
    elif peaks.get("sm_max_mhz"):
        sm_mhz, src = float(peaks["sm_max_mhz"]), "the maximum SM clock of MEASURED_PEAKS.json"
    else:
        sm_mhz, src = 2070.0, "the nominal maximum SM clock"
    peak = FP64_LANES_PER_SM * SM_COUNT * sm_mhz * 1e6 / 1e9
    ach = per * units / (ms * 1e-3) / 1e9
    return {"unit": "G FP64 thread-instructions/s", "achieved": ach, "peak": peak,
            "frac": ach / peak, "inst_per_unit": per,
            "unit_counted": "contact" if kernel == "force" else "particle",
            "peak_source": f"{FP64_LANES_PER_SM} FP64 lanes per SM per cycle x {SM_COUNT} SMs "
                           f"at {sm_mhz:.0f} MHz ({src})"}
L2_FLUSH_BYTES = 256 << 20

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
# of each dominant kernel, from one ncu capture each, with the particles that
# launch processed.  The batched captures ran on the first 64 scenes of the
# batch (431,416 spheres); their traffic is scaled to a launch by particles
# processed.  Keys: workload and timed window ("c2" the cube in its impact
# window, "c3" the pour settling, "c3bed" the compacted bed), kernel.
NCU_TRAFFIC = {
    ("c2", "force"): (7.470848e6, 17576),          # k_force<double>, step 4,006
    ("c2", "contacts"): (2.336768e6, 17576),       # k_search, list step, step 4,006
    ("c2", "integrate"): (9.095680e6, 17576),      # k_integrate_split, step 4,006
    ("c3bed", "force"): (94.237e6, 400000),        # k_force4<float>, 400,000-sphere bed
    ("c3bed", "contacts"): (51.041e6, 400000),     # k_search, list step (one lane per particle)
    ("c3bed", "integrate"): (181.203e6, 400000),   # k_integrate3 (FP32 gather)
    ("c3", "integrate"): (628.523e6, 2000000),     # k_integrate3 (FP32 mode, no contacts)
    ("c3", "contacts"): (43.036e6, 2000000),       # k_search, list step (wide pass)
    ("c4", "force"): (186.237e6, 431416),          # k_force<float, 1>
    ("c4", "integrate"): (176.134e6, 431416),      # k_integrate3<1> (FP32 gather)
    ("c4", "contacts"): (35.621e6, 431416),        # k_search<0, 1>, list step
}


def ncu_traffic(workload: str, kernel: str, n: int):
    t = NCU_TRAFFIC.get((workload, kernel))
    return None if t is None else t[0] * n / t[1]


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured",
                "sm_max_mhz": d.get("sm_max_mhz")}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is live (first line in)
            t_end = time.time() + 3.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def count(self) -> int:
        """Samples taken since the timed region started."""
        return len(self.lines) if self.proc else 1 << 30

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_scene(name: str, pour_n: int = 2_000_000):
    from taichi_dem_julia_port_gb300 import scenes
    if name == "c1":
        return scenes.c1(), "bonded cube 10^3 = 1,000 spheres, -10 m/s, FP64, dt 1e-6"
    if name == "c2":
        return scenes.c2(), "bonded cube 26^3 = 17,576 spheres, 20 m/s, FP64, dt 1e-6"
    if name == "c3":
        return (scenes.c3(pour_n),
                f"unbonded pour {pour_n:,} spheres in 0.4 x 0.4 x 1.2 m, FP32 force, dt 2e-7")
    if name == "c3bed":
        f = (pour_n / 2_000_000) ** 0.5  # the same column height on a smaller floor
        return (scenes.granular_bed(pour_n, box=(0.4 * f, 0.4 * f, 1.2)),
                f"the pour's {pour_n:,} spheres pre-compacted into a bed of touching columns "
                "(about one Hertz contact per sphere), FP32 force, dt 2e-7")
    raise ValueError(name)


def batched_scenes(count: int):
    from taichi_dem_julia_port_gb300 import scenes
    batch = scenes.mixed_batch(count)
    n = sum(s.n for s in batch)
    desc = (f"{count} independent scenes, 500-20,000 spheres log-uniform ({n:,} total), half "
            "bonded cubes / half unbonded pours, per-scene E U(1e7,1e9) friction U(0.2,0.8), "
            "FP32 force / FP64 state, one arena, CUDA graph per step")
    return batch, n, desc


def oracle_sample(scene_list, seconds: float) -> dict:
    """CPU oracle (all host threads) over the given scenes in turn, a few
    steps each, for about `seconds`."""
    from oracle.oracle import OracleScene, host_threads
    threads = host_threads()
    work, el, used = 0, 0.0, 0
    per = max(seconds / max(len(scene_list), 1), 0.5)
    for sc in scene_list:
        o = OracleScene(sc.cfg, sc.particles, threads=threads)
        if sc.bonded:
            o.initialize()
        o.simulate(1)
        steps, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < per and steps < 2000:
            o.simulate(1)
            steps += 1
        el += time.perf_counter() - t0
        work += sc.n * steps
        used += 1
        if el >= seconds:
            break
    return {"value": work / el, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{used} scenes of the workload, {work:,} particle-steps in {el:.1f} s "
                      "on the CPU oracle"}


def precision_errors(scene_list, steps: int, lib) -> dict:
    """FP32 force mode against FP64 on the same scenes (each alone on a
    single-scene handle; the FP64 path equals the CPU oracle within 1e-9 in
    the parity tests): after `steps` steps from the same start, the kinetic
    energy, broken-bond count and positions; then one step from an identical
    state (the FP64 state copied into the FP32 handle), the particle forces."""
    from taichi_dem_julia_port_gb300 import GlobalData
    ke_err, pos_err, force_err, bond_diff, bonds = 0.0, 0.0, 0.0, 0, 0
    for sc in scene_list:
        hs = []
        for prec in ("fp64", "fp32"):
            g = GlobalData(sc.cfg, sc.particles, precision=prec, lib=lib)
            if sc.bonded:
                g.initialize()
            g.simulate(steps)
            hs.append(g)
        g64, g32 = hs
        m = np.asarray(sc.particles.mass, dtype=np.float64)
        p64, p32 = g64.particles(), g32.particles()
        ke = [0.5 * float(np.sum(m * np.sum(p["vel"] ** 2, axis=1))) for p in (p64, p32)]
        if ke[0] > 0:
            ke_err = max(ke_err, abs(ke[1] - ke[0]) / ke[0])
        r = np.median(np.cbrt(3.0 * np.asarray(sc.particles.volume) / (4.0 * np.pi)))
        pos_err = max(pos_err, float(np.max(np.abs(p32["pos"] - p64["pos"]))) / r)
        s64, s32 = g64.stats(), g32.stats()
        bond_diff = max(bond_diff, abs(s32["bonds_broken"] - s64["bonds_broken"]))
        bonds += s64["bonded"]
        # one step from an identical state
        g32.set_particles(**{k: p64[k] for k in ("pos", "vel", "omega", "quat", "wall_shear")})
        g32.set_contacts(g64.contacts())
        g64.simulate(1)
        g32.simulate(1)
        f64, f32 = g64.particles()["force"], g32.particles()["force"]
        scale = float(np.max(np.linalg.norm(f64, axis=1)))
        if scale > 0:
            force_err = max(force_err, float(np.max(np.linalg.norm(f32 - f64, axis=1))) / scale)
        g64.close()
        g32.close()
    return {"scenes": len(scene_list), "steps": steps,
            "kinetic_energy_rel_err_max": ke_err, "position_err_max_in_radii": pos_err,
            "force_rel_err_max_one_step": force_err,
            "broken_bond_count_diff_max": bond_diff, "bonds": bonds,
            "note": "FP32 force mode vs the FP64 path, each scene alone; force error relative "
                    "to the scene's largest particle force"}


def run_batched(args, lib, quick: bool = False, dist=None) -> dict:
    """The batched workload on one arena: returns the JSON fields."""
    import torch
    from taichi_dem_julia_port_gb300 import Arena, GlobalData
    from taichi_dem_julia_port_gb300.autotune import autotune

    batch, n_total, desc = batched_scenes(args.scenes)
    precision = args.precision or "fp32"
    arena = Arena(n_total, max_scenes=len(batch), precision=precision, lib=lib)
    for sc in batch:
        arena.add(sc.cfg, sc.particles, init_bonds=sc.bonded)
    arena.step(max(args.warmup, 3))
    tune = None
    if not getattr(args, "no_tune", False):
        tune = autotune(arena, sm_count=torch.cuda.get_device_properties(0).multi_processor_count,
                        steps=5 if quick else 10)
    steps = min(args.steps, 50) if quick else args.steps
    clocks = ClockSampler(torch.cuda.current_device())
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks.start()
    ms = arena.step_timed(steps)  # CUDA events on the arena's stream
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist)  # every rank steps its own replica
    ms_per_step = ms / steps
    ph = arena.step_profiled()
    stats = [arena.stats(k) for k in arena.scenes()]
    contacts = sum(x["contacts"] for x in stats)
    bonded = sum(x["bonded"] for x in stats)
    errors = sorted({x["error"] for x in stats})
    arena.close()
    value = n_total * steps / (ms * 1e-3)
    # the plain FP64 path, scene by scene on single-scene handles
    plain_ms = 0.0
    for sc in ([] if getattr(args, "no_plain", False) else batch):
        g = GlobalData(sc.cfg, sc.particles, precision="fp64", lib=lib)
        if sc.bonded:
            g.initialize()
        g.simulate(3)
        plain_ms += g.simulate_timed(10) / 10
        g.close()
    plain = n_total / (plain_ms * 1e-3) if plain_ms > 0 else None
    peaks = load_peaks()
    alg = algorithmic_bytes(n_total, contacts, bonded)
    dom = max(ph, key=ph.get)
    roof = {"bound": "hbm", "kernel": dom, "unit": "GB/s", "peak": peaks["hbm_gbs"],
            "peak_source": peaks["source"], "traffic": ncu_traffic("c4", dom, n_total),
            "phase_ms": ph}
    if dom in alg:
        ach = alg[dom] / (ph[dom] * 1e-3) / 1e9
        roof.update({"achieved": ach, "frac": ach / peaks["hbm_gbs"], "algorithmic_bytes": alg[dom]})
    fr = fp64_roofline(dom, precision, n_total, bonded, ph.get(dom), clk, peaks,
                       n_hertz=contacts - bonded)
    if fr:
        roof["fp64_pipe"] = fr
    perr = None
    if precision == "fp32":
        perr = precision_errors(batch[:8] if quick else batch[:16], 300, lib)
    return {"value": value, "ms_per_step": ms_per_step, "steps": steps, "desc": desc,
            "fp32_error_vs_fp64": perr,
            "n_particles": n_total, "scenes": len(batch), "contacts": contacts,
            "contact_steps_per_s": contacts * steps / (ms * 1e-3), "precision": precision,
            "plain_fp64_scene_by_scene": plain,
            "speedup_vs_plain": value / plain if plain else None,
            "tune": tune.as_dict() if tune else None, "roofline": roof, "clocks": clk, "errors": errors,
            "batch": batch}


def run_batched_e2e(args, lib, batch, steps: int, dist=None) -> dict:
    """The batched job end to end through the public API: scenes uploaded from
    host arrays (dem_arena_add), `steps` steps, every scene's state read back."""
    from taichi_dem_julia_port_gb300 import Arena
    n_total = sum(s.n for s in batch)
    h2d = sum(s.particles.volume.nbytes + s.particles.mass.nbytes + s.particles.pos.nbytes +
              s.particles.vel.nbytes for s in batch)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    arena = Arena(n_total, max_scenes=len(batch), precision=args.precision or "fp32", lib=lib)
    ids = [arena.add(sc.cfg, sc.particles, init_bonds=sc.bonded) for sc in batch]
    arena.step(steps)
    d2h = 0
    for sid in ids:
        st = arena.particles(sid, forces=False)
        d2h += st["pos"].nbytes + st["vel"].nbytes
    el = max_over_ranks(time.perf_counter() - t0, dist)
    arena.close()
    ws = dist.get_world_size() if dist else 1
    return {"value": ws * n_total * steps / el, "unit": "particle-steps/s",
            "h2d_bytes_per_step": int(h2d / steps), "d2h_bytes_per_step": int(d2h / steps),
            "steps": steps, "note": "whole job: arena set-up and upload, steps, read-back"}


def main_batched(args, lib, ws, rank, dist=None) -> None:
    r = run_batched(args, lib, dist=dist)
    e2e = run_batched_e2e(args, lib, r["batch"], args.e2e_steps * 4, dist=dist)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = oracle_sample(r["batch"][:16], args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": ws * r["value"], "unit": "particle-steps/s",
            "n_gpus": ws, "steps": r["steps"], "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-force/f64-state" if r["precision"] == "fp32" else "f64",
            "data": "synthetic (seeded scenes)",
            "config": {"workload": r["desc"], "n_particles": r["n_particles"],
                       "scenes": r["scenes"], "contacts": r["contacts"],
                       "contact_steps_per_s": ws * r["contact_steps_per_s"],
                       "plain_fp64_scene_by_scene": r["plain_fp64_scene_by_scene"],
                       "speedup_vs_plain": r["speedup_vs_plain"], "autotune": r["tune"],
                       "fp32_error_vs_fp64": r["fp32_error_vs_fp64"],
                       "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "one arena"},
            "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": e2e, "clocks": r["clocks"],
            "gpu_launches": KERNELS_PER_STEP * r["steps"],
        }
        print(json.dumps(line), flush=True)


def main_served(args, lib, ws, rank, dist=None) -> None:
    import torch
    from taichi_dem_julia_port_gb300.serving import (ArenaSizing, Server, poisson_requests,
                                                     sequential_plain)
    reqs = poisson_requests(args.requests, rate=50.0, seed=5)
    sizing = ArenaSizing.from_budget(args.hbm_budget_gb * 1e9)
    for r in reqs:  # request payloads exist before the stream starts
        r.scene()
    clocks = ClockSampler(torch.cuda.current_device())
    with Server(sizing, precision=args.precision or "fp32", chunk_steps=200, lib=lib,
                keep_state=False, policy=args.policy, max_active=args.max_active) as srv:
        if dist:
            dist.barrier()
        clocks.start()
        rep = srv.run(reqs, realtime=True)
        clk = clocks.stop()
    # every rank serves its own copy of the stream: the job ends with the slowest
    makespan = max_over_ranks(rep.makespan_s, dist)
    job_rate = ws * rep.particle_steps / makespan if makespan > 0 else 0.0
    pct = rep.latency_percentiles()
    plain = sequential_plain(reqs, lib=lib)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = oracle_sample([r.make_scene() for r in reqs[:4]], args.cpu_seconds)
    h2d = sum(r.n * 8 * 8 for r in rep.results)  # V, m, pos, vel per particle
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": job_rate, "unit": "particle-steps/s",
            "n_gpus": ws, "steps": rep.launches, "warmup": 0,
            "ms_per_step": 1e3 * rep.makespan_s / max(rep.launches, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-force/f64-state",
            "data": "synthetic (seeded Poisson request stream)",
            "config": {"workload": (f"served: {len(reqs)} requests, Poisson 50/s, 1e3-1e6 spheres "
                                    "log-uniform, 1e3-5e4 steps, mixed bonded/unbonded, "
                                    f"{args.hbm_budget_gb:g} GB HBM budget, continuous batching"),
                       "requests": len(reqs), "latency_p50_s": pct.get("p50"),
                       "latency_p99_s": pct.get("p99"), "makespan_s": rep.makespan_s,
                       "particle_steps": rep.particle_steps,
                       "admissions_deferred": rep.admissions_deferred,
                       "policy": args.policy, "max_active": args.max_active,
                       "arena_slots": sizing.max_particles,
                       "plain_fp64_scene_by_scene": plain,
                       "speedup_vs_plain": rep.throughput / plain["particle_steps_per_s"],
                       "l2": "inputs larger than L2 (no flush)", "parallelism": "one arena"},
            "roofline": None, "cpu_baseline": cpu,
            "e2e": {"value": job_rate, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": int(h2d / max(rep.launches, 1)),
                    "d2h_bytes_per_step": 0,
                    "note": "the served loop is end to end: uploads at admission, device-side "
                            "completion, host bookkeeping; results are step counts and stats"},
            "clocks": clk, "gpu_launches": KERNELS_PER_STEP * rep.launches,
        }
        print(json.dumps(line), flush=True)


def host_link(nbytes: int, reps: int = 20) -> dict:
    """Copy-engine bandwidth of one page-locked buffer of `nbytes` to and from
    the device (CUDA events around `reps` copies): what an exchange of that
    size can reach over this host link."""
    import torch
    n = max(nbytes // 8, 1)
    h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    out = {}
    for name, f in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                    ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            f()
        e1.record()
        torch.cuda.synchronize()
        out[name] = 8 * n * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return out


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """The largest value of x over the ranks (one all-reduce); x itself with
    no process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import OracleScene, host_threads
    if args.workload in ("c4", "c5"):
        if args.workload == "c4":
            scs, _, desc = batched_scenes(args.scenes)
        else:
            from taichi_dem_julia_port_gb300.serving import poisson_requests
            scs = [r.make_scene() for r in poisson_requests(args.requests, seed=5)[:4]]
            desc = f"served request stream ({args.requests} requests), first 4 scenes"
        t_all = time.perf_counter()
        cpu = oracle_sample(scs, max(10.0, 0.5 * args.steps))
        value = cpu["value"]
        line = {
            "impl": "reference", "metric": "particle-steps/s", "value": value,
            "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded scenes)",
            "config": {"workload": desc, "parallelism": "cpu-openmp, scenes in turn",
                       "wall_s": time.perf_counter() - t_all},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "CPU restatement of the reference step on a bounded sample of the scenes",
        }
        print(json.dumps(line), flush=True)
        return
    sc, desc = make_scene(args.workload, args.pour_n)
    threads = host_threads()
    o = OracleScene(sc.cfg, sc.particles, threads=threads)
    if sc.bonded:
        o.initialize()
    o.simulate(args.advance + args.warmup)  # the same timed window as the GPU arm
    t0 = time.perf_counter()
    o.simulate(args.steps)
    dt_s = time.perf_counter() - t0
    value = sc.n * args.steps / dt_s
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value,
        "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lattice)",
        "config": {"workload": desc, "n_particles": sc.n, "parallelism": "cpu-openmp",
                   "timed_window": {"start_step": args.advance + args.warmup + 1,
                                    "steps": args.steps}},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                         "kind": "port",
                         "sample": f"steps {args.advance + args.warmup + 1}-"
                                   f"{args.advance + args.warmup + args.steps} of the full "
                                   "workload (the GPU arm's timed window)"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference step (oracle/dem_oracle.cpp); the reference's "
                "Julia/CUDA.jl GPU path is unavailable (no Julia toolchain, CUDA.jl 4.0 predates sm_103)",
    }
    print(json.dumps(line), flush=True)


def run_proxy(args, sc, flush, advance: int) -> dict:
    """The reference-structured GPU proxy (baseline/refproxy: the reference's
    kernel decomposition, AoS records, BitTables and three host reads per
    step, in plain CUDA C++) on the same scene and window, timed the same way:
    `advance` untimed steps and the same warm-up, then one step at a time
    between L2 flushes, CUDA events."""
    import torch
    from baseline.refproxy import RefProxy
    p = RefProxy(sc.cfg, sc.particles)
    if sc.bonded:
        p.initialize()
    steps = min(args.steps, 500)
    for _ in range(advance + args.warmup):
        p.simulate(1)
    total = 0.0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        total += p.simulate_timed(1)
    p.close()
    ms = total / steps
    return {"value": sc.n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms,
            "steps": steps, "warmup": args.warmup, "start_step": advance + args.warmup,
            "kind": "reference-structured CUDA C++ proxy for the reference's CUDA.jl path "
                    "(AoS 272/136-byte records, BitTables, ~25 launches and 3 device-to-host "
                    "reads per step); the CUDA.jl path itself cannot run on this GPU"}


def snapshot(g) -> dict:
    """A handle's particle and contact state (for restoring a window)."""
    return {"particles": g.particles(forces=False), "contacts": g.contacts()}


def restore(h, snap: dict) -> None:
    """Puts a snapshot into a GPU handle or an oracle scene."""
    p = snap["particles"]
    h.set_particles(pos=p["pos"], vel=p["vel"], omega=p["omega"], quat=p["quat"],
                    wall_shear=p["wall_shear"])
    h.set_contacts(snap["contacts"])


def cpu_baseline(sc, snap: dict, seconds: float, start_step: int) -> dict:
    """The CPU oracle (all host threads) from the timed window's first state,
    for about `seconds`."""
    from oracle.oracle import OracleScene, host_threads
    threads = host_threads()
    o = OracleScene(sc.cfg, sc.particles, threads=threads)
    restore(o, snap)
    o.simulate(1)
    steps, t0 = 0, time.perf_counter()
    while True:
        o.simulate(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 5000:
            break
    return {"value": sc.n * steps / el, "unit": "particle-steps/s", "cores": threads,
            "kind": "port",
            "sample": f"{steps} steps ({el:.1f} s) of the same scene from step {start_step + 1} "
                      "(the timed window's state) on the CPU oracle"}


def wall_contacts(snap: dict) -> int:
    return int(np.count_nonzero(np.any(snap["particles"]["wall_shear"] != 0, axis=1)))


def measure_scene(args, lib, sc, precision: str, steps: int, warmup: int, advance: int, flush,
                  dist=None, ws: int = 1, settling: bool = False, e2e_min_steps: int = 0,
                  profile_steps: int = 20, traffic_key: str = "") -> dict:
    """One scene on a single-scene handle: `advance` untimed steps (past the
    start-up transient, e.g. into a cube's wall impact), `warmup` flushed
    steps, then `steps` timed steps, each after an L2 flush and bracketed by
    CUDA events on the library's stream.  Returns the window's numbers; the
    handle's state at the window's first step is kept (`snap`) so that the
    per-phase profile, the end-to-end loop and the CPU baseline run the same
    window."""
    import torch
    from taichi_dem_julia_port_gb300 import GlobalData
    g = GlobalData(sc.cfg, sc.particles, precision=precision, lib=lib)
    if sc.bonded:
        g.initialize()
    if advance:
        g.simulate(advance)
        g.sync()

    def flushed_step() -> float:
        flush.zero_()
        torch.cuda.synchronize()
        return g.simulate_timed(1)

    for _ in range(warmup):
        flushed_step()
    snap = snapshot(g)
    s0 = g.stats()
    clocks = ClockSampler(torch.cuda.current_device())
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    if getattr(args, "profiler_window", False):
        torch.cuda.cudart().cudaProfilerStart()  # for `ncu --profile-from-start off`
    total_ms, contacts, bonds = 0.0, [], []
    s1 = s0
    for _ in range(steps):
        total_ms += flushed_step()
        s1 = g.stats()
        contacts.append(s1["contacts"])
        bonds.append(s1["bonded"])
    if getattr(args, "profiler_window", False):
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
    # the sampler polls every 20 ms: a short window keeps the same load on
    # (untimed steps) until five samples are in
    pad = 0
    while clocks.count() < 5 and pad < 20000:
        flushed_step()
        pad += 1
    torch.cuda.synchronize()
    clk = clocks.stop()
    clk["padding_steps"] = pad
    if dist:
        dist.barrier()
        total_ms = max_over_ranks(total_ms, dist)
    ms_per_step = total_ms / steps
    window = {"start_step": s0["steps_done"] + 1, "steps": steps,
              "contacts_mean": float(np.mean(contacts)), "bonds_mean": float(np.mean(bonds)),
              "hertz_contacts_mean": float(np.mean(contacts) - np.mean(bonds)),
              "wall_contacts_at_start": wall_contacts(snap),
              "bonds_broken_in_window": s1["bonds_broken"] - s0["bonds_broken"],
              "bonds_broken_total": s1["bonds_broken"],
              "full_searches_in_window": s1["full_searches"] - s0["full_searches"]}
    # per-phase device times over the same window (events between the step's kernels, L2 flushed)
    restore(g, snap)
    phases = []
    for _ in range(profile_steps):
        flush.zero_()
        torch.cuda.synchronize()
        phases.append(g.simulate_profiled())
    ph = {k: float(np.mean([q[k] for q in phases])) for k in phases[0]}
    c_mean, b_mean = window["contacts_mean"], window["bonds_mean"]
    alg = algorithmic_bytes(sc.n, int(round(c_mean)), int(round(b_mean)), settling)
    dom = max(ph, key=ph.get)
    peaks = load_peaks()
    roof = {"bound": "hbm", "kernel": dom, "unit": "GB/s", "peak": peaks["hbm_gbs"],
            "peak_source": peaks["source"], "phase_ms": ph, "algorithmic_bytes": alg[dom],
            "achieved": alg[dom] / (ph[dom] * 1e-3) / 1e9,
            "traffic": ncu_traffic(traffic_key, dom, sc.n)}
    roof["frac"] = roof["achieved"] / peaks["hbm_gbs"]
    if dom == "force":
        # re-reads of particles gathered by more than one contact (L2 hits)
        roof["gather_bytes"] = max(0, 2 * int(round(c_mean)) - sc.n) * GATHER_BYTES_PER_CONTACT_END
    fr = fp64_roofline(dom, precision, sc.n, int(round(b_mean)), ph.get(dom), clk, peaks,
                       "c3" if settling else None, n_hertz=int(round(c_mean - b_mean)))
    if fr:
        roof["fp64_pipe"] = fr
    # every phase's figures (the phases of a step are close in length, so the
    # dominant one alone does not describe the step)
    roof["phases"] = {}
    for k, ms_k in ph.items():
        e = {"ms": ms_k, "algorithmic_bytes": alg.get(k),
             "traffic": ncu_traffic(traffic_key, k, sc.n)}
        if alg.get(k) and ms_k:
            e["achieved_gbs"] = alg[k] / (ms_k * 1e-3) / 1e9
            e["frac_hbm"] = e["achieved_gbs"] / peaks["hbm_gbs"]
        f64 = fp64_roofline(k, precision, sc.n, int(round(b_mean)), ms_k, clk, peaks,
                            "c3" if settling else None, n_hertz=int(round(c_mean - b_mean)))
        if f64:
            e["fp64_frac"] = f64["frac"]
        roof["phases"][k] = e
    out = {"value": ws * sc.n * steps / (total_ms / 1e3), "ms_per_step": ms_per_step,
           "contact_steps_per_s": ws * c_mean * steps / (total_ms / 1e3), "window": window,
           "roofline": roof, "clocks": clk, "snap": snap, "n": sc.n}
    if e2e_min_steps:
        # end to end through the public API with host buffers, on the same
        # window: page-locked state arrays bound to the handle
        # (GlobalData.state_buffers) are uploaded, stepped and read back every
        # step (one dem_step_exchange call); the window is replayed from its
        # first state until at least e2e_min_steps steps are timed
        buf = g.state_buffers()
        h2d = sum(a.nbytes for a in buf.arrays.values())
        reps = max(1, math.ceil(e2e_min_steps / steps))
        e2e_s = 0.0
        for rep_ in range(reps):
            restore(g, snap)
            buf.download()
            torch.cuda.synchronize()
            marked = rep_ == 0 and getattr(args, "profile_e2e", False)
            if marked:
                torch.cuda.cudart().cudaProfilerStart()
            t0 = time.perf_counter()
            for _ in range(steps):
                buf.step(1)  # upload, step, download (dem_step_exchange)
            e2e_s += time.perf_counter() - t0
            if marked:
                torch.cuda.cudart().cudaProfilerStop()
        buf.close()
        e2e_s = max_over_ranks(e2e_s, dist)
        n_e2e = reps * steps
        e2e = {"value": ws * sc.n * n_e2e / e2e_s, "unit": "particle-steps/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(h2d),
               "steps": n_e2e, "window_replays": reps, "ms_per_step": 1e3 * e2e_s / n_e2e}
        link = host_link(int(h2d))
        e2e["host_link"] = link
        # the device step and one copy-engine copy of the state each way, one
        # after the other: what the exchange costs without overlapping the
        # host-link traffic with the step
        e2e["serial_ms_per_step"] = ms_per_step + 1e3 * h2d * (1 / link["h2d_gbs"] +
                                                               1 / link["d2h_gbs"]) / 1e9
        out["e2e"] = e2e
    g.close()
    return out


def pour_summary(args, lib, flush) -> dict:
    """The 2,000,000-sphere pour (FP32 force, dt 2e-7) in two phases: settling
    (the seeded non-overlapping start, free fall: no contacts) and a
    pre-compacted bed of the same spheres with about one contact per sphere
    (scenes.granular_bed)."""
    from taichi_dem_julia_port_gb300 import scenes
    out = {"metric": "particle-steps/s", "precision": "fp32"}
    steps = min(args.steps, args.pour_steps)
    for name, sc, settling in (("settling", scenes.c3(args.pour_n), True),
                               ("bed", scenes.granular_bed(args.pour_n), False)):
        r = measure_scene(args, lib, sc, "fp32", steps, args.warmup, 0, flush,
                          settling=settling, profile_steps=5,
                          traffic_key="c3" if settling else "c3bed")
        out[name] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "steps": steps,
                     "n_particles": sc.n, "contact_steps_per_s": r["contact_steps_per_s"],
                     "window": r["window"], "roofline": r["roofline"]}
    out["workload"] = (f"{args.pour_n:,} spheres, radii lognormal (median 1 mm, sigma 0.25, "
                       "clipped to [0.5, 2] mm), 0.4 x 0.4 m floor, FP32 force / FP64 state, "
                       "dt 2e-7 s; settling: non-overlapping seeded start in 0.4 x 0.4 x 1.2 m "
                       "(no contacts in the window); bed: the same radii stacked in touching "
                       "columns (about one Hertz contact per sphere)")
    return out


def served_summary(args, lib) -> dict:
    """A shortened served stream for the default line: `served_requests`
    Poisson requests (50/s, 1e3-1e6 spheres log-uniform, mixed bonded /
    unbonded) with step counts scaled by `served_steps_scale`, against the
    plain FP64 path scene by scene."""
    import torch
    from taichi_dem_julia_port_gb300.serving import (ArenaSizing, Server, poisson_requests,
                                                     sequential_plain)
    sc = args.served_steps_scale
    reqs = poisson_requests(args.served_requests, rate=50.0, seed=5,
                            smin=max(1, int(1_000 * sc)), smax=max(1, int(50_000 * sc)))
    sizing = ArenaSizing.from_budget(args.hbm_budget_gb * 1e9)
    # each request's payload (its particle arrays) exists before the stream
    # starts, as a client would send it; the plain path is timed without
    # building its scenes either
    for r in reqs:
        r.scene()
    clocks = ClockSampler(torch.cuda.current_device())
    with Server(sizing, precision="fp32", chunk_steps=200, lib=lib, keep_state=False,
                policy=args.policy, max_active=args.max_active) as srv:
        clocks.start()
        rep = srv.run(reqs, realtime=True)
        clk = clocks.stop()
    pct = rep.latency_percentiles()
    plain = sequential_plain(reqs, lib=lib)
    return {"metric": "particle-steps/s", "value": rep.throughput,
            "latency_p50_s": pct.get("p50"), "latency_p99_s": pct.get("p99"),
            "makespan_s": rep.makespan_s, "requests": len(reqs), "time_split": rep.extra,
            "particle_steps": rep.particle_steps, "launches": rep.launches,
            "policy": args.policy, "max_active": args.max_active,
            "plain_fp64_scene_by_scene": plain,
            "speedup_vs_plain": rep.throughput / plain["particle_steps_per_s"],
            "p99_vs_plain": pct.get("p99", 0.0) / plain["p99_s"] if plain["p99_s"] else None,
            "clocks": clk,
            "workload": (f"served: {len(reqs)} Poisson requests (50/s), 1e3-1e6 spheres "
                         "log-uniform, alternately bonded cubes and unbonded pours, step counts "
                         f"uniform in [{int(1_000 * sc)}, {int(50_000 * sc)}] (the served "
                         f"workload's 1,000-50,000 scaled by {sc:g}), FP32 force, "
                         f"{args.hbm_budget_gb:g} GB HBM budget, continuous batching; request "
                         "payloads built before the stream starts")}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c3bed", "c4", "c5"])
    ap.add_argument("--advance", type=int, default=None,
                    help="untimed steps before the warm-up (default: 4,000 for the "
                         "17,576-sphere cube and 2,000 for the 1,000-sphere cube, so the timed "
                         "window lies in the fragmentation after the wall impact; 0 for the pour)")
    ap.add_argument("--scenes", type=int, default=256, help="c4: number of scenes")
    ap.add_argument("--requests", type=int, default=12, help="c5: number of requests")
    ap.add_argument("--hbm-budget-gb", type=float, default=160.0, help="c5: arena budget")
    ap.add_argument("--policy", default="sjf", choices=["fifo", "sjf"],
                    help="c5: admission policy (sjf: least work first, capped active particles)")
    ap.add_argument("--max-active", type=int, default=2_000_000,
                    help="c5 sjf: particles the live scenes may hold before admission waits")
    ap.add_argument("--no-batched", action="store_true",
                    help="default workload: skip the batched summary")
    ap.add_argument("--no-pour", action="store_true", help="default workload: skip the pour")
    ap.add_argument("--no-served", action="store_true",
                    help="default workload: skip the served summary")
    ap.add_argument("--served-requests", type=int, default=100)
    ap.add_argument("--served-steps-scale", type=float, default=0.05)
    ap.add_argument("--pour-steps", type=int, default=50, help="pour summary: timed steps")
    ap.add_argument("--no-tune", action="store_true", help="c4: keep the default launch shape")
    ap.add_argument("--no-plain", action="store_true",
                    help="c4: skip the scene-by-scene plain-path comparison")
    ap.add_argument("--precision", default=None, choices=["fp64", "fp32"])
    ap.add_argument("--pour-n", type=int, default=2_000_000,
                    help="c3: spheres in the pour (smaller pours for profiling captures)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--e2e-steps", type=int, default=500,
                    help="least number of end-to-end steps (the window is replayed)")
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profiler-window", action="store_true",
                    help="mark the timed window with cudaProfilerStart/Stop (for ncu "
                         "--profile-from-start off); the work done is unchanged")
    ap.add_argument("--profile-e2e", action="store_true",
                    help="mark the first pass of the end-to-end loop instead (its "
                         "exchanged steps)")
    ap.add_argument("--no-proxy", action="store_true",
                    help="skip the reference-structured GPU proxy (c1/c2)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.advance is None:
        args.advance = {"c1": 2000, "c2": 4000}.get(args.workload, 0)

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from taichi_dem_julia_port_gb300 import _abi

    lib = _abi.load_library()
    _abi.check(lib, lib.dem_set_device(local), "dem_set_device")
    if args.workload == "c4":
        main_batched(args, lib, ws, rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == "c5":
        main_served(args, lib, ws, rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    sc, desc = make_scene(args.workload, args.pour_n)
    precision = args.precision or ("fp32" if args.workload in ("c3", "c3bed") else "fp64")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    r = measure_scene(args, lib, sc, precision, args.steps, args.warmup, args.advance, flush,
                      dist=dist, ws=ws, settling=args.workload == "c3",
                      e2e_min_steps=args.e2e_steps, profile_steps=args.profile_steps,
                      traffic_key=args.workload)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, r["snap"], args.cpu_seconds, r["window"]["start_step"] - 1)
    proxy = None
    if rank == 0 and args.workload in ("c1", "c2") and not args.no_proxy:
        proxy = run_proxy(args, sc, flush, args.advance)
    extra = {}
    if args.workload == "c2" and rank == 0:
        if not args.no_batched:
            b = run_batched(args, lib, quick=True)
            extra["batched"] = {k: b[k] for k in (
                "desc", "value", "ms_per_step", "steps", "n_particles", "contact_steps_per_s",
                "plain_fp64_scene_by_scene", "speedup_vs_plain", "precision", "tune",
                "fp32_error_vs_fp64")}
            extra["batched"]["phase_ms"] = b["roofline"]["phase_ms"]
            extra["batched"]["metric"] = "particle-steps/s"
        if not args.no_pour:
            extra["pour"] = pour_summary(args, lib, flush)
        if not args.no_served:
            extra["served"] = served_summary(args, lib)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": r["value"], "unit": "particle-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f32-force/f64-state",
            "data": "synthetic (seeded lattice)" if sc.bonded else "synthetic (seeded pour)",
            "config": {"workload": desc, "n_particles": sc.n, "precision": precision,
                       "timed_window": r["window"],
                       "contacts_mean": r["window"]["contacts_mean"],
                       "contact_steps_per_s": r["contact_steps_per_s"],
                       "advance_steps": args.advance,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single scene"},
            "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r.get("e2e"),
            "clocks": r["clocks"], "gpu_launches": KERNELS_PER_STEP * args.steps,
        }
        if proxy:
            line["reference_gpu_proxy"] = proxy
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
