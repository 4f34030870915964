#!/usr/bin/env python
"""DEM step throughput on GB300 (one JSON line on stdout).

Workload (default): the 17,576-sphere bonded-cube impact — 26x26x26 simple
cubic lattice, radius 0.01 m ±5 %, 50,700 EBPM bonds, 20 m/s toward a rigid
plane, FP64, dt = 1e-6 s.  One "step" is one DEM time step (`simulate!`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Our arm: W untimed steps, then K steps each timed with CUDA events on the
library's stream, with a 256 MiB write between steps to flush L2 (the scene
itself fits in L2).  value = particle-steps/s over all ranks (max time over
ranks).  `e2e` repeats the metric through the C ABI with host buffers: every
step uploads the particle state from host memory (dem_set_particles), steps,
and reads it back (dem_get_particles).  `roofline` reports the dominant kernel
from per-phase CUDA events (dem_step_profiled).  `cpu_baseline` times the CPU
oracle (OpenMP, all host threads) on a bounded sample of the same workload.

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

# Algorithmic bytes of the force kernel per contact, from its SoA field list
# (k_force in dem_kernels.cu): contact ids + flags (12 B), particle gathers of
# i and j (pos, vel, ω, r, m: 2 × 88 B), contact state read (bond: 𝐅, 𝛕ᵢ, 𝛕ⱼ 72 B;
# Hertz: 𝐬 24 B), state write (bond: 𝐤, 𝐅, 𝛕ᵢ, 𝛕ⱼ, 𝐬 120 B; Hertz: 𝐤, 𝐅, 𝐬 72 B),
# force contributions (9 × 8 B).
FORCE_BYTES_BOND = 12 + 176 + 72 + 120 + 72
FORCE_BYTES_HERTZ = 12 + 176 + 24 + 72 + 72
# Algorithmic bytes of the other phases per particle / per contact
BROADPHASE_BYTES_PER_PARTICLE = 24 + 16 + 4 + 4 + 4 + 8 + 24 + 8 + 32 + 16  # hash..canon
INTEGRATE_BYTES_PER_PARTICLE = 13 * 8 * 2 + 4 * 8 + 6 * 8 + 3 * 8 * 2 + 8 + 4  # state r/w
KERNELS_PER_STEP = 8  # hash, scan, scatter, canon, detect, compact, force, integrate
L2_FLUSH_BYTES = 256 << 20


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
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
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

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


def make_scene(name: str):
    from taichi_dem_julia_port_gb300 import scenes
    if name == "c1":
        return scenes.c1(), "bonded cube 10^3 = 1,000 spheres, -10 m/s, FP64, dt 1e-6"
    if name == "c2":
        return scenes.c2(), "bonded cube 26^3 = 17,576 spheres, 20 m/s, FP64, dt 1e-6"
    if name == "c3":
        return scenes.c3(), "unbonded pour 2,000,000 spheres, FP32 force, dt 2e-7"
    raise ValueError(name)


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
    sc, desc = make_scene(args.workload)
    threads = host_threads()
    o = OracleScene(sc.cfg, sc.particles, threads=threads)
    if sc.bonded:
        o.initialize()
    o.simulate(args.warmup)
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
        "config": {"workload": desc, "n_particles": sc.n, "parallelism": "cpu-openmp"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{args.steps} steps of the full workload after {args.warmup} warm-up steps"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference step (oracle/dem_oracle.cpp); the reference's "
                "Julia/CUDA.jl GPU path is unavailable (no Julia toolchain, CUDA.jl 4.0 predates sm_103)",
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(sc, seconds: float) -> dict:
    from oracle.oracle import OracleScene, host_threads
    threads = host_threads()
    o = OracleScene(sc.cfg, sc.particles, threads=threads)
    if sc.bonded:
        o.initialize()
    o.simulate(2)
    steps, t0 = 0, time.perf_counter()
    while True:
        o.simulate(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 5000:
            break
    return {"value": sc.n * steps / el, "unit": "particle-steps/s", "cores": threads,
            "kind": "port",
            "sample": f"{steps} steps ({el:.1f} s) of the same scene from t=0 on the CPU oracle"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3"])
    ap.add_argument("--precision", default=None, choices=["fp64", "fp32"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

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

    from taichi_dem_julia_port_gb300 import GlobalData, _abi

    lib = _abi.load_library()
    _abi.check(lib, lib.dem_set_device(local), "dem_set_device")
    sc, desc = make_scene(args.workload)
    precision = args.precision or ("fp32" if args.workload == "c3" else "fp64")
    g = GlobalData(sc.cfg, sc.particles, precision=precision)
    if sc.bonded:
        g.initialize()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flushed_step() -> float:
        flush.zero_()
        torch.cuda.synchronize()
        return g.simulate_timed(1)

    for _ in range(args.warmup):
        flushed_step()
    contacts = []
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        total_ms += flushed_step()
        contacts.append(g.stats()["contacts"])
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    g.sync()
    ms_per_step = total_ms / args.steps
    value = ws * sc.n * args.steps / (total_ms / 1e3)
    mean_c = float(np.mean(contacts))
    stats = g.stats()

    # per-phase device times (eager launches, L2 flushed before each step)
    phases = []
    for _ in range(args.profile_steps):
        flush.zero_()
        torch.cuda.synchronize()
        phases.append(g.simulate_profiled())
    ph = {k: float(np.mean([p[k] for p in phases])) for k in phases[0]}
    st = g.stats()
    c_now = st["contacts"]
    n_bond = st["bonded"]
    force_bytes = n_bond * FORCE_BYTES_BOND + (c_now - n_bond) * FORCE_BYTES_HERTZ
    alg = {"force": force_bytes,
           "broadphase": sc.n * BROADPHASE_BYTES_PER_PARTICLE,
           "integrate": sc.n * INTEGRATE_BYTES_PER_PARTICLE}
    dom = max(ph, key=ph.get)
    dom_bytes = alg.get(dom)
    peaks = load_peaks()
    roofline = {"bound": "hbm", "kernel": dom, "unit": "GB/s",
                "peak": peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": None, "phase_ms": ph}
    if dom_bytes is not None:
        ach = dom_bytes / (ph[dom] * 1e-3) / 1e9
        roofline.update({"achieved": ach, "frac": ach / peaks["hbm_gbs"],
                         "algorithmic_bytes": dom_bytes})
    else:
        roofline.update({"achieved": None, "frac": None})

    # e2e through the C ABI with host buffers
    st0 = g.particles(forces=False)
    keys = ("pos", "vel", "omega", "quat", "wall_shear")
    host = {k: np.ascontiguousarray(st0[k]) for k in keys}
    h2d = sum(host[k].nbytes for k in keys)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        g.set_particles(**host)
        g.simulate(1)
        out = g.particles(forces=False)
        host = {k: out[k] for k in keys}
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": ws * sc.n * args.e2e_steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(h2d),
           "steps": args.e2e_steps, "ms_per_step": 1e3 * e2e_s / args.e2e_steps}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f32-force/f64-state",
            "data": "synthetic (seeded lattice)",
            "config": {"workload": desc, "n_particles": sc.n, "contacts_mean": mean_c,
                       "contact_steps_per_s": ws * mean_c * args.steps / (total_ms / 1e3),
                       "bonds_broken": stats["bonds_broken"], "precision": precision,
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single scene"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": KERNELS_PER_STEP * args.steps,
        }
        print(json.dumps(line), flush=True)
    g.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
