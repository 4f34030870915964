"""Autotuner for a stepping handle (an `Arena` or a `GlobalData`).

Picks the search-cell factor (arenas) and the launch shape of the grid-stride
kernels (contact forces, integration) by timing real steps
on the live workload with CUDA events.  None of these knobs changes a result:
the search grid only changes which buckets the pair search visits (contact
ends follow the reference's cells), and every kernel computes the same values
for any launch shape; the arena tests check both bit for bit.  The steps taken
while tuning are ordinary simulation steps.

The search is coordinate descent: cell factor first, then the force kernel's
block and grid, then the integration block, the FP32
force kernel's register budget, the launch mode (ordinary or programmatic
dependent launches) and the pair search's register budget; each
candidate is timed over `steps` steps after one untimed step.  The run moves
on while candidates are timed, so the choice is confirmed at the end: the
chosen and the starting settings are timed alternately (`confirm_rounds`
times each) and the faster is kept.
"""
from __future__ import annotations

from dataclasses import dataclass, field

CELL_FACTORS = (1.0, 0.8, 0.6, 0.45, 0.35)
BLOCKS = (64, 128, 256)
GRIDS_PER_SM = (4, 8, 16, 32)
INTEGRATE_BLOCKS = (32, 64, 128, 256)
DETECT_BLOCKS = (3, 4)  # pair-search register budget (blocks per SM)
DEPENDENT = (0, 1, 2)   # ordinary / programmatic dependent launches (2: early trigger)
FORCE_BLOCKS = (0, 4)   # FP32 force kernel register budget (0: compiler's choice)


@dataclass
class TuneResult:
    cell_factor: float | None
    shape: dict
    ms_per_step: float
    trials: list = field(default_factory=list)

    def as_dict(self) -> dict:
        return {"cell_factor": self.cell_factor, "shape": self.shape,
                "ms_per_step": self.ms_per_step, "trials": len(self.trials)}


def _time(target, steps: int) -> float:
    target.step(1) if hasattr(target, "step") else target.simulate(1)
    t = target.step_timed(steps) if hasattr(target, "step_timed") else \
        target.simulate_timed(steps)
    return t / steps


def autotune(target, sm_count: int = 152, steps: int = 10, cell_factors=CELL_FACTORS,
             blocks=BLOCKS, grids_per_sm=GRIDS_PER_SM,
             integrate_blocks=INTEGRATE_BLOCKS, detect_blocks=DETECT_BLOCKS,
             force_blocks=FORCE_BLOCKS, dependent=DEPENDENT,
             confirm_rounds: int = 3) -> TuneResult:
    """Tunes `target` in place and returns the chosen settings."""
    trials = []
    is_arena = hasattr(target, "set_cell_factor")
    best_cf = None
    start_cf = 1.0 if is_arena else None
    start_shape = target.launch_shape()
    best = _time(target, steps)
    trials.append(({"baseline": True}, best))
    if is_arena:
        best_cf = 1.0
        for cf in cell_factors:
            target.set_cell_factor(cf)
            t = _time(target, steps)
            trials.append(({"cell_factor": cf}, t))
            if t < best:
                best, best_cf = t, cf
        target.set_cell_factor(best_cf)
    shape = target.launch_shape()
    for fb in blocks:
        for g in grids_per_sm:
            cand = dict(shape, force_block=fb, force_grid=g * sm_count)
            target.set_launch_shape(**cand)
            t = _time(target, steps)
            trials.append((cand, t))
            if t < best:
                best, shape = t, cand
    for ib in integrate_blocks:
        cand = dict(shape, integrate_block=ib)
        target.set_launch_shape(**cand)
        t = _time(target, steps)
        trials.append((cand, t))
        if t < best:
            best, shape = t, cand
    for fb in force_blocks:
        cand = dict(shape, force_blocks_per_sm=fb)
        target.set_launch_shape(**cand)
        t = _time(target, steps)
        trials.append((cand, t))
        if t < best:
            best, shape = t, cand
    for dl in dependent:
        cand = dict(shape, dependent_launch=dl)
        target.set_launch_shape(**cand)
        t = _time(target, steps)
        trials.append((cand, t))
        if t < best:
            best, shape = t, cand
    for db in detect_blocks:
        cand = dict(shape, detect_blocks_per_sm=db)
        target.set_launch_shape(**cand)
        t = _time(target, steps)
        trials.append((cand, t))
        if t < best:
            best, shape = t, cand
    # the run moves on while the candidates are timed (cubes reach their walls,
    # contacts form), so the choice is confirmed against the starting settings
    # on one stretch of the run, the two alternating
    if confirm_rounds <= 0:
        target.set_launch_shape(**shape)
        return TuneResult(best_cf, shape, best, trials)
    t_new = t_start = 0.0
    for _ in range(confirm_rounds):
        _apply(target, start_cf, start_shape, is_arena)
        t_start += _time(target, steps)
        _apply(target, best_cf, shape, is_arena)
        t_new += _time(target, steps)
    trials.append(({"confirm": True, "start": t_start, "chosen": t_new}, t_new / confirm_rounds))
    if t_start < t_new:
        best_cf, shape, best = start_cf, start_shape, t_start / confirm_rounds
        _apply(target, best_cf, shape, is_arena)
    else:
        best = t_new / confirm_rounds
    return TuneResult(best_cf, shape, best, trials)


def _apply(target, cell_factor, shape, is_arena) -> None:
    if is_arena and cell_factor is not None:
        target.set_cell_factor(cell_factor)
    target.set_launch_shape(**shape)
