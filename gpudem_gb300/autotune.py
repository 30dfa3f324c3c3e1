"""Autotuner for the step engine.

Picks, for one scene, the mixed-precision step kernel and the occupancy it is
compiled for (the block configuration), the Verlet skin (which sets the list
cutoff and, through the refresh threshold skin/2, the rebuild cadence), the
cell size, the inner skin (the rows the step scans and their rebuild cadence),
and the number of steps per CUDA-graph launch, by timing short runs of each
candidate on the GPU.  The skin, cell size and graph length leave the
trajectory unchanged: the lists only decide which pairs are tested, the
contact set is the same while they are valid, and forces are summed in
partner-pId order whatever the storage order.  The kernel variants compute
the same contact law with the same FP32 operations (their trajectories are
bit-identical on the GPU).  So the choice is about speed alone.

The search is greedy, one parameter at a time in the order above, each stage
keeping the best setting of the stages before it.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

# (mixed_kernel, occupancy): warp-cooperative at 4/5/6 CTAs per SM,
# warp-staged, one thread per particle at 2/3 CTAs per SM
KERNELS = [(1, 4), (1, 5), (1, 6), (2, 0), (3, 2), (3, 3)]
SKIN_FACTORS = [0.5, 1.0, 1.5]          # x r_max
INNER_FACTORS = [0.05, 0.1, 0.2]        # x r_max (at most the skin)
GRAPH_STEPS = [4, 8, 16]


@dataclass
class Tuning:
    settings: dict
    ms_per_step: float
    trials: list = field(default_factory=list)   # (settings, ms_per_step)


def time_settings(scene, settings: dict, steps: int, warmup: int, base: dict) -> float:
    """ms per step of `scene` under `settings` (wall clock around `steps`
    steps after `warmup`, device synchronised on both sides)."""
    from .engine import Engine
    E = Engine(scene, **base, **settings)
    try:
        E.step(warmup)
        E.sync()
        t0 = time.perf_counter()
        E.step(steps)
        E.sync()
        return 1e3 * (time.perf_counter() - t0) / steps
    finally:
        E.close()


def candidate_stages(scene, precision: str):
    """The stages of the greedy search: lists of partial settings."""
    rmax = float(np.max(scene.r))
    stages = []
    if precision == "mixed":
        stages.append([dict(mixed_kernel=k, occupancy=o) for k, o in KERNELS])
    skins = [f * rmax for f in SKIN_FACTORS]
    # FP64 keeps the reference's cell of at least 4 r_max (its keys and order);
    # mixed mode takes the smallest cell the scan allows
    cell = (lambda s: 2.0 * rmax + s) if precision == "mixed" else (lambda s: max(4.0 * rmax, 2.0 * rmax + s))
    stages.append([dict(skin=s, cell_size=cell(s)) for s in skins])
    if precision == "mixed":
        stages.append([dict(inner_skin=f * rmax) for f in INNER_FACTORS])
    stages.append([dict(steps_per_graph=k) for k in GRAPH_STEPS])
    return stages


def search(stages, measure, start: dict | None = None) -> Tuning:
    """Greedy search over `stages` with `measure(settings) -> ms/step`."""
    best = dict(start or {})
    trials = []
    best_ms = None
    for options in stages:
        stage_best, stage_ms = None, None
        for opt in options:
            cand = {**best, **opt}
            ms = measure(cand)
            trials.append((cand, ms))
            if stage_ms is None or ms < stage_ms:
                stage_best, stage_ms = cand, ms
        best, best_ms = stage_best, stage_ms
    return Tuning(settings=best, ms_per_step=best_ms, trials=trials)


def autotune(scene, precision="mixed", model="hertz_mindlin", steps=64, warmup=8, log=None, **engine_kw) -> Tuning:
    """Tune the engine for `scene`; returns the best settings (keyword
    arguments of Engine), their ms per step and every trial."""
    base = dict(precision=precision, model=model, **engine_kw)

    def measure(settings):
        ms = time_settings(scene, settings, steps, warmup, base)
        if log is not None:
            log(f"autotune {settings}: {ms:.4f} ms/step")
        return ms

    return search(candidate_stages(scene, precision), measure)
