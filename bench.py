"""Benchmark of the GB300 DEM step engine.

Workload (the configuration the headline metric is quoted on): 1,000,000
spheres with lognormal radii (median 1 mm, sigma_log 0.15, clipped to
[0.6, 1.6] mm) poured into a seeded parametric helical chute (radius 0.3 m,
pitch 0.1 m, 3 turns, ~50,000 triangles), Hertz-Mindlin, dt = 1e-6 s, 2,000
timed steps.  The pour itself (a loose lattice above every turn, settled on
the GPU with a larger time step before timing) is part of the setup, not of
the timed region; the timed steps run on the resulting dense bed (about 4.6
contacts per sphere).  Synthetic, seeded inputs; no dataset.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

A "step" is one timestep of the whole scene (contacts, integration, refresh
test and, when triggered on the device, the list rebuild).  `value` is
particle-steps/s with the state resident in HBM; `e2e` is the same metric
through the C ABI with host buffers (state uploaded from pinned host memory
and positions read back every step, inside the timed region).  The
reference arm times the reference algorithm's CPU implementation (the oracle
restatement, OpenMP over all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M spheres, FP32-mixed vs FP64 plain on 1 GB300 (err≤1e-4·r_min)"
# DRAM bytes (read + write) per sphere of one step-kernel launch on the 1M
# poured chute bed, from a one-pass ncu capture of the DRAM byte counters on
# that launch itself (profiles/k_step_mixed_coop_poured_bed_1M_dram.txt);
# scaled by the spheres of a launch
TRAFFIC_POURED_BED_PER_SPHERE = 758_400_000.0 / 999_999
# bytes per sphere of one step-kernel launch on the periodic channel, from an
# ncu capture of the 1M-sphere channel (the 10M one is too large to capture);
# the launch's traffic scales with the spheres it steps
TRAFFIC_CHANNEL_PER_SPHERE = 218_407_936.0 / 1_000_000
UNIT = "particle-steps/s"
METRIC_CHANNEL = "particle-steps/s at 10M spheres in a channel periodic in x, FP32-mixed on 1 GB300"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == "0"] or \
               [[c.strip() for c in r] for r in rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def sort_launches(n_keys):
    """Kernels of one 4-pass radix sort of n_keys keys: upsweep and scatter per
    pass, plus a digit-scan kernel per pass above 32 tiles of 2048 keys."""
    tiles = max(1, -(-n_keys // 2048))
    return 4 * (2 if tiles <= 32 else 3)


def algorithmic_bytes(st, n_active, s=8, s_h=8):
    """Force-kernel bytes per launch: N(S_read+S_write) + 4(2N + sum n_nei +
    sum n_w) + (sum n_c + sum n_wc)(6 s_h + 8), S_read = 24 + 8s, S_write = 24 + 6s.
    With inner rows the step reads those instead of the list rows (sum n_inner
    for sum n_nei, sum n_inner_wall for sum n_w)."""
    s_read = 24 + 6 * s + 2 * s
    s_write = 24 + 6 * s
    inner = st.get("n_inner", 0) > 0
    rows = st["n_inner"] if inner else st["n_nei"]
    wrows = st["n_inner_wall"] if inner else st["n_wall"]
    return (n_active * (s_read + s_write) + 4 * (2 * n_active + rows + wrows)
            + (st["n_contacts"] + st["n_wall_contacts"]) * (6 * s_h + 8))


def aggregate_replicas(ms, n_active, steps, dist=None):
    """Whole-job numbers of N replicas: the slowest rank's time, and the
    particle-steps of all ranks over that time (each rank steps its own
    copy of the workload)."""
    import torch
    work = torch.tensor([float(n_active) * steps], dtype=torch.float64)
    t = torch.tensor([float(ms)], dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(work, op=dist.ReduceOp.SUM)
    ms = float(t.item())
    return ms, float(work.item()) / (ms / 1e3)


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return dist, dist.get_rank(), ws
    return None, 0, 1


def _nvtx(name=None):
    """Open an NVTX range (name) or close the innermost one (None); a no-op
    where NVTX is unavailable."""
    import torch
    try:
        if name is None:
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push(name)
    except Exception:  # noqa: BLE001
        pass


def _time_steps(E, steps, warmup, stream, clk=None, tag="timed"):
    """Warm-up steps, then `steps` steps between two CUDA events on the
    engine's stream.  The timed steps sit in an NVTX range named `tag`, so a
    profiler can be restricted to them (ncu --nvtx --nvtx-include "timed/")."""
    import torch
    E.step(warmup)
    E.sync()
    st0 = E.stats()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if clk is not None:
        clk.__enter__()
    _nvtx(tag)
    start.record(stream)
    E.step(steps)
    stop.record(stream)
    stop.synchronize()
    _nvtx()
    torch.cuda.synchronize()
    if clk is not None:
        clk.__exit__()
    st1 = E.stats()
    return start.elapsed_time(stop), st0, st1


def workload(args):
    """The benchmark scene: the poured chute bed (default), the loose lattice
    over the chute with random velocities (`--workload lattice`), or the
    channel periodic in x over a corrugated floor (`--workload channel`)."""
    from gpudem_gb300 import scenes
    if args.workload == "lattice":
        return scenes.config3_helical_chute(n=args.n, n_tri=args.ntri, v_sigma=args.v_sigma), 0.0
    if args.workload == "channel":
        return scenes.config5_periodic_channel(n=args.n, n_tri=args.ntri, v_sigma=args.v_sigma), 0.0
    t0 = time.time()
    sc = scenes.settle_scene(scenes.config3_chute_pour(n=args.n, n_tri=args.ntri), steps=args.settle_steps)
    return sc, time.time() - t0


def describe(args, sc):
    """(data, workload) strings of the bench line."""
    if args.workload == "channel":
        return ("synthetic (seeded bidisperse spheres on a lattice in a generated channel periodic in x)",
                f"periodic channel 1 m (x, periodic) x 0.5 m, {sc.n} spheres r = 1.0 / 1.5 mm at 70 / 30, "
                f"corrugated floor (amplitude 3 mm) + side walls, {sc.tris.shape[0]} triangles, dt=1e-6 s, "
                f"{args.model} with rolling friction 0.05, {args.precision}, loose lattice, v_sigma "
                f"{args.v_sigma} m/s")
    chute = (f"helical chute, {sc.n} lognormal spheres (median 1 mm, sigma_log 0.15), "
             f"{sc.tris.shape[0]} triangles, dt=1e-6 s, {args.model}, {args.precision}, ")
    if args.workload == "poured":
        return ("synthetic (seeded lognormal spheres poured into a generated helical chute, settled on the GPU "
                "before timing)", chute + f"poured bed (settled {args.settle_steps} steps at dt=2e-5 s, e=0.1)")
    return ("synthetic (seeded lognormal spheres on a lattice over a generated helical chute)",
            chute + f"loose lattice, v_sigma {args.v_sigma} m/s")


def run_engine(args):
    import torch
    from gpudem_gb300 import engine, scenes
    dist, rank, ws = dist_init()
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(lrank)
    sc, pour_s = workload(args)
    kw = dict(model=args.model, reorder=True, nei_capacity=args.nei_cap, steps_per_graph=8,
              skin=args.skin if args.skin > 0 else None, hist_capacity=32,
              bvh_every_step=not args.bvh_once)
    t0 = time.time()
    E = engine.Engine(sc, precision=args.precision, **kw)
    setup_s = time.time() - t0
    stream = torch.cuda.ExternalStream(E.stream())
    if dist:
        dist.barrier()
    clk = Clocks(os.path.join(args.clocks_dir or tempfile.gettempdir(), f"clocks_r{rank}.csv"))
    ms, st0, st1 = _time_steps(E, args.steps, args.warmup, stream, clk)
    ms, value = aggregate_replicas(ms, 0.5 * (st0["n_active"] + st1["n_active"]), args.steps, dist)
    # dominant kernel: the step kernel alone, CUDA events on the engine stream
    _nvtx("profile")
    k_ms = E.profile_step(args.profile_iters)
    _nvtx()
    stk = E.stats()
    # one forced list rebuild (keys, sort, reorder, cells, Verlet and wall
    # lists), CUDA events on the engine stream around the call
    _nvtx("rebuild")
    rb0, rb1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rb0.record(stream)
    E.rebuild()
    rb1.record(stream)
    rb1.synchronize()
    _nvtx()
    rebuild_ms = rb0.elapsed_time(rb1)
    mixed = args.precision == "mixed"
    bytes_launch = algorithmic_bytes(stk, stk["n_active"], s=4 if mixed else 8, s_h=8)
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (k_ms / 1e3) / 1e9
    traffic = args.traffic
    traffic_source = "--traffic" if traffic is not None else None
    if traffic is None and mixed and args.workload == "poured" and args.model == "hertz_mindlin":
        # dram__bytes_read.sum + dram__bytes_write.sum per sphere of one launch
        # on the 1M bed (profiles/k_step_mixed_coop_poured_bed_1M_dram.txt)
        traffic = TRAFFIC_POURED_BED_PER_SPHERE * stk["n_active"]
        traffic_source = ("one-pass ncu capture of the DRAM counters on the 1M bed "
                          "(profiles/k_step_mixed_coop_poured_bed_1M_dram.txt), per sphere times the spheres of "
                          "this launch; not measured in this run")
    if traffic is None and mixed and args.workload == "channel" and args.model == "hertz_mindlin":
        # (profiles/k_step_mixed_coop_channel_1M.txt), scaled to this launch's spheres
        traffic = TRAFFIC_CHANNEL_PER_SPHERE * stk["n_active"]
        traffic_source = ("ncu capture on the 1M channel (profiles/k_step_mixed_coop_channel_1M.txt), scaled by "
                          "the spheres of this launch; not measured in this run")
    reb = int(st1["rebuilds"] - st0["rebuilds"])
    E.close()
    extra = {}
    if not args.bvh_once:
        # context: the same steps with the tree of the static mesh built once
        E1 = engine.Engine(sc, precision=args.precision, **dict(kw, bvh_every_step=False))
        ms1, a0, a1 = _time_steps(E1, max(10, args.steps // 4), args.warmup, torch.cuda.ExternalStream(E1.stream()),
                                  tag="timed_tree_once")
        E1.close()
        extra["value_mesh_tree_built_once"] = 0.5 * (a0["n_active"] + a1["n_active"]) * max(10, args.steps // 4) / (ms1 / 1e3)
    if mixed and not args.no_fp64:
        # the same engine in plain FP64 on the same workload (the ratio's denominator)
        F = engine.Engine(sc, precision="fp64", **kw)
        fstream = torch.cuda.ExternalStream(F.stream())
        fsteps = max(10, args.steps // 4)
        fms, f0, f1 = _time_steps(F, fsteps, args.warmup, fstream, tag="timed_fp64")
        fval = 0.5 * (f0["n_active"] + f1["n_active"]) * fsteps / (fms / 1e3)
        F.close()
        extra.update({"fp64_value": fval, "fp64_steps": fsteps, "mixed_over_fp64": value / fval})
        if args.error_steps > 0:
            extra.update(position_error(sc, kw, args.error_steps))
    if args.workload == "poured" and not args.no_extra:
        extra.update(extra_lines(args, sc, kw, rebuild_ms))
    # end to end through the C ABI with host buffers
    e2e = run_e2e(args, sc, kw) if not args.no_e2e else None
    out = {
        "metric": METRIC if args.workload != "channel" else METRIC_CHANNEL, "value": value, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if mixed else "f64",
        "data": describe(args, sc)[0],
        "config": {"workload": describe(args, sc)[1],
                   "n_particles": args.n, "n_triangles": int(sc.tris.shape[0]), "precision": args.precision,
                   "model": args.model, "l2": "inputs larger than L2 (state + lists > 129 MB per step)",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "mesh_tree": "built once (static mesh)" if args.bvh_once else "rebuilt every step",
                   "rebuilds_in_timed_region": reb, "rebuild_ms": round(rebuild_ms, 3),
                   "setup_s": round(setup_s, 2), "pour_s": round(pour_s, 1),
                   "contacts_per_sphere": round(stk["n_contacts"] / max(stk["n_active"], 1), 3),
                   "wall_contacts_per_sphere": round(stk["n_wall_contacts"] / max(stk["n_active"], 1), 3),
                   **extra},
        "clocks": clk.summary(),
        # one step kernel per step (+ the mesh tree rebuild: keys, 4 sort
        # passes, tree) + the kernels of each list rebuild (keys, 4 sort passes,
        # reorder (+ its inverse order in mixed mode), cell clear, cell ranges,
        # the occupied-cell list (count, scan, emit), Verlet (+ the FP32
        # position copy in FP64 mode), cell wall candidates, walls) + each
        # inner-row build
        "gpu_launches": args.steps * (1 + (0 if args.bvh_once else 2 + sort_launches(int(sc.tris.shape[0]))))
                        + reb * (11 + sort_launches(sc.n))
                        + int(st1["inner_builds"] - st0["inner_builds"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_source,
                     "peak_kind": f"{peak_kind} hbm_gbs",
                     "kernel": f"k_step<{'Mixed' if mixed else 'FP64'},{args.model}>", "kernel_ms": k_ms,
                     "algorithmic_bytes": bytes_launch,
                     "counts": {k: stk[k] for k in ("n_active", "n_nei", "n_inner", "n_wall", "n_inner_wall", "n_contacts",
                                                    "n_wall_contacts")}},
        "e2e": e2e,
        "cpu_baseline": cpu_baseline(args, sc) if (rank == 0 and ws == 1 and not args.no_cpu) else None,
    }
    if rank == 0:
        print(json.dumps(out))


def extra_lines(args, sc, kw, rebuild_ms):
    """Context lines beside the settled-bed value, each on the same engine
    and GPU:
    * the pour itself, with list rebuilds in the timed steps: the chute's
      inlet state poured for `pour_pre_steps` steps at dt = 2e-5 s (e = 0.1),
      then timed at the workload's dt = 1e-6 s, and timed at the pour's own
      dt = 2e-5 s (a list rebuild every few steps);
    * the linear contact law (the reference's only one) in mixed precision and
      in FP64 on the settled bed, the like-for-like partner of the reference
      arm's CPU path;
    * the mixed step scanning the list rows instead of the inner rows, which
      splits the mixed/FP64 ratio into precision and algorithm."""
    import torch
    from dataclasses import replace
    from gpudem_gb300 import engine, scenes
    out = {}

    def timed(scene, precision, steps, tag, **over):
        E = engine.Engine(scene, precision=precision, **dict(kw, **over))
        ms, a0, a1 = _time_steps(E, steps, args.warmup, torch.cuda.ExternalStream(E.stream()), tag=tag)
        E.close()
        n_act = 0.5 * (a0["n_active"] + a1["n_active"])
        return {"value": n_act * steps / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps,
                "rebuilds": int(a1["rebuilds"] - a0["rebuilds"]),
                "inner_builds": int(a1["inner_builds"] - a0["inner_builds"])}

    mid = scenes.settle_scene(scenes.config3_chute_pour(n=args.n, n_tri=args.ntri), steps=args.pour_pre_steps)
    for tag, scene, steps in (("pour_dt1e-6", mid, args.steps),
                              ("pour_dt2e-5", replace(mid, dt=2e-5, e=0.1), max(50, args.steps // 4))):
        r = timed(scene, args.precision, steps, "timed_" + tag)
        # share of the timed region spent in list rebuilds (each as long as
        # the forced rebuild timed on the settled bed)
        r["rebuild_share"] = round(min(1.0, r["rebuilds"] * rebuild_ms / (r["ms_per_step"] * steps)), 4)
        r["state"] = f"chute inlet poured {args.pour_pre_steps} steps at dt=2e-5 s, e=0.1"
        out[tag] = r
    fsteps = max(10, args.steps // 4)
    lin_mixed = timed(sc, "mixed", args.steps, "timed_linear_mixed", model="linear")
    lin_fp64 = timed(sc, "fp64", fsteps, "timed_linear_fp64", model="linear")
    out["linear_model"] = {"mixed_value": lin_mixed["value"], "fp64_value": lin_fp64["value"],
                           "mixed_over_fp64": lin_mixed["value"] / lin_fp64["value"],
                           "note": "the reference's contact law, same bed; the reference arm times it in FP64 on "
                                   "the host cores"}
    if args.precision == "mixed":
        out["mixed_no_inner_value"] = timed(sc, "mixed", max(10, args.steps // 2), "timed_no_inner",
                                            inner_skin=-1.0)["value"]
    return out


def position_error(sc, kw, steps):
    """max |x_mixed - x_fp64| after `steps` steps from the same state."""
    from gpudem_gb300 import engine
    A = engine.Engine(sc, precision="fp64", **kw)
    A.step(steps)
    xa = A.export_positions()
    A.close()
    B = engine.Engine(sc, precision="mixed", **kw)
    B.step(steps)
    xb = B.export_positions()
    B.close()
    e = np.linalg.norm((xa - xb).reshape(-1, 3), axis=1)
    rmin = float(np.min(sc.r))
    return {"pos_err_steps": steps, "pos_err_max_over_rmin": float(e.max() / rmin),
            "pos_err_p9999_over_rmin": float(np.percentile(e, 99.99) / rmin),
            "pos_err_p99_over_rmin": float(np.percentile(e, 99) / rmin),
            "pos_err_median_over_rmin": float(np.median(e) / rmin),
            "pos_err_n_above_1e-4_rmin": int((e > 1e-4 * rmin).sum())}


def run_e2e(args, sc, kw):
    """Same metric through the C ABI with host buffers: the state uploaded from
    host memory, K steps, every step's positions read back into pinned host
    memory (write_frame_bin's frame), all inside the timed region.  Each
    step's copy runs on the engine's copy stream while the next step computes
    (gdem_export_positions_async into two pinned buffers in turn); the last
    synchronise waits for all of them."""
    import torch
    from gpudem_gb300 import engine
    n = sc.n
    steps = max(1, min(args.steps, args.e2e_steps))
    E = engine.Engine(sc, precision=args.precision, **kw)
    frames = [torch.empty(3 * n, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    frame = frames[0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E.import_particles(sc, history=sc.history, hist_stride=sc.hist_stride)
    t_import = time.perf_counter() - t0
    for k in range(steps):
        E.step(1)
        E.export_positions_async(frames[k % 2])
    E.sync()
    dt_s = time.perf_counter() - t0
    E.close()
    h2d = n * (3 * 8 * 3 + 4 * 8 + 4)
    if sc.history is not None:
        h2d += sum(int(np.asarray(a).nbytes) for a in sc.history.values())
    return {"value": n * steps / dt_s, "unit": UNIT, "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": frame.nbytes, "steps": steps, "import_ms": round(1e3 * t_import, 2),
            "total_ms": round(1e3 * dt_s, 2)}


def active_only(sc):
    """The scene without the spheres that have left the box (frozen, never a
    contact partner again), for the CPU path, which takes no activity flags."""
    from dataclasses import replace
    if sc.active is None or bool(np.all(sc.active)):
        return sc
    a = np.asarray(sc.active, bool)
    pick = lambda x: None if x is None else np.asarray(x)[a]
    return replace(sc, x=sc.x[a], r=sc.r[a], m=sc.m[a], k=sc.k[a], eta=sc.eta[a], v=pick(sc.v), w=pick(sc.w),
                   history=None, hist_stride=0, active=None)


def cpu_sample_scene(args, sc):
    """The CPU path's share of the workload: all of it, except for the 10M
    channel, whose full state does not fit the host path's fixed 100-slot
    rows in memory: there the spheres of a tenth of the period (|x| < 5 cm),
    with the whole mesh and the periodic x."""
    from dataclasses import replace
    sc = active_only(sc)
    if args.workload != "channel" or sc.n <= 2_000_000:
        return sc, ""
    a = np.abs(sc.x[:, 0]) < 0.05
    pick = lambda x: None if x is None else np.asarray(x)[a]
    sub = replace(sc, x=sc.x[a], r=sc.r[a], m=sc.m[a], k=sc.k[a], eta=sc.eta[a], v=pick(sc.v), w=pick(sc.w))
    return sub, f"; the {sub.n} spheres with |x| < 5 cm (a tenth of the period), whole mesh"


def cpu_baseline(args, sc):
    """The reference algorithm's CPU implementation on the host cores, on a
    bounded sample of the same workload."""
    try:
        from oracle import port
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                "sample": f"unavailable: {e}"}
    sub, note = cpu_sample_scene(args, sc)
    out = port.time_sample(sub, budget_s=args.cpu_budget)
    out["sample"] += note
    return out


_BED_FIELDS = ("x", "r", "m", "k", "eta", "mu", "dt", "tris", "inlet_lo", "inlet_hi", "g", "v", "w", "skin",
               "refresh", "E", "nu", "e", "mu_roll", "active")


def save_bed(args):
    """Write the workload's scene (the bed the engine arm steps) to
    args.save_bed; run in a process of its own by the reference arm."""
    sc, _ = workload(args)
    np.savez(args.save_bed, **{f: np.asarray(getattr(sc, f)) for f in _BED_FIELDS if getattr(sc, f) is not None})


def load_bed(args):
    """The engine arm's bed, prepared by a separate process (the GPU pour), so
    that the reference arm's own process maps no part of the engine."""
    from gpudem_gb300.scenes import Scene
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bed.npz")
        cmd = [sys.executable, os.path.abspath(__file__), "--save-bed", path, "--workload", args.workload,
               "--n", str(args.n), "--ntri", str(args.ntri), "--settle-steps", str(args.settle_steps),
               "--v-sigma", str(args.v_sigma)]
        subprocess.run(cmd, check=True)
        z = dict(np.load(path))
    scal = {f: float(z[f]) for f in ("mu", "dt", "skin", "refresh", "E", "nu", "e", "mu_roll")}
    return Scene(x=z["x"], r=z["r"], m=z["m"], k=z["k"], eta=z["eta"], tris=z["tris"], inlet_lo=z["inlet_lo"],
                 inlet_hi=z["inlet_hi"], g=z["g"], v=z.get("v"), w=z.get("w"), active=z.get("active"), **scal)


def run_reference(args):
    dist, rank, ws = dist_init()
    if rank != 0:
        return
    # the same bed as the engine arm, poured by the engine on the GPU in a
    # separate process as input preparation; this process runs the CPU path only
    try:
        sc = load_bed(args)
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"bed preparation failed: {e}"}))
        return
    try:
        from oracle import port
        res = port.time_steps(active_only(sc), steps=args.steps, warmup=args.warmup, budget_s=args.cpu_budget)
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"oracle port failed: {e}"}))
        return
    out = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": ws,
           "steps": res["steps"], "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": {"workload": f"helical chute, {args.n} lognormal spheres, {args.workload} "
                                                       f"bed, reference CPU path (linear model), sample"},
           "cpu_baseline": {"value": res["value"], "unit": UNIT, "cores": res["cores"], "kind": "port",
                            "sample": res["sample"]},
           "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_batched(args):
    """Batched ensemble: 256 independent scenes of uneven size packed into one
    engine (one persistent step launch per step, CUDA graphs), against the
    same scenes stepped one by one, each in its own engine.  Both arms run the
    mixed-precision Hertz-Mindlin step with each scene's own friction and
    restitution."""
    import torch
    from gpudem_gb300 import engine, scenes
    dist, rank, ws = dist_init()
    if rank != 0:
        return
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    scs = scenes.config4_batched(n_scenes=args.n_scenes)
    packed, offs, starts = scenes.pack_scenes(scs)
    kw = dict(model="hertz_mindlin", steps_per_graph=8)
    tuned = None
    if args.autotune:
        from gpudem_gb300 import autotune
        t0 = time.time()
        tuned = autotune.autotune(packed, precision=args.precision, model="hertz_mindlin", steps=32, warmup=8)
        kw.update(tuned.settings)
        tune_s = time.time() - t0
    E = engine.Engine(packed, precision=args.precision, **kw)
    stream = torch.cuda.ExternalStream(E.stream())
    clk = Clocks(os.path.join(args.clocks_dir or tempfile.gettempdir(), "clocks_batched.csv"))
    ms, st0, st1 = _time_steps(E, args.steps, args.warmup, stream, clk)
    n_act = 0.5 * (st0["n_active"] + st1["n_active"])
    value = n_act * args.steps / (ms / 1e3)
    reb = int(st1["rebuilds"] - st0["rebuilds"])
    E.close()
    # one by one: each scene in its own engine, timed steps only
    seq_steps = max(10, args.seq_steps)
    seq_ms = 0.0
    seq_ps = 0.0
    for sc in scs:
        Es = engine.Engine(sc, precision=args.precision, **kw)
        sst = torch.cuda.ExternalStream(Es.stream())
        t_ms, a0, a1 = _time_steps(Es, seq_steps, 3, sst)
        seq_ms += t_ms
        seq_ps += 0.5 * (a0["n_active"] + a1["n_active"]) * seq_steps
        Es.close()
    seq_value = seq_ps / (seq_ms / 1e3)
    out = {"metric": f"particle-steps/s, {len(scs)} uneven scenes in one launch (batched) vs one by one",
           "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if args.precision == "mixed" else "f64",
           "data": "synthetic (256 seeded box-drop scenes, config 4 of the benchmark set)",
           "config": {"workload": f"{len(scs)} box-drop scenes, {packed.n} spheres in all (per scene "
                                  f"{min(sc.n for sc in scs)}..{max(sc.n for sc in scs)}), "
                                  f"{packed.tris.shape[0]} triangles in all (per scene "
                                  f"{min(sc.tris.shape[0] for sc in scs)}..{max(sc.tris.shape[0] for sc in scs)}), "
                                  f"hertz_mindlin, per-scene mu and e, {args.precision}",
                      "autotuned": None if tuned is None else {k: (round(v, 7) if isinstance(v, float) else v)
                                                               for k, v in tuned.settings.items()},
                      "autotune_s": None if tuned is None else round(tune_s, 1),
                      "one_by_one_value": seq_value, "one_by_one_steps_per_scene": seq_steps,
                      "batched_over_one_by_one": value / seq_value, "rebuilds_in_timed_region": reb},
           "clocks": clk.summary(),
           "gpu_launches": args.steps + reb * (11 + sort_launches(packed.n))
                           + int(st1["inner_builds"] - st0["inner_builds"])}
    print(json.dumps(out))


def parse_args(argv=None):
    """Command line with the workload-dependent defaults filled in."""
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (2000; 500 for the channel)")
    ap.add_argument("--warmup", type=int, default=40)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=None, help="spheres (1M; 10M for the channel)")
    ap.add_argument("--ntri", type=int, default=None, help="triangles (50k; 200k for the channel)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--model", default="hertz_mindlin", choices=["linear", "hertz_mindlin"])
    ap.add_argument("--error-steps", type=int, default=None,
                    help="steps of the mixed-vs-FP64 position comparison (1000; 500 for the channel)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per step-kernel launch from an ncu capture, if known")
    ap.add_argument("--nei-cap", type=int, default=64)
    ap.add_argument("--skin", type=float, default=-1.0)
    ap.add_argument("--v-sigma", type=float, default=0.5)
    ap.add_argument("--profile-iters", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--workload", default="poured", choices=["poured", "lattice", "batched", "channel"])
    ap.add_argument("--n-scenes", type=int, default=256)
    ap.add_argument("--seq-steps", type=int, default=200)
    ap.add_argument("--autotune", action="store_true",
                    help="batched workload: tune kernel, occupancy, skin, cell size and graph length first")
    ap.add_argument("--bvh-once", action="store_true",
                    help="build the static mesh's tree once instead of in every step (the channel's default)")
    ap.add_argument("--tree-every-step", action="store_true",
                    help="channel: rebuild the static mesh's tree in every step, as the chute workload does")
    ap.add_argument("--settle-steps", type=int, default=12000)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the pour, linear-model and list-row context lines")
    ap.add_argument("--pour-pre-steps", type=int, default=3000,
                    help="steps at dt=2e-5 s from the chute inlet to the pouring state of the pour lines")
    ap.add_argument("--save-bed", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--clocks-dir", default=None,
                    help="where the nvidia-smi clock samples of the timed region go (default: the temp dir)")
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)
    channel = args.workload == "channel"
    # the channel runs 500 steps over a static mesh whose tree is built once;
    # the chute bed 2,000 steps with the tree rebuilt in every step
    if args.steps is None:
        args.steps = 500 if channel else 2000
    if args.error_steps is None:
        args.error_steps = 500 if channel else 1000
    if channel and not args.tree_every_step:
        args.bvh_once = True
    if args.n is None:
        args.n = 10_000_000 if channel else 1_000_000
    if args.ntri is None:
        args.ntri = 200_000 if channel else 50_000
    return args


def main():
    args = parse_args()
    if args.save_bed:
        save_bed(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
