"""Benchmark of the GB300 DEM step engine.

Workload (the configuration the headline metric is quoted on): 1,000,000
spheres with lognormal radii (median 1 mm, sigma_log 0.15, clipped to
[0.6, 1.6] mm) over a seeded parametric helical chute (radius 0.3 m, pitch
0.1 m, ~50,000 triangles), dt = 1e-6 s.  Synthetic, seeded inputs; no dataset.

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
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M spheres, FP32-mixed vs FP64 plain on 1 GB300 (err≤1e-4·r_min)"
UNIT = "particle-steps/s"


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


def algorithmic_bytes(st, n_active, s=8, s_h=8):
    """Force-kernel bytes per launch: N(S_read+S_write) + 4(2N + sum n_nei +
    sum n_w) + (sum n_c + sum n_wc)(6 s_h + 8), S_read = 24 + 8s, S_write = 24 + 6s."""
    s_read = 24 + 6 * s + 2 * s
    s_write = 24 + 6 * s
    return (n_active * (s_read + s_write) + 4 * (2 * n_active + st["n_nei"] + st["n_wall"])
            + (st["n_contacts"] + st["n_wall_contacts"]) * (6 * s_h + 8))


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return dist, dist.get_rank(), ws
    return None, 0, 1


def _time_steps(E, steps, warmup, stream, clk=None):
    import torch
    E.step(warmup)
    E.sync()
    st0 = E.stats()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if clk is not None:
        clk.__enter__()
    start.record(stream)
    E.step(steps)
    stop.record(stream)
    stop.synchronize()
    torch.cuda.synchronize()
    if clk is not None:
        clk.__exit__()
    st1 = E.stats()
    return start.elapsed_time(stop), st0, st1


def run_engine(args):
    import torch
    from gpudem_gb300 import engine, scenes
    dist, rank, ws = dist_init()
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(lrank)
    sc = scenes.config3_helical_chute(n=args.n, n_tri=args.ntri, v_sigma=args.v_sigma)
    kw = dict(model=args.model, reorder=True, nei_capacity=args.nei_cap, steps_per_graph=8,
              skin=args.skin if args.skin > 0 else None)
    t0 = time.time()
    E = engine.Engine(sc, precision=args.precision, **kw)
    setup_s = time.time() - t0
    stream = torch.cuda.ExternalStream(E.stream())
    if dist:
        dist.barrier()
    out_dir = os.path.join(ROOT, "gpurun_out") if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else "/tmp"
    clk = Clocks(os.path.join(out_dir, f"clocks_r{rank}.csv"))
    ms, st0, st1 = _time_steps(E, args.steps, args.warmup, stream, clk)
    if dist:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    n_act = 0.5 * (st0["n_active"] + st1["n_active"])
    value = n_act * args.steps * ws / (ms / 1e3)
    # dominant kernel: the step kernel alone, CUDA events on the engine stream
    k_ms = E.profile_step(args.profile_iters)
    stk = E.stats()
    mixed = args.precision == "mixed"
    bytes_launch = algorithmic_bytes(stk, stk["n_active"], s=4 if mixed else 8, s_h=8)
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (k_ms / 1e3) / 1e9
    reb = int(st1["rebuilds"] - st0["rebuilds"])
    E.close()
    extra = {}
    if mixed and not args.no_fp64:
        # the same engine in plain FP64 on the same workload (the ratio's denominator)
        F = engine.Engine(sc, precision="fp64", **kw)
        fstream = torch.cuda.ExternalStream(F.stream())
        fsteps = max(10, args.steps // 4)
        fms, f0, f1 = _time_steps(F, fsteps, args.warmup, fstream)
        fval = 0.5 * (f0["n_active"] + f1["n_active"]) * fsteps / (fms / 1e3)
        F.close()
        extra = {"fp64_value": fval, "fp64_steps": fsteps, "mixed_over_fp64": value / fval}
        if args.error_steps > 0:
            extra.update(position_error(sc, kw, args.error_steps))
    # end to end through the C ABI with host buffers
    e2e = run_e2e(args, sc, kw) if not args.no_e2e else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if mixed else "f64",
        "data": "synthetic (seeded lognormal spheres on a lattice over a generated helical chute)",
        "config": {"workload": f"helical chute, {args.n} lognormal spheres (median 1 mm, sigma_log 0.15), "
                               f"{sc.tris.shape[0]} triangles, dt=1e-6 s, {args.model}, {args.precision}",
                   "n_particles": args.n, "n_triangles": int(sc.tris.shape[0]), "precision": args.precision,
                   "model": args.model, "l2": "inputs larger than L2 (state + lists > 129 MB per step)",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "rebuilds_in_timed_region": reb, "setup_s": round(setup_s, 2), **extra},
        "clocks": clk.summary(),
        # one step kernel per step + the rebuild kernels of each rebuild
        # (keys, 4 x 3 sort passes, reorder, cell clear, cell ranges, Verlet, walls)
        # (+ the FP32 position copy of the FP64 mode's list prefilter)
        "gpu_launches": args.steps + reb * (18 if mixed else 19),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": args.traffic,
                     "peak_kind": f"{peak_kind} hbm_gbs",
                     "kernel": f"k_step<{'Mixed' if mixed else 'FP64'},{args.model}>", "kernel_ms": k_ms,
                     "algorithmic_bytes": bytes_launch,
                     "counts": {k: stk[k] for k in ("n_active", "n_nei", "n_wall", "n_contacts",
                                                    "n_wall_contacts")}},
        "e2e": e2e,
        "cpu_baseline": cpu_baseline(args, sc) if (rank == 0 and ws == 1 and not args.no_cpu) else None,
    }
    if rank == 0:
        print(json.dumps(out))


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
    host memory, K steps, positions read back into pinned host memory every
    step (write_frame_bin's frame), all inside the timed region."""
    import torch
    from gpudem_gb300 import engine
    n = sc.n
    steps = max(1, min(args.steps, args.e2e_steps))
    E = engine.Engine(sc, precision=args.precision, **kw)
    frame = torch.empty(3 * n, dtype=torch.float64).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E.import_particles(sc)
    for _ in range(steps):
        E.step(1)
        E.export_positions(out=frame)
    E.sync()
    dt_s = time.perf_counter() - t0
    E.close()
    h2d = n * (4 * 8 * 3 + 4 * 8)
    return {"value": n * steps / dt_s, "unit": UNIT, "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": frame.nbytes, "steps": steps}


def cpu_baseline(args, sc):
    """The reference algorithm's CPU implementation on the host cores, on a
    bounded sample of the same workload."""
    try:
        from oracle import port
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                "sample": f"unavailable: {e}"}
    return port.time_sample(sc, budget_s=args.cpu_budget)


def run_reference(args):
    dist, rank, ws = dist_init()
    if rank != 0:
        return
    from gpudem_gb300 import scenes
    sc = scenes.config3_helical_chute(n=args.n, n_tri=args.ntri, v_sigma=args.v_sigma)
    try:
        from oracle import port
        res = port.time_steps(sc, steps=args.steps, warmup=args.warmup, budget_s=args.cpu_budget)
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"oracle port failed: {e}"}))
        return
    out = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": ws,
           "steps": res["steps"], "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": {"workload": f"helical chute, {args.n} lognormal spheres, "
                                                       f"reference CPU path (linear model), sample"},
           "cpu_baseline": {"value": res["value"], "unit": UNIT, "cores": res["cores"], "kind": "port",
                            "sample": res["sample"]},
           "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=40)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--ntri", type=int, default=50_000)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--model", default="hertz_mindlin", choices=["linear", "hertz_mindlin"])
    ap.add_argument("--error-steps", type=int, default=1000)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per step-kernel launch from an ncu capture, if known")
    ap.add_argument("--nei-cap", type=int, default=64)
    ap.add_argument("--skin", type=float, default=-1.0)
    ap.add_argument("--v-sigma", type=float, default=0.5)
    ap.add_argument("--profile-iters", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
