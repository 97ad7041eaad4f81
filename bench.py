"""Throughput benchmark of the DE timestep: cell-steps/s on one GB300.

Workload (one "step" = one full DE1 RK2 timestep of the whole mesh):
inflow_bumps, a 1000 x 1000 rectangular cross mesh (4.0M triangles) over
10 km x 10 km, slope + 64 Gaussian bumps (~30% dry), Dirichlet 2 m inflow west,
transmissive east, reflective north/south, Manning U(0.02, 0.06).  Synthetic
seeded data (workloads.inflow_bumps).  The state (>1 GB) is far larger than
the 129 MB L2, so no explicit flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU oracle (the restated reference algorithm,
OpenMP over all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT]

METRIC = "cell-steps/s (plain FP64 vs batched mixed) + p50/p99 latency @<=1 mm depth error"
UNIT = "cell-steps/s"

# Compulsory HBM bytes per cell per DE1 step of the ideal fused kernel
# (every array read or written once; neighbour gathers served on chip).
ALG_BYTES_PER_CELL_STEP = {"fp64": 488.0, "mixed": 352.0}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during timing."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(m, precision):
    from anuga_core_gb300 import workloads
    d = workloads.inflow_bumps(m=m, precision=precision)
    return d


def cpu_baseline(m, steps, threads):
    """Oracle (restated reference, OpenMP) on the same workload: `steps` DE1
    steps of the full mesh after one warm-up step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from anuga_core_gb300 import workloads
    d = workloads.inflow_bumps(m=m)
    oracle.build()
    oracle.set_threads(threads)
    oracle.set_parallel_extrapolation(True)
    od = oracle.OracleDomain(d.mesh, "DE1")
    Q = d.quantities
    od.set_centroid_state(Q["stage"].centroid_values, Q["xmomentum"].centroid_values,
                          Q["ymomentum"].centroid_values, Q["elevation"].centroid_values,
                          Q["friction"].centroid_values)
    kinds = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    od.set_boundaries([(d.mesh.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in d.mesh.tag_boundary_cells])
    gen = od.evolve(yieldstep=1e9, finaltime=None, max_steps=steps + 1)
    next(gen)                      # initial distribute
    od.relative_yieldtime = 1e300
    od.relative_finaltime = None
    od.rk2_step(1e300, None)       # warm-up step
    t0 = time.perf_counter()
    for _ in range(steps):
        od.rk2_step(1e300, None)
        od.relative_time += od.timestep
    el = time.perf_counter() - t0
    N = len(d.mesh)
    return {"value": N * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d DE1 steps of the %d-triangle inflow_bumps mesh (%.1f s)" % (steps, N, el)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per_step = []
    base = None
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(args.m, args.cpu_steps, threads)
        if i >= args.warmup:
            per_step.append(r["value"])
        base = r
    v = float(np.median(per_step)) if per_step else base["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * (4 * args.m * args.m) / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "inflow_bumps %dx%d rectangular cross (%d triangles), DE1 RK2" %
                       (args.m, args.m, 4 * args.m * args.m), "l2": "inputs larger than L2"},
            "cpu_baseline": dict(base, value=v),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--m", type=int, default=1000, help="mesh side (4*m*m triangles)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-steps", type=int, default=3, dest="cpu_steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="inflow_bumps", choices=["inflow_bumps", "batch"],
                    help="inflow_bumps: one 4M-triangle mesh; batch: 256 scenarios (~20M triangles) in one pool")
    ap.add_argument("--batch-count", type=int, default=256, dest="batch_count")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from anuga_core_gb300 import _lib
    if args.workload == "batch":
        return run_batch(args, torch, rank, world, local, dist)
    d = build_workload(args.m, args.precision)
    N = len(d)
    d.distribute_to_vertices_and_edges()
    scn = d._scn
    stream = torch.cuda.Stream()          # a real stream: the legacy default one has handle 0
    torch.cuda.set_stream(stream)
    scn.set_stream(stream.cuda_stream)
    tune = None
    if args.precision == "mixed":
        from anuga_core_gb300.autotune import tune_pool
        res, best = tune_pool(scn.pool, steps=5, reps=2)
        tune = {"chosen": best, "s_per_step": res}
    d.advance_steps(args.warmup)
    launches0 = _lib.kernel_launches()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    st = d.advance_steps(args.steps)
    e1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    launches = _lib.kernel_launches() - launches0
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * N * args.steps / (ms / 1e3)

    # per-kernel event timing (direct launches) for the roofline
    phases = scn.time_phases(reps=3)
    step_ms = sum(phases.values())
    dominant = max(phases, key=phases.get)
    hbm, peak_kind = _peaks()
    alg_bytes_step = ALG_BYTES_PER_CELL_STEP[args.precision] * N
    achieved_step = alg_bytes_step / (ms_per_step / 1e3) / 1e9

    # e2e: through the C ABI with host buffers, copies inside the timed region
    pin = {f: torch.empty(N, dtype=torch.float64, pin_memory=True).numpy() for f in ("stage_c", "xmom_c", "ymom_c")}
    for f in pin:
        scn.get(f, out=pin[f])
    d.relative_yieldtime = float("inf")
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    barrier()
    e2.record(stream)
    for _ in range(args.steps):
        for f in pin:
            scn.set(f, pin[f])
        scn.set_clock(d.relative_time, 1e300, -1.0)
        scn.advance(1)
        for f in pin:
            scn.get(f, out=pin[f])
    e3.record(stream)
    barrier()
    e2e_ms = e2.elapsed_time(e3)
    e2e_value = world * N * args.steps / (e2e_ms / 1e3)

    if rank == 0:
        cpu = None
        if not args.no_cpu and world == 1:
            cpu = cpu_baseline(args.m, args.cpu_steps, os.cpu_count() or 1)
        dom_ms = phases[dominant]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32 flux / f64 accumulate",
            "data": "synthetic",
            "config": {"workload": "inflow_bumps %dx%d rectangular cross (%d triangles), DE1 RK2, %s" %
                       (args.m, args.m, N, args.precision), "cells": N, "precision": args.precision,
                       "l2": "inputs larger than L2 (state %.0f MB)" % (scn_bytes(d) / 1e6),
                       "parallelism": "replicas" if world > 1 else "single", "autotune": tune},
            "roofline": {"bound": "hbm", "achieved": achieved_step, "peak": hbm, "unit": "GB/s",
                         "frac": achieved_step / hbm, "peak_kind": peak_kind,
                         "traffic": None, "kernel": "whole step (%s dominant: %.1f%% of step time)" %
                         (dominant, 100.0 * dom_ms / max(step_ms, 1e-9)),
                         "phase_ms": phases,
                         "note": "achieved = %d algorithmic B/cell-step x cells / step time" %
                         ALG_BYTES_PER_CELL_STEP[args.precision]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 24 * N, "d2h_bytes_per_step": 24 * N},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args, torch, rank, world, local, dist):
    """256 independent scenarios (mesh sides log-uniform in [20, 400], ~20M
    triangles) in one device pool, mixed precision, all advanced by the same
    persistent kernels and one graph launch per call."""
    from anuga_core_gb300 import workloads, _lib
    from anuga_core_gb300.batch import Batch
    t0 = time.time()
    doms, info = workloads.batch_workload(count=args.batch_count)
    B = Batch(doms, distribute=True)
    setup_s = time.time() - t0
    N = B.cells()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    B.set_stream(stream.cuda_stream)
    from anuga_core_gb300.autotune import tune_pool
    res, best = tune_pool(B.pool, steps=3, reps=2)
    B.advance_steps(args.warmup)
    launches0 = _lib.kernel_launches()
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    B.advance_steps(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    launches = _lib.kernel_launches() - launches0
    phases = B.pool.time_phases(reps=2)
    value = N * args.steps / (ms / 1e3)
    hbm, peak_kind = _peaks()
    ach = ALG_BYTES_PER_CELL_STEP["mixed"] * N / (ms / args.steps / 1e3) / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 flux / f64 accumulate", "data": "synthetic",
            "config": {"workload": "batch of %d rectangular-cross scenarios, sides log-uniform [20,400], %d triangles, "
                       "DE1 mixed, one pool" % (len(doms), N), "cells": N, "scenarios": len(doms),
                       "setup_s": setup_s, "draw": info["draw"], "l2": "inputs larger than L2",
                       "autotune": {"chosen": best, "s_per_step": res}},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "peak_kind": peak_kind, "traffic": None, "phase_ms": phases},
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line))


def scn_bytes(d):
    from anuga_core_gb300 import _lib
    if d.precision == "mixed":
        from anuga_core_gb300 import mixed
        return mixed.footprint(len(d), d.mesh.boundary_length, 1)
    T = d._tables
    return _lib.footprint(T["conn"].shape[0], T["boundary_slot"].shape[0], T["edge_slot"].shape[0])


if __name__ == "__main__":
    main()
