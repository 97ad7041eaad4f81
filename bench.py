"""Throughput benchmark of the DE timestep: cell-steps/s on one GB300.

Workload (one "step" = one full DE1 RK2 timestep of the whole mesh):
inflow_bumps, a 1000 x 1000 rectangular cross mesh (4.0M triangles) over
10 km x 10 km, slope + 64 Gaussian bumps (~30% dry), Dirichlet 2 m inflow west,
transmissive east, reflective north/south, Manning U(0.02, 0.06).  Synthetic
seeded data (workloads.inflow_bumps).  The state (>1 GB) is far larger than
the 129 MB L2, so no explicit flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

By default the plain FP64 path and then the mixed-precision path run on the
same workload; the line's value, roofline and e2e are the mixed path's, and
`plain_fp64` holds the plain path's figures (`mixed_over_plain` = ratio).
`accuracy` holds the mixed path's error against the plain FP64 path after
2000 mixed steps of the same workload, at the same simulated time (max depth
and velocity error, relative volume difference); `batched` the batched form
(256 scenarios, ~20M triangles, one pool, 500 timed steps) with its error on
a sample of scenarios; `serving` the serving form (256 requests of a Poisson
stream, p50/p99 latency).  `--workload batch` and `--workload serve` run the
batched and serving forms alone.

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


def max_over_ranks(ms, dist):
    """The slowest rank's time: each rank is an independent replica (no
    data-path collective); the job's time is the maximum over ranks."""
    if dist is None:
        return ms
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells_per_rank, steps, ms_max, world):
    """Whole-job throughput: every rank advances its own replica."""
    return world * cells_per_rank * steps / (ms_max / 1e3)


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
            t0 = time.perf_counter()            # sampling is running before the timed region starts
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
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


def _oracle_domain(m, threads, workload="inflow_bumps", cells=1.2e6):
    """The oracle (restated reference, OpenMP) set up with the workload's mesh,
    initial state, boundaries and operators, after one warm-up step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from anuga_core_gb300 import workloads
    if workload == "rain_polygon":
        d = workloads.rain_polygon(target_cells=cells, precision="fp64")
        kinds = {"inflow": ("dirichlet", (3.0, 0.0, 0.0)), "wall": ("reflective", None)}
        rates = [(op.indices, op.rate) for op in d.fractional_step_operators if hasattr(op, "rate")]
    else:
        d = workloads.inflow_bumps(m=m)
        kinds = {"left": ("dirichlet", (2.0, 0.0, 0.0)), "right": ("transmissive", None),
                 "top": ("reflective", None), "bottom": ("reflective", None)}
        rates = []
    oracle.build()
    oracle.set_threads(threads)
    oracle.set_parallel_extrapolation(True)
    od = oracle.OracleDomain(d.mesh, "DE1")
    Q = d.quantities
    od.set_centroid_state(Q["stage"].centroid_values, Q["xmomentum"].centroid_values,
                          Q["ymomentum"].centroid_values, Q["elevation"].centroid_values,
                          Q["friction"].centroid_values)
    od.set_boundaries([(d.mesh.tag_boundary_cells[t], kinds[t][0], kinds[t][1]) for t in d.mesh.tag_boundary_cells])
    for idx, rate in rates:
        od.add_rate(idx, rate)
    gen = od.evolve(yieldstep=1e9, finaltime=None, max_steps=10**9)
    next(gen)                      # initial distribute
    od.relative_yieldtime = 1e300
    od.relative_finaltime = None
    od.rk2_step(1e300, None)       # warm-up step
    return od, len(d.mesh)


def _oracle_steps(od, steps):
    t0 = time.perf_counter()
    for _ in range(steps):
        od.rk2_step(1e300, None)
        od.relative_time += od.timestep
    return time.perf_counter() - t0


def cpu_baseline(m, steps, threads, workload="inflow_bumps", cells=1.2e6):
    """Oracle (restated reference, OpenMP) on the same workload: `steps` DE1
    steps of the full mesh after one warm-up step."""
    od, N = _oracle_domain(m, threads, workload, cells)
    el = _oracle_steps(od, steps)
    return {"value": N * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d DE1 steps of the %d-triangle %s mesh (%.1f s)" % (steps, N, workload, el)}


def run_reference(args):
    """The oracle port (the reference's CPU algorithm, OpenMP on every host
    core); one bench step = one DE1 step of the full mesh."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    od, N = _oracle_domain(args.m, threads, args.workload, args.cells)
    _oracle_steps(od, args.warmup)
    el = _oracle_steps(od, args.steps)
    v = N * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload_name(args, N), "cells": N, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d DE1 steps of the full %d-triangle mesh after %d warm-up steps (%.1f s)"
                             % (args.steps, N, args.warmup, el)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 50; 500 for --workload batch, about a second of timing)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--m", type=int, default=1000, help="mesh side (4*m*m triangles)")
    ap.add_argument("--precision", default="both", choices=["both", "fp64", "mixed"],
                    help="both: plain FP64 then mixed on the same workload; the line's value is mixed")
    ap.add_argument("--cpu-steps", type=int, default=60, dest="cpu_steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--requests", type=int, default=256, help="serve workload: number of requests")
    ap.add_argument("--chunk-steps", type=int, default=128, help="serve workload: device steps per chunk")
    ap.add_argument("--err-steps", type=int, default=2000, dest="err_steps",
                    help="mixed steps of the accuracy check against plain FP64 (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=500, dest="batch_steps",
                    help="timed steps of the batched form in the default line")
    ap.add_argument("--no-batch", action="store_true", help="leave the batched form out of the default line")
    ap.add_argument("--no-serve", action="store_true", help="leave the serving form out of the default line")
    ap.add_argument("--cells", type=float, default=1.2e6, help="rain_polygon workload: target triangles")
    ap.add_argument("--workload", default="inflow_bumps", choices=["inflow_bumps", "rain_polygon", "batch", "serve"],
                    help="inflow_bumps: one 4M-triangle mesh; batch: 256 scenarios (~20M triangles) in one pool")
    ap.add_argument("--batch-count", type=int, default=256, dest="batch_count")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 500 if args.workload == "batch" else 50
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
    if args.workload == "serve":
        return run_serve(args, torch)
    precisions = ["fp64", "mixed"] if args.precision == "both" else [args.precision]
    if args.workload == "rain_polygon":
        from anuga_core_gb300 import workloads as W

        def builder(prec):
            return W.rain_polygon(target_cells=args.cells, precision=prec)
    else:
        def builder(prec):
            return build_workload(args.m, prec)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    res = {}
    for prec in precisions:
        res[prec] = measure_single(args, prec, torch, world, barrier, dist, builder)
    clocks = sampler.stop()
    both = args.precision == "both"
    accuracy = measure_accuracy(args, builder) if both and args.err_steps > 0 else None
    batched = serving = None
    if both and args.workload == "inflow_bumps":
        if not args.no_batch:
            batched = measure_batch(args, torch, world, dist, args.batch_steps, err_sample=args.batch_count)
            batched["over_plain_fp64"] = batched["value"] / res["fp64"]["value"]
        if not args.no_serve and world == 1:
            serving = measure_serve(args, torch)
    if rank == 0:
        head = res[precisions[-1]]
        N = head["cells"]
        cpu = None
        if not args.no_cpu and world == 1:
            cpu = cpu_baseline(args.m, args.cpu_steps, os.cpu_count() or 1, args.workload, args.cells)
        line = {
            "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head["precision"] == "fp64" else "f32 flux / f64 accumulate",
            "data": "synthetic",
            "config": {"workload": workload_name(args, N), "cells": N, "precision": head["precision"],
                       "l2": "inputs larger than L2 (state %.0f MB)" % (head["state_bytes"] / 1e6),
                       "parallelism": "replicas" if world > 1 else "single", "autotune": head["autotune"]},
            "roofline": head["roofline"],
            "step_roofline": head["step_roofline"],
            "e2e": head["e2e"],
            "gpu_launches": int(sum(r["launches"] for r in res.values())),
            "clocks": clocks,
        }
        if "fp64" in res and head["precision"] != "fp64":
            pf = res["fp64"]
            line["plain_fp64"] = {k: pf[k] for k in ("value", "ms_per_step", "roofline", "step_roofline", "e2e")}
            line["mixed_over_plain"] = head["value"] / pf["value"]
        if accuracy is not None:
            line["accuracy"] = accuracy
            for k in ("max_depth_err_m", "max_velocity_err_ms", "rel_volume_err"):
                line[k] = accuracy[k]
        if batched is not None:
            line["batched"] = batched
            line["gpu_launches"] += int(batched.get("gpu_launches", 0))
        if serving is not None:
            line["serving"] = serving
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


# Compulsory bytes per cell and step of the dominant kernel category, for
# the per-kernel roofline (the arrays each kernel must read or write once).
# mixed "flux": stage-1 flux (static 96 + lnk 4 + record 16 read, E 20
# written) + stage-2 flux (168 read, 40 written).  mixed "update": 60 read,
# 40 written.  fp64 "extrap", per RK2 stage: conn and surr (32), extrapolation
# geometry (11 x 8), centroid w, h, u, v (32) read; edge w, h, uh, vh, z
# (5 x 3 x 8) written.
KERNEL_BYTES_PER_CELL = {"mixed": {"flux": 136.0 + 208.0, "update": 100.0},
                         "fp64": {"extrap": 2 * 272.0}}


def workload_name(args, N):
    if args.workload == "rain_polygon":
        return ("rain_polygon: 20-vertex random polygon, %d triangles (Delaunay, <=50 m^2, <=12.5 m^2 in the "
                "refined region), value-noise bed, rain 50 mm/h on 1 km^2, 3 m inflow, DE1 RK2" % N)
    return "inflow_bumps %dx%d rectangular cross (%d triangles), DE1 RK2" % (args.m, args.m, N)


def measure_single(args, precision, torch, world, barrier, dist, builder):
    """Device-resident throughput, per-kernel roofline and the end-to-end
    figure (host buffers through the C ABI) of one precision form."""
    from anuga_core_gb300 import _lib
    d = builder(precision)
    N = len(d)
    d.distribute_to_vertices_and_edges()
    scn = d._scn
    stream = torch.cuda.Stream()          # a real stream: the legacy default one has handle 0
    torch.cuda.set_stream(stream)
    scn.set_stream(stream.cuda_stream)
    tune = None
    if precision == "mixed":
        from anuga_core_gb300.autotune import tune_pool
        res, best = tune_pool(scn.pool, steps=5, reps=2)
        tune = {"chosen": best, "s_per_step": res}
    d.advance_steps(args.warmup)
    launches0 = _lib.kernel_launches()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    d.advance_steps(args.steps)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    launches = _lib.kernel_launches() - launches0
    ms = max_over_ranks(ms, dist)
    ms_per_step = ms / args.steps
    value = replica_value(N, args.steps, ms, world)

    # per-kernel CUDA-event timing (direct launches on the same stream)
    phases = scn.time_phases(reps=3)
    step_ms = sum(phases.values())
    hbm, peak_kind = _peaks()
    kb = KERNEL_BYTES_PER_CELL[precision]
    dominant = max(phases, key=phases.get)
    dom_bytes = kb.get(dominant)
    ach_k = dom_bytes * N / (phases[dominant] / 1e3) / 1e9 if dom_bytes else None
    roof = {"bound": "hbm", "achieved": ach_k, "peak": hbm, "unit": "GB/s",
            "frac": ach_k / hbm if ach_k else None, "peak_kind": peak_kind,
            "traffic": TRAFFIC_PER_STEP.get((precision, dominant), {}).get("bytes_per_cell", None),
            "kernel": "%s (%.1f%% of step time)" % (dominant, 100.0 * phases[dominant] / max(step_ms, 1e-9)),
            "kernel_ms_per_step": phases[dominant], "alg_bytes_per_cell": dom_bytes,
            "phase_ms": phases}
    if roof["traffic"] is not None:
        roof["traffic"] = roof["traffic"] * N
        roof["traffic_note"] = TRAFFIC_PER_STEP[(precision, dominant)]["note"]
    if precision == "fp64":
        fp = _lib.fp64_throughput()
        roof["fp64_measured"] = fp
        # the FP64 instruction counts per cell were captured on the inflow_bumps mesh
        roof["fp64"] = fp64_roofline(N, ms_per_step, fp["dfma_gops"]) if args.workload == "inflow_bumps" else None
        roof["note"] = ("FP64-pipe bound, not HBM bound: GB300 runs FP64 at 1/54 of its FP32 rate "
                        "(fp64_measured, G ops/s); roofline.fp64 puts the step against the measured DFMA rate")
    alg_step = ALG_BYTES_PER_CELL_STEP[precision] * N
    ach_s = alg_step / (ms_per_step / 1e3) / 1e9
    step_roof = {"achieved": ach_s, "peak": hbm, "unit": "GB/s", "frac": ach_s / hbm,
                 "note": "%d algorithmic B/cell-step of the ideal fused step x cells / step time" %
                 ALG_BYTES_PER_CELL_STEP[precision]}

    # e2e: through the C ABI with host buffers, copies inside the timed region
    pin = {f: torch.empty(N, dtype=torch.float64, pin_memory=True).numpy() for f in ("stage_c", "xmom_c", "ymom_c")}
    for f in pin:
        scn.get(f, out=pin[f])
    d.relative_yieldtime = float("inf")
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    barrier()
    e2.record(stream)
    w, uh, vh = pin["stage_c"], pin["xmom_c"], pin["ymom_c"]
    for _ in range(args.steps):              # the Domain calls a user makes
        d.set_conserved_state(w, uh, vh)
        d.advance_steps(1)
        d.get_conserved_state(w, uh, vh)
    e3.record(stream)
    barrier()
    e2e_ms = max_over_ranks(e2.elapsed_time(e3), dist)
    e2e_value = replica_value(N, args.steps, e2e_ms, world)
    out = {"precision": precision, "cells": N, "value": value, "ms_per_step": ms_per_step, "roofline": roof,
           "step_roofline": step_roof, "launches": launches, "autotune": tune, "state_bytes": scn_bytes(d),
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 24 * N, "d2h_bytes_per_step": 24 * N,
                   "path": "conserved state w, uh, vh from and to page-locked host buffers each step through "
                           "Domain.set_conserved_state / advance_steps(1) / get_conserved_state (agx_set_state, "
                           "agx_advance, agx_get_state; the mixed pool reads and writes mapped host memory "
                           "directly; the plain path copies)"}}
    del d, scn
    torch.cuda.synchronize()
    return out


# DRAM traffic per cell-step of the dominant kernel category, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum summed over that
# category's launches of one step, divided by the cells of the captured mesh).
# FP64-pipe instructions per cell of one DE1 step (two stages) of the plain
# path, from one ncu capture (sm__thread_inst_executed_pipe_fp64_pred_on.sum:
# lanes that did work; sm__inst_executed_pipe_fp64.sum x 32: lane slots the
# warps occupied, idle lanes of divergent branches included) of each kernel
# of a stage (prep, extrapolation, flux, accumulation, update) on the
# 1.0M-triangle inflow_bumps case, divided by its cells, times two stages.
FP64_PER_CELL_STEP = {
    "lane_ops": 2 * (7.241 + 102.7 + 102.9 + 55.64 + 52.47),
    "warp_slots": 2 * 32 * (2.318e5 + 3.958e6 + 3.516e6 + 1.820e6 + 1.690e6) / 1.0e6,
    "note": "ncu --metrics sm__thread_inst_executed_pipe_fp64_pred_on.sum,sm__inst_executed_pipe_fp64.sum of "
            "k_prep, k_extrap<0,1>, k_flux, k_accum, k_update on the 1.0M-triangle inflow_bumps case (m=500), "
            "per cell and launch, x 2 stages of a DE1 step"}


def fp64_roofline(cells, ms_per_step, dfma_gops):
    """The plain step against the FP64 pipe: FP64 lane operations per second
    (the instructions the step issues per cell x cells / step time) over the
    measured DFMA rate, and the same for the lane slots the warps occupied."""
    sec = ms_per_step / 1e3
    ach = FP64_PER_CELL_STEP["lane_ops"] * cells / sec / 1e9
    occ = FP64_PER_CELL_STEP["warp_slots"] * cells / sec / 1e9
    return {"bound": "fp64", "achieved": ach, "peak": dfma_gops, "unit": "G FP64 lane-ops/s",
            "frac": ach / dfma_gops, "slots_achieved": occ, "slots_frac": occ / dfma_gops,
            "lane_ops_per_cell_step": FP64_PER_CELL_STEP["lane_ops"],
            "warp_slots_per_cell_step": FP64_PER_CELL_STEP["warp_slots"],
            "peak_kind": "measured live (agx_fp64_throughput, DFMA)", "note": FP64_PER_CELL_STEP["note"]}


TRAFFIC_PER_STEP = {
    ("mixed", "flux"): {
        "bytes_per_cell": (117.678592e6 + 15.682304e6 + 177.783552e6 + 32.170752e6) / 1.0e6,
        "note": "ncu --set full of k_pool_flux stage 1 + stage 2 on the 1.0M-triangle inflow_bumps case "
                "(m=500, MINB=8 variant), dram__bytes_read.sum + dram__bytes_write.sum per step, "
                "scaled by cells"},
    ("fp64", "extrap"): {
        "bytes_per_cell": 2 * (137.848576e6 + 85.762944e6) / 1.0e6,
        "note": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum of k_extrap<0,1> (edges only, cells in "
                "branch-class order, flowing state) on the 1.0M-triangle inflow_bumps case (m=500), per launch x 2 "
                "launches per DE1 step, scaled by cells"},
}


def measure_accuracy(args, builder):
    """Error of the mixed form against the plain FP64 form on the same
    workload: the mixed form takes `err_steps` steps from the protected
    initial state; the plain form evolves to the same simulated time.
    Max depth error, max velocity error over cells wetter than 1 cm in both,
    and the relative difference of the water volumes."""
    t0 = time.time()
    dm = builder("mixed")
    dm.distribute_to_vertices_and_edges()
    st = dm.advance_steps(args.err_steps)
    T = st.time
    Qm = dm.quantities
    wm, um, vm = (Qm[q].centroid_values.copy() for q in ("stage", "xmomentum", "ymomentum"))
    dm._scn.close()
    dm._scn = None
    dp = builder("fp64")
    for _ in dp.evolve(yieldstep=T, finaltime=T):
        pass
    Qp = dp.quantities
    z = Qp["elevation"].centroid_values
    wp, up, vp = (Qp[q].centroid_values for q in ("stage", "xmomentum", "ymomentum"))
    hm, hp = np.maximum(wm - z, 0.0), np.maximum(wp - z, 0.0)
    wet = (hm > 0.01) & (hp > 0.01)
    dvel = max(float(np.abs(um[wet] / hm[wet] - up[wet] / hp[wet]).max()),
               float(np.abs(vm[wet] / hm[wet] - vp[wet] / hp[wet]).max())) if wet.any() else 0.0
    A = dp.mesh.areas
    vol_m, vol_p = float(np.sum(A * hm)), float(np.sum(A * hp))
    out = {"max_depth_err_m": float(np.abs(hm - hp).max()), "max_velocity_err_ms": dvel,
           "rel_volume_err": abs(vol_m - vol_p) / max(vol_p, 1e-300),
           "mixed_steps": int(args.err_steps), "plain_steps": int(dp.total_steps), "simulated_s": T,
           "wet_cells_compared": int(wet.sum()), "bound_m": 1.0e-3,
           "against": "plain FP64 path (bit-exact with the reference's FP64 DE1 step) at the same simulated time",
           "wall_s": time.time() - t0}
    dp._scn.close()
    dp._scn = None
    return out


def measure_batch(args, torch, world, dist, steps, err_sample=0):
    """256 independent scenarios (mesh sides log-uniform in [20, 400], ~20M
    triangles) in one device pool, mixed precision, all advanced by the same
    persistent kernels and one graph launch per call.  With err_sample > 0,
    that many scenarios (evenly spaced) are also run alone in plain FP64 to
    the same simulated time and their max depth error is reported."""
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
    order_s, order = B.tune_order(steps=3, reps=2)
    res, best = B.kernel_form
    B.advance_steps(args.warmup)
    launches0 = _lib.kernel_launches()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    B.advance_steps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dist)
    launches = _lib.kernel_launches() - launches0
    phases = B.pool.time_phases(reps=2)
    value = replica_value(N, steps, ms, world)
    hbm, peak_kind = _peaks()
    ach = ALG_BYTES_PER_CELL_STEP["mixed"] * N / (ms / steps / 1e3) / 1e9
    dominant = max(phases, key=phases.get)
    kb = KERNEL_BYTES_PER_CELL["mixed"].get(dominant)
    ach_k = kb * N / (phases[dominant] / 1e3) / 1e9 if kb else None
    tr = TRAFFIC_PER_STEP.get(("mixed", dominant))
    out = {"value": value, "unit": UNIT, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
           "workload": "batch of %d rectangular-cross scenarios, sides log-uniform [20,400], %d triangles, "
                       "DE1 mixed, one pool" % (len(doms), N), "cells": N, "scenarios": len(doms),
           "setup_s": setup_s, "draw": info["draw"],
           "autotune": {"chosen": best, "s_per_step": res, "order": order, "order_s_per_step": order_s},
           "roofline": {"bound": "hbm", "achieved": ach_k, "peak": hbm, "unit": "GB/s",
                        "frac": ach_k / hbm if ach_k else None, "peak_kind": peak_kind,
                        "traffic": tr["bytes_per_cell"] * N if tr else None,
                        "traffic_note": tr["note"] if tr else None,
                        "kernel": "%s (%.1f%% of step time)" % (dominant, 100.0 * phases[dominant] / max(sum(phases.values()), 1e-9)),
                        "kernel_ms_per_step": phases[dominant], "alg_bytes_per_cell": kb, "phase_ms": phases},
           "step_roofline": {"achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                             "note": "352 algorithmic B/cell-step of the ideal fused step x cells / step time"},
           "gpu_launches": int(launches), "clocks": clocks}
    if err_sample > 0:
        # each checked scenario alone in plain FP64 to the same time (no yields
        # in either run); where the depth differs by more than 1 mm, the FP64
        # run is repeated with ten yields to show how far the FP64 solution
        # itself moves when only its timestep sequence changes
        t1 = time.time()
        pick = np.unique(np.linspace(0, len(doms) - 1, err_sample).round().astype(int))
        worst = [0.0, 0.0]
        over = []

        def plain(i, T, yields):
            dp = workloads.batch_scenario(info["sides"][i], 42 * 1000 + int(i), "dam" if i % 2 == 0 else "inflow",
                                          precision="fp64")
            for _ in dp.evolve(yieldstep=T / yields, finaltime=T):
                pass
            z = dp.quantities["elevation"].centroid_values
            h = np.maximum(dp.quantities["stage"].centroid_values - z, 0.0)
            A = dp.mesh.areas
            dp._scn.close()
            dp._scn = None
            return h, z, A

        for i in pick:
            st = B.stats(int(i))
            got = B.get_centroids(int(i))
            hp, z, A = plain(int(i), st.time, 1)
            hm = np.maximum(got["stage_c"] - z, 0.0)
            e = float(np.abs(hm - hp).max())
            vol = abs(float(np.sum(A * hm)) - float(np.sum(A * hp))) / max(float(np.sum(A * hp)), 1e-300)
            worst[1] = max(worst[1], vol)
            if e > 1.0e-3:
                h10 = plain(int(i), st.time, 10)[0]
                over.append({"scenario": int(i), "max_depth_err_m": e,
                             "fp64_spread_m": float(np.abs(h10 - hp).max())})
            else:
                worst[0] = max(worst[0], e)
        out["accuracy"] = {"max_depth_err_m": max([worst[0]] + [o["max_depth_err_m"] for o in over]),
                           "max_depth_err_within_bound_m": worst[0], "rel_volume_err": worst[1],
                           "scenarios_checked": int(len(pick)), "scenarios_over_1mm": over,
                           "against": "each scenario alone in plain FP64 at the same simulated time, same "
                                      "(yield-free) timestep sequence; fp64_spread_m = how far the FP64 "
                                      "solution moves when run with ten yields instead",
                           "wall_s": time.time() - t1}
    B.close()
    torch.cuda.set_stream(torch.cuda.default_stream())
    return out


def run_batch(args, torch, rank, world, local, dist):
    """The batched form alone: 256 scenarios in one pool (see measure_batch)."""
    b = measure_batch(args, torch, world, dist, args.steps, err_sample=0)
    line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 flux / f64 accumulate", "data": "synthetic",
            "config": {"workload": b["workload"], "cells": b["cells"], "scenarios": b["scenarios"],
                       "setup_s": b["setup_s"], "draw": b["draw"], "l2": "inputs larger than L2",
                       "autotune": b["autotune"]},
            "roofline": b["roofline"], "step_roofline": b["step_roofline"], "gpu_launches": b["gpu_launches"],
            "clocks": b["clocks"]}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def measure_serve(args, torch):
    """Poisson stream (20 req/s, seed 99) of flood scenarios: rectangular cross
    or Delaunay meshes with 10k-2M triangles (log-uniform), final times
    U(60, 3600) s, mixed precision, continuous batching in one pool.  The
    first `--requests` requests of the stream are served in real time."""
    from anuga_core_gb300.serve import FloodServer, MeshCache, poisson_requests
    reqs = poisson_requests(n=args.requests)
    cache = MeshCache()
    t0 = time.time()
    for r in reqs:                 # build the meshes of the stream up front (mesh cache warm)
        cache.get(r.kind, r.cells)
    setup_s = time.time() - t0
    srv = FloodServer(max_scenarios=256, chunk_steps=args.chunk_steps, mesh_cache=cache)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    summ = srv.run(reqs, realtime=True)
    clocks = sampler.stop()
    srv.close()
    return {"value": summ["cell_steps_per_s"], "unit": UNIT, "requests": summ["requests"],
            "p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "wall_s": summ["wall_s"],
            "cell_steps": summ["cell_steps"], "mesh_setup_s": setup_s,
            "chunks": summ["chunks"], "device_s": summ["device_s"], "admit_s": summ["admit_s"],
            "retire_s": summ["retire_s"], "idle_s": summ["idle_s"],
            "device_cell_steps_per_s": summ["device_cell_steps_per_s"],
            "workload": "serving: %d Poisson requests (20/s, seed 99), rectangular cross or Delaunay, 10k-2M "
                        "triangles, final time 60-3600 s, DE1 mixed, continuous batching in one pool, latency = "
                        "arrival to final state on the host" % len(reqs),
            "clocks": clocks}


def run_serve(args, torch):
    """The serving form alone (see measure_serve)."""
    sv = measure_serve(args, torch)
    line = {"metric": METRIC, "value": sv["value"], "unit": UNIT, "n_gpus": 1,
            "steps": sv["requests"], "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 flux / f64 accumulate", "data": "synthetic",
            "config": {"workload": sv["workload"], "mesh_setup_s": sv["mesh_setup_s"]},
            "latency": {"p50_s": sv["p50_s"], "p99_s": sv["p99_s"], "wall_s": sv["wall_s"],
                        "cell_steps": sv["cell_steps"], "chunks": sv["chunks"], "device_s": sv["device_s"],
                        "admit_s": sv["admit_s"], "retire_s": sv["retire_s"], "idle_s": sv["idle_s"],
                        "device_cell_steps_per_s": sv["device_cell_steps_per_s"]},
            "clocks": sv["clocks"]}
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
