#!/usr/bin/env python
"""Benchmark: RK4 particle-steps/s of flowVC's FTLE workload on a tet mesh.

Workload (one bench step = one complete FTLE window, the unit ompVC's FTLE
output is produced in): a unit cube of 64^3 cells split into 6 Kuhn
tetrahedra (1,572,864 tets, 274,625 nodes, interior nodes jittered +-0.2h
with seed 0), ABC velocity scaled by (1 + 0.1 sin 2 pi t) at 51 frames
dt = 0.02, an FTLE seed grid of 128^3 points over [0,1]^3 integrated forward
over T = 1 with RK4 h = 0.005, neighbour-walk point location with the global
search fallback (LocalSearchChecking = 1).  Inputs are synthetic, generated
here with fixed seeds (no dataset is involved).

value      accepted RK4 steps / s with mesh and frames resident in HBM; each
           step seeds and locates the grid, advects every interval
           (including the early-FTLE advections of points that leave) and
           reduces the FTLE field.  Early-FTLE advections that repeat the
           main pass exactly are read from its per-step record; their steps
           are counted (ompVC performs them) and also reported on their own
           (steps_early_recorded).  ftle_points_per_s counts no steps.
e2e        the same through the C ABI from pinned host buffers: mesh and all
           frames copied host->device inside each step, FTLE fields copied back.
roofline   the main advection kernel (k_ftle_pass1) against the measured HBM
           copy bandwidth, 1,384 algorithmic bytes per unstructured FP64 RK4
           step (4 stages x (connectivity 16 + node coordinates 96 + 4 nodes x
           2 frames x 3 x 8) + final containment 112 + state 56).
cpu_baseline  the CPU oracle (the reference's algorithm restated in C,
           OpenMP over all host cores) on a bounded sample: the same grid and
           mesh over the first 5 frame intervals (T = 0.1).

tracers    the cube's second workload: 1M tracers released at t = 0, outputs
           every 10 steps, FP64 and BF16 forms.
batched    the bent-tube batch of 64 tracer releases (uneven seed counts and
           windows) in the BF16 form and the FP64 form, one CUDA graph each.
served     a Poisson request stream over the tube and the cube, served in the
           BF16 and FP64 forms: p50 / p95 / p99 latency and steps/s.

--impl reference runs that CPU implementation alone, every step one bounded
sample, on the same metric.  Multi-GPU (torchrun, N > 1): every rank runs the
whole workload on its own GPU (replicas; the window has no exchange step),
value = all ranks' steps / the slowest rank's time.
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
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "flowvc-1_gb300")
for _p in (PKG, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

BYTES_PER_STEP = 1384        # unstructured FP64 RK4 step, algorithmic
CUBE_N = 64
NFRAMES, DT = 51, 0.02
H = 0.005
T_WINDOW = 1.0
SAMPLE_T = 0.1               # CPU sample: first 5 frame intervals


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--grid", type=int, default=128, help="FTLE seed grid edge")
    ap.add_argument("--cube", type=int, default=CUBE_N, help="mesh cells per edge")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the BF16 / FP16 mixed forms")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-tracers", action="store_true", help="skip the 1M-tracer release on the cube")
    ap.add_argument("--tracers", type=int, default=1_000_000)
    ap.add_argument("--no-batched", action="store_true", help="skip the bent-tube batch")
    ap.add_argument("--no-served", action="store_true", help="skip the served request stream")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--served-rate", type=float, default=200.0, help="requests / s")
    ap.add_argument("--served-seconds", type=float, default=10.0, help="arrival window, s")
    return ap.parse_args()


def make_inputs(n):
    import synth
    xyz, conn, adj = synth.kuhn_cube_mesh(n, jitter=0.2, seed=0)
    frames = [synth.abc_flow(xyz, f * DT) for f in range(NFRAMES)]
    return xyz, conn, adj, frames


def grid_tuple(g):
    return (0.0, 1.0, 0.0, 1.0, 0.0, 1.0, g, g, g)


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        finally:
            try:
                os.remove(self.path)
            except OSError:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ peaks

def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per k_ftle_pass1 launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ftle_pass1_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_step"), d
    except (OSError, ValueError):
        return None, None


# ------------------------------------------------------------------ CPU side

def cpu_sample(inputs, grid, threads, tmpdir):
    """The oracle on the bounded sample; returns (steps/s, steps, seconds, threads)."""
    import oracle_lib
    import synth
    xyz, conn, adj, frames = inputs
    d = os.path.join(tmpdir, "c2")
    if not os.path.exists(os.path.join(d, "cube_coordinates.bin")):
        os.makedirs(d, exist_ok=True)
        synth.write_unstructured_mesh(os.path.join(d, "cube"), xyz, conn, adj)
        nfr = int(round(SAMPLE_T / DT)) + 2
        for f in range(min(nfr, NFRAMES)):
            synth.write_frame(os.path.join(d, f"cube_vel.{f}.bin"), f * DT, frames[f])
    out = os.path.join(tmpdir, "c2out")
    os.makedirs(out, exist_ok=True)
    inp = os.path.join(tmpdir, "c2.in")
    g = grid
    synth.write_in_file(
        inp, Path_Data=d + "/", Path_Output=out + "/", Dimensions=3, Data_MeshType=1, Data_InFilePrefix="cube",
        Data_TRes=NFRAMES, Data_TDelta=DT, FTLE_Compute=1, FTLE_IntTLength=SAMPLE_T, Int_TimeStep=H,
        LocalSearchChecking=1, **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0,
                                  "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                                  "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0,
                                  "FTLE_MeshBounds.ZMax": 1.0, "FTLE_MeshBounds.XRes": g,
                                  "FTLE_MeshBounds.YRes": g, "FTLE_MeshBounds.ZRes": g})
    nthr = threads if threads > 0 else (os.cpu_count() or 1)
    rc, secs, steps, err = oracle_lib.run(inp, nthr)
    if rc:
        raise RuntimeError(f"oracle failed: {err}")
    return steps / secs, steps, secs, nthr


def run_reference(args, rank, world):
    if rank != 0:
        return
    inputs = make_inputs(args.cube)
    with tempfile.TemporaryDirectory() as td:
        for _ in range(args.warmup):
            cpu_sample(inputs, args.grid, args.cpu_threads, td)
        vals, steps_tot, secs_tot = [], 0, 0.0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v, st, secs, nthr = cpu_sample(inputs, args.grid, args.cpu_threads, td)
            vals.append(v)
            steps_tot += st
            secs_tot += secs
        wall = time.perf_counter() - t0
    value = steps_tot / secs_tot
    line = {
        "impl": "reference", "metric": "RK4 particle-steps/s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"FTLE {args.grid}^3 seeds, {args.cube}^3x6 jittered Kuhn tets, ABC flow, "
                               f"RK4 h={H}; sample: first {int(round(SAMPLE_T / DT))} frame intervals (T={SAMPLE_T})",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": nthr, "kind": "port",
                         "sample": f"FTLE {args.grid}^3 over T={SAMPLE_T} (5 of 50 intervals), advection phase timed"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ tracers

def bench_tracers(args, inputs):
    """The cube's tracer workload: args.tracers tracers released uniformly at
    t = 0 (seed 0), RK4 h = 0.005 over T = 1, positions output every 10 steps
    (t = 0, 0.05, ..., 1: 21 outputs, each copied to the host), through the
    single-release loop of ompVC's Compute_Tracer (flow.run_tracers), in the
    FP64 form and the BF16 form; endpoint errors of BF16 against FP64."""
    import flow
    import fvc
    import synth
    xyz, conn, adj, frames = inputs
    ax = flow.TimeAxis(0.0, DT, NFRAMES, 0)
    seeds = synth.uniform_seeds(args.tracers, 3, seed=0)
    out = {"workload": f"{args.tracers} tracers uniform in the cube at t=0, T={T_WINDOW}, RK4 h={H}, "
                       "positions output every 10 steps (21 outputs copied to the host)"}
    finals = {}
    for prec in ("fp64", "bf16"):
        ctx = fvc.Context(3, 1)
        ctx.set_unstruct_mesh(xyz, conn, adj)
        ctx.set_bounds([0, 1, 0, 1, 0, 1])
        ctx.set_integrator(1, H, 0)
        ctx.set_precision(prec)
        flow.upload_frames(ctx, ax, frames)
        flow.run_tracers(ctx, ax, seeds[:4096], 0.0, 0.05, 21)          # warm-up
        t0 = time.perf_counter()
        fin = {}
        outs, steps, st = flow.run_tracers(ctx, ax, seeds, 0.0, 0.05, 21, state=fin)
        wall = time.perf_counter() - t0
        finals[prec] = fin
        out[prec] = {"value": steps / wall, "unit": "steps/s", "steps": int(steps), "wall_s": wall,
                     "kernel_value": st["steps_main"] / (st["ms_main"] / 1e3) if st["ms_main"] > 0 else None,
                     "outputs": len(outs), "written": int(sum(len(o) for o in outs))}
        ctx.close()
    # final tracer states: endpoints (the last position inside for tracers that
    # left) over tracers whose exit status agrees, exit-time and id mismatches
    a, b = finals["fp64"], finals["bf16"]
    same = a["left"] == b["left"]
    d = np.linalg.norm(b["X"][same] - a["X"][same], axis=1) if same.any() else np.zeros(1)
    both = same & (a["left"] == 1)
    out["bf16"]["errors_vs_fp64"] = {
        "endpoint_max": float(d.max()), "endpoint_rms": float(np.sqrt((d ** 2).mean())),
        "eid_mismatch_rate": float((a["eid"][same] != b["eid"][same]).mean()) if same.any() else 0.0,
        "left_mismatch_rate": float((~same).mean()),
        "exit_time_mismatch_rate": float((np.abs(a["ldt"][both] - b["ldt"][both]) > 1e-9).mean()) if both.any() else 0.0,
        "left_fraction": float((a["left"] == 1).mean())}
    out["speedup_vs_fp64"] = out["bf16"]["value"] / out["fp64"]["value"]
    return out


# ------------------------------------------------------------------ batched / served

SERVED_BUDGET = 150 * 10 ** 9   # device bytes for frames plus job state, both sites


def bench_batched(args, tube, frames):
    """The bent-tube batch: 64 tracer releases (seed counts log-uniform in
    [1e3, 1e6] on random cross-sections, windows U[0.2, 2] periods, forward or
    backward), one persistent launch per tick, the whole schedule one CUDA
    graph, launch shape autotuned; BF16 frames with FP32 stages against the
    FP64 form on the same jobs."""
    import serve
    jobs = serve.tube_batch_jobs(tube, args.batch_jobs)
    out = {"workload": f"{len(jobs)} tracer releases on the bent tube ({len(tube.conn)} tets, "
                       f"{len(tube.xyz)} nodes, Womersley alpha=4, {serve.TUBE_FRAMES} frames a period), "
                       "seeds log-uniform in [1e3, 1e6], T in U[0.2, 2] periods, +-direction, RK4 h=0.002",
           "particles": int(sum(len(j[1]) for j in jobs)), "graph": True}
    res = {}
    for prec in ("bf16", "fp64"):
        site = serve.tube_site(prec, tube=tube, frames=frames)
        serve.warm_pairs(site)
        steps, secs, wall, st, r = serve.run_batched(site, jobs, graph=True, tune=True, results=True)
        res[prec] = r
        out[prec] = {"value": steps / wall, "unit": "steps/s", "steps": int(steps), "wall_s": wall,
                     "device_s": secs, "device_value": steps / secs if secs > 0 else None,
                     "tuned": {"threads": st["tuned_threads"], "blocks": st["tuned_blocks"],
                               "resort_every": st["tuned_resort"]}}
        site.close()
    out["speedup_vs_fp64"] = out["bf16"]["value"] / out["fp64"]["value"]
    import serve as _s
    out["bf16"]["errors_vs_fp64"] = _s.endpoint_errors(res["fp64"], res["bf16"])
    return out


def bench_served(args, tube, frames, cube_inputs):
    """A request stream over both resident data sets: Poisson arrivals for
    args.served_seconds, 50% tracer releases on the tube, 40% FTLE grids on
    the cube, 10% residence-time releases on the tube; admission by an HBM
    budget; latency from arrival to results on the host.  The same stream is
    served in the BF16 form and in the FP64 form."""
    import serve
    xyz, conn, adj, cframes = cube_inputs
    kw = dict(rate=args.served_rate, duration=args.served_seconds, seed=7)
    out = {"workload": f"Poisson {args.served_rate:g} requests/s for {args.served_seconds:g} s: 50% tracer releases "
                       "(tube, 1e3-1e5 seeds log-uniform, 0.2-2 periods), 40% FTLE grids (cube, 16^3-48^3, T=1), "
                       "10% residence time (tube, 1e4 seeds, 3 periods)",
           "hbm_budget_bytes": SERVED_BUDGET}
    for prec in ("bf16", "fp64"):
        reqs = serve.poisson_requests(tube, **kw)
        frame_bytes = 32 * (len(tube.xyz) * serve.TUBE_FRAMES + len(xyz) * len(cframes))
        budget = max((SERVED_BUDGET - frame_bytes) // 2, 1)
        sites = {"tube": serve.tube_site(prec, tube=tube, frames=frames, hbm_budget=budget),
                 "cube": serve.cube_site(prec, mesh=(xyz, conn, adj), frames=cframes, hbm_budget=budget)}
        serve.warm_pairs(sites["tube"])
        serve.run_batched(sites["cube"], [("ftle", (0, 1, 0, 1, 0, 1, 8, 8, 8), 0.0, 1.0)], graph=False, tune=False)
        r = serve.serve(sites, reqs)
        out[prec] = r
        out["requests"] = r["requests"]
        for st in sites.values():
            st.close()
    out["speedup_vs_fp64"] = out["bf16"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    return out


# ------------------------------------------------------------------ ranks

def form_errors(ref, got):
    """Errors of a mixed-precision window against the FP64 one.  Endpoints:
    each point's final position (for a point that left, its last position
    inside), over the points whose exit status agrees; element ids over the
    same points; exit-flag and exit-time mismatches; FTLE errors relative to
    the largest FP64 value and pointwise (floor 1e-3 of the largest)."""
    (rT, rs), (gT, gs) = ref, got
    same = rs["left"] == gs["left"]
    d = np.linalg.norm(gs["X"][same] - rs["X"][same], axis=1) if same.any() else np.zeros(1)
    both_left = same & (rs["left"] == 1)
    scale = float(np.abs(rT).max()) or 1.0
    e = np.abs(gT - rT)
    rel = e / np.maximum(np.abs(rT), 1e-3 * scale)
    return {"endpoint_max": float(d.max()), "endpoint_rms": float(np.sqrt((d ** 2).mean())),
            "ftle_max_rel_to_max": float(e.max() / scale), "ftle_rms_rel_to_max": float(np.sqrt((e ** 2).mean()) / scale),
            "ftle_median_rel": float(np.median(rel)), "ftle_p99_rel": float(np.quantile(rel, 0.99)),
            "ftle_max_rel": float(rel.max()),
            "eid_mismatch_rate": float((gs["eid"][same] != rs["eid"][same]).mean()) if same.any() else 0.0,
            "left_mismatch_rate": float((~same).mean()),
            "exit_time_mismatch_rate": float((np.abs(gs["ldt"][both_left] - rs["ldt"][both_left]) > 1e-9).mean())
            if both_left.any() else 0.0,
            "points_left": float((rs["left"] == 1).mean())}


def precision_forms(ctx, ax, grid, stream, barrier, args, fp64_value):
    """BF16 and FP16 frames with FP32 stages (fvc_set_precision) on the same
    context and workload: one warm-up window, then args.steps timed windows
    with CUDA events; errors against one more FP64 window."""
    import torch

    import flow
    ref_state = {}
    ref_T = flow.run_ftle(ctx, ax, grid, T_WINDOW, state=ref_state)[0]
    out = {}
    for name in ("bf16", "fp16"):
        ctx.set_precision(name)
        flow.run_ftle(ctx, ax, grid, T_WINDOW)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps, stats, st_last, T_last = 0, [], {}, None
        e0.record(stream)
        for k in range(args.steps):
            wT, wN, st, js = flow.run_ftle(ctx, ax, grid, T_WINDOW)
            steps += st
            stats.append(js)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        got_state = {}
        T_last = flow.run_ftle(ctx, ax, grid, T_WINDOW, state=got_state)[0]
        value = steps / (ms / 1000.0)
        out[name] = {"value": value, "unit": "steps/s", "ms_per_step": ms / args.steps,
                     "ftle_points_per_s": args.grid ** 3 * args.steps / (ms / 1000.0),
                     "speedup_vs_fp64": value / fp64_value,
                     "steps_early_recorded_per_step": sum(x["steps_early_recorded"] for x in stats) / args.steps,
                     "phases_ms_per_step": {k: sum(s[k] for s in stats) / args.steps
                                            for k in ("ms_setup", "ms_main", "ms_early", "ms_reduce")},
                     "errors": form_errors((ref_T, ref_state), (T_last, got_state))}
    ctx.set_precision("fp64")
    return out


def reduce_over_ranks(secs, units, world):
    """(max seconds over ranks, sum of units over ranks).  Every rank calls it;
    uses the process group's device (CUDA for NCCL, CPU for gloo)."""
    if world <= 1:
        return float(secs), float(units)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(secs)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ------------------------------------------------------------------ GPU side

def run_engine(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    import flow
    import fvc
    import build as fvc_build

    fvc_build.build()
    torch.cuda.set_device(local_rank)
    inputs = make_inputs(args.cube)
    xyz, conn, adj, frames = inputs
    ax = flow.TimeAxis(0.0, DT, NFRAMES, 0)
    grid = grid_tuple(args.grid)
    npts = args.grid ** 3

    try:
        fma_s, div_s = fvc.probe_fp64(local_rank)
        fp64 = {"fma_per_s": fma_s, "div_per_s": div_s}
    except fvc.FvcError:
        fp64 = None
    ctx = fvc.Context(3, 1, device=local_rank)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, H, 0)
    flow.upload_frames(ctx, ax, frames)
    stream = torch.cuda.ExternalStream(ctx.stream())

    for _ in range(args.warmup):
        flow.run_ftle(ctx, ax, grid, T_WINDOW)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    stats = []
    steps_total = 0
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            wT, wN, st, js = flow.run_ftle(ctx, ax, grid, T_WINDOW)
            steps_total += st
            stats.append(js)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    clocks = clk.summary()
    secs = ms / 1000.0
    secs_max, steps_all = reduce_over_ranks(secs, steps_total, world)

    # roofline of the main advection kernel from its CUDA-event times
    ms_main = sum(s["ms_main"] for s in stats)
    steps_main = sum(s["steps_main"] for s in stats)
    launches_main = sum(s["intervals"] for s in stats)
    peak, peak_kind = measured_peak()
    achieved = (steps_main * BYTES_PER_STEP) / (ms_main / 1000.0) / 1e9 if ms_main > 0 else 0.0
    traffic_per_step, prof = profiled_traffic()
    traffic = traffic_per_step * steps_main / launches_main if traffic_per_step else None
    # the bound that applies: FP64 issue (ops per step from the committed
    # instruction-mix profile) against the FMA rate the probe measured
    fp64_pipe = None
    if prof and prof.get("fp64_pipe_ops_per_step") and fp64 and ms_main > 0:
        ops = prof["fp64_pipe_ops_per_step"] * steps_main / (ms_main / 1000.0)
        fp64_pipe = {"ops_per_step": prof["fp64_pipe_ops_per_step"], "achieved": ops / 1e9,
                     "peak": fp64["fma_per_s"] / 1e9, "unit": "G FP64-pipe ops/s",
                     "frac": ops / fp64["fma_per_s"], "kernel": "k_ftle_pass1"}
    gpu_launches = int(sum(s["launches"] for s in stats))

    # the mixed-precision forms on the same workload, against this FP64 run
    forms = None
    if not args.no_precision:
        forms = precision_forms(ctx, ax, grid, stream, barrier, args, steps_all / secs_max)

    # end to end through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        pxyz, pconn, padj = pin(xyz), pin(conn), pin(adj)
        pframes = [pin(f) for f in frames]
        h2d = pxyz.nbytes + pconn.nbytes + padj.nbytes + sum(f.nbytes for f in pframes)
        d2h = 2 * 8 * npts
        ctx.close()
        barrier()
        t0 = time.perf_counter()
        e2e_steps = 0
        for _ in range(args.steps):
            c2 = fvc.Context(3, 1, device=local_rank)
            c2.set_unstruct_mesh(pxyz, pconn, padj)
            c2.set_bounds([0, 1, 0, 1, 0, 1])
            c2.set_integrator(1, H, 0)
            flow.upload_frames(c2, ax, pframes, asynchronous=True)
            wT, wN, st, _ = flow.run_ftle(c2, ax, grid, T_WINDOW)
            e2e_steps += st
            c2.close()
        barrier()
        e2e_secs, e2e_all = reduce_over_ranks(time.perf_counter() - t0, e2e_steps, world)
        e2e = {"value": e2e_all / e2e_secs, "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
    else:
        ctx.close()

    tracers = None if args.no_tracers else bench_tracers(args, inputs)
    batched = served = None
    if not (args.no_batched and args.no_served):
        import serve
        import synth
        tube = synth.bent_tube_mesh()
        _, tframes = synth.womersley_frames(tube, nframes=serve.TUBE_FRAMES)
        if not args.no_batched:
            batched = bench_batched(args, tube, tframes)
        if not args.no_served:
            served = bench_served(args, tube, tframes, inputs)
        del tube, tframes

    cpu = None
    if rank == 0 and not args.no_cpu:
        with tempfile.TemporaryDirectory() as td:
            v, st, s2, nthr = cpu_sample(inputs, args.grid, args.cpu_threads, td)
        cpu = {"value": v, "unit": "steps/s", "cores": nthr, "kind": "port",
               "sample": f"FTLE {args.grid}^3 over T={SAMPLE_T} (5 of 50 intervals), {st} steps in {s2:.2f} s "
                         f"of advection"}

    if rank == 0:
        value = steps_all / secs_max
        line = {
            "metric": "RK4 particle-steps/s", "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"FTLE {args.grid}^3 seeds over T={T_WINDOW}, {args.cube}^3x6 jittered Kuhn tets "
                                   f"({6 * args.cube ** 3} tets), ABC flow {NFRAMES} frames, RK4 h={H}",
                       "l2": "inputs larger than L2 (frames 51 x 8.8 MB + 420 MB of grid state)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "ftle_points_per_s": npts * args.steps * world / secs_max,
            "steps_main": int(steps_main), "steps_early": int(sum(s["steps_early"] for s in stats)),
            "steps_early_recorded": int(sum(s["steps_early_recorded"] for s in stats)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "k_ftle_pass1", "bytes_per_step": BYTES_PER_STEP},
            "gpu_launches": gpu_launches,
            "fp64_pipe": fp64_pipe,
            "precision_forms": forms,
            "tracers": tracers,
            "batched": batched,
            "served": served,
            "phases_ms_per_step": {k: sum(s[k] for s in stats) / args.steps
                                   for k in ("ms_setup", "ms_main", "ms_early", "ms_reduce")},
            "fp64_probe": fp64,
            "clocks": clocks,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_engine(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
