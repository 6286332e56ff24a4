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
           reduces the FTLE field, which stays in HBM (the end-to-end
           figure reads it back).  Early-FTLE advections that repeat the
           main pass exactly are read from its per-step record; their steps
           are counted (ompVC performs them) and also reported on their own
           (steps_early_recorded).  ftle_points_per_s counts no steps.
e2e        the same through the C ABI from pinned host buffers: mesh and all
           frames copied host->device inside each step (the mesh validated and
           its records and bucket grid rebuilt), both FTLE fields copied back
           into page-locked arrays; one context for all steps.
roofline   the main advection kernel (k_ftle_pass1) against the bound that
           applies to it, the FP64 pipe: FP64-pipe instructions per step (the
           committed instruction-mix profile) x steps / CUDA-event time,
           against the FP64 FMA rate measured on the same device in the same
           run (tests/cuda/fp64_rate.cu).  roofline.hbm gives the same kernel
           against the measured HBM copy bandwidth, 1,384 algorithmic bytes per
           unstructured FP64 RK4 step (4 stages x (connectivity 16 + node
           coordinates 96 + 4 nodes x 2 frames x 3 x 8) + final containment
           112 + state 56), with the DRAM traffic ncu measured.
steps_computed  the steps the GPU actually advanced (value also counts the
           early-FTLE steps read from the main pass's record).
parity     one more FP64 window against the CPU oracle's run of the same
           window on the same inputs (final grid state bit for bit, FTLE
           fields within 1e-12) and against ompVC's own outputs for this
           workload (the committed summaries of tests/golden/scale/).
cpu_baseline  the CPU oracle (the reference's algorithm restated in C,
           OpenMP over all host cores) on the same workload: the whole
           T = 1 window, advection phase timed.
double_gyre   the 2D Cartesian workload: double gyre on 257 x 129 nodes,
           101 frames dt = 0.1, FTLE on 512 x 256 seeds over T = 10, RK4
           h = 0.01, FP64: steps/s, FTLE points/s, the 816 B/step roofline,
           parity and the CPU oracle on the same window.

tracers    the cube's second workload: 1M tracers released at t = 0, outputs
           every 10 steps, FP64 and BF16 forms.
batched    the bent-tube batch of 64 tracer releases (uneven seed counts and
           windows) in the BF16 form and the FP64 form, one CUDA graph each.
served     a Poisson request stream over the tube and the cube (200 requests/s
           for 60 s at the served workload's sizes), served in the BF16 and
           FP64 forms: p50 / p95 / p99 latency and steps/s; a form that cannot
           keep up is stopped and reported with its backlog.

--impl reference runs that CPU implementation alone on the same workload
(every step one whole T = 1 window), on the same metric.  Multi-GPU (torchrun, N > 1): every rank runs the
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
# config 1: the double gyre on a Cartesian grid
DG_NX, DG_NY, DG_FRAMES, DG_DT = 257, 129, 101, 0.1
DG_GRID = (0.0, 2.0, 0.0, 1.0, 0.0, 0.0, 512, 256, 1)
DG_H, DG_T = 0.01, 10.0
DG_BYTES_PER_STEP = 816      # Cartesian 2D FP64 RK4 step, algorithmic


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
    ap.add_argument("--no-dg", action="store_true", help="skip the double-gyre (Cartesian 2D) workload")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity window")
    ap.add_argument("--probe-advect", type=int, default=0, metavar="NPTS",
                    help="instead of the benchmark: a fixed step-level workload for instruction-mix profiles "
                         "(fvc_advect, RK4 h=0.005 over one frame interval, NPTS points on the 32^3 cube, "
                         "two calls; per-step figures = the second k_advect launch's counters / its steps)")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--served-rate", type=float, default=200.0, help="requests / s")
    ap.add_argument("--served-seconds", type=float, default=60.0, help="arrival window, s")
    ap.add_argument("--served-sweep", action="store_true", help="add a rate sweep of the served form")
    ap.add_argument("--served-forms", default="bf16,fp64", help="arithmetic forms of the served stream")
    ap.add_argument("--sweep-seconds", type=float, default=15.0, help="arrival window of each sweep point, s")
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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # the timed region starts once the sampler is writing (its start-up
        # would otherwise take most of a short region)
        t0 = time.time()
        while self.proc and time.time() - t0 < 3.0 and os.path.getsize(self.path) == 0:
            time.sleep(0.01)
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


# ------------------------------------------------------------------ FP64 rate

def probe_fp64(device):
    """(FP64 FMAs / s, IEEE divisions / s) of the device, from the rate probe
    tests/cuda/fp64_rate.cu (built here with nvcc); None if it cannot run."""
    src = os.path.join(ROOT, "tests", "cuda", "fp64_rate.cu")
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "fp64_rate")
        try:
            subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe, src],
                           check=True, capture_output=True, timeout=300)
            r = subprocess.run([exe, str(device)], check=True, capture_output=True, text=True, timeout=120)
            d = json.loads(r.stdout.strip().splitlines()[-1])
            return {"fma_per_s": float(d["fma_per_s"]), "div_per_s": float(d["div_per_s"])}
        except (OSError, subprocess.SubprocessError, ValueError, KeyError, IndexError):
            return None


# ------------------------------------------------------------------ CPU side

def write_cube_files(inputs, d, nframes=NFRAMES):
    import synth
    xyz, conn, adj, frames = inputs
    if not os.path.exists(os.path.join(d, f"cube_vel.{nframes - 1}.bin")):
        os.makedirs(d, exist_ok=True)
        synth.write_unstructured_mesh(os.path.join(d, "cube"), xyz, conn, adj)
        for f in range(nframes):
            synth.write_frame(os.path.join(d, f"cube_vel.{f}.bin"), f * DT, frames[f])
    return d


def cpu_window(inputs, grid, threads, tmpdir, dump=None):
    """The oracle on the whole FTLE window (T = 1) of the benchmark, with all
    host threads: returns (steps/s of the advection phase, steps, seconds,
    threads, output directory).  dump: directory for its final grid state."""
    import oracle_lib
    import synth
    d = write_cube_files(inputs, os.path.join(tmpdir, "c2"))
    out = os.path.join(tmpdir, "c2out")
    os.makedirs(out, exist_ok=True)
    inp = os.path.join(tmpdir, "c2.in")
    g = grid
    synth.write_in_file(
        inp, Path_Data=d + "/", Path_Output=out + "/", Dimensions=3, Data_MeshType=1, Data_InFilePrefix="cube",
        Data_TRes=NFRAMES, Data_TDelta=DT, FTLE_Compute=1, FTLE_IntTLength=T_WINDOW, Int_TimeStep=H,
        LocalSearchChecking=1, **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0,
                                  "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                                  "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0,
                                  "FTLE_MeshBounds.ZMax": 1.0, "FTLE_MeshBounds.XRes": g,
                                  "FTLE_MeshBounds.YRes": g, "FTLE_MeshBounds.ZRes": g})
    nthr = threads if threads > 0 else (os.cpu_count() or 1)
    old = os.environ.get("ORC_DUMP_STATE")
    os.environ["ORC_DUMP_STATE"] = dump or ""
    try:
        rc, secs, steps, err = oracle_lib.run(inp, nthr)
    finally:
        if old is None:
            del os.environ["ORC_DUMP_STATE"]
        else:
            os.environ["ORC_DUMP_STATE"] = old
    if rc:
        raise RuntimeError(f"oracle failed: {err}")
    return steps / secs, steps, secs, nthr, out


def run_reference(args, rank, world):
    if rank != 0:
        return
    inputs = make_inputs(args.cube)
    with tempfile.TemporaryDirectory() as td:
        for _ in range(args.warmup):
            cpu_window(inputs, args.grid, args.cpu_threads, td)
        steps_tot, secs_tot = 0, 0.0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v, st, secs, nthr, _ = cpu_window(inputs, args.grid, args.cpu_threads, td)
            steps_tot += st
            secs_tot += secs
        wall = time.perf_counter() - t0
    value = steps_tot / secs_tot
    line = {
        "impl": "reference", "metric": "RK4 particle-steps/s", "value": value, "unit": "steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"FTLE {args.grid}^3 seeds over T={T_WINDOW}, {args.cube}^3x6 jittered Kuhn tets "
                               f"({6 * args.cube ** 3} tets), ABC flow {NFRAMES} frames, RK4 h={H}",
                   "l2": "inputs larger than L2 (frames 51 x 8.8 MB + 420 MB of grid state)",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": nthr, "kind": "port",
                         "sample": f"the whole window: FTLE {args.grid}^3 over T={T_WINDOW} (50 intervals), "
                                   "advection phase timed"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ parity

def parity_against_oracle(state, wT, wN, orc_dump, orc_out):
    """A GPU window's final grid state and FTLE fields against the oracle's
    run of the same window (its ORC_DUMP_STATE file and output fields)."""
    f = os.path.join(orc_dump, "state.0.bin")
    a = np.fromfile(f, np.uint8)
    n = int(a[:4].view(np.int32)[0])
    X = a[4:4 + 24 * n].view(np.float64).reshape(n, 3)
    ia = a[4 + 24 * n:].view(np.int32).reshape(3, n)
    live = ia[1] == 0
    res = {"points": n,
           "positions_differing": int((X != state["X"]).any(1).sum()),
           "left_differing": int((ia[1] != state["left"]).sum()),
           "have_differing": int(((ia[2] != 0) != (state["have"] != 0)).sum()),
           "eid_differing": int((ia[0][live] != state["eid"][live]).sum())}
    worst = 0.0
    for name, got in (("ftle.0.bin", wT), ("ftle_noT.0.bin", wN)):
        ref = np.fromfile(os.path.join(orc_out, name), "<f8")[1:]
        worst = max(worst, float((np.abs(got - ref) / np.maximum(np.abs(ref), 1e-13)).max()))
    res["ftle_max_rel"] = worst
    res["bitexact"] = not any(res[k] for k in ("positions_differing", "left_differing", "have_differing",
                                                "eid_differing"))
    return res


def parity_against_ompvc(case, wT, wN, time_stamp):
    """FTLE fields of a GPU window against ompVC's outputs for the same
    inputs, through the committed summaries (every 509th value, block sums);
    None when the fixture is missing."""
    try:
        import scale_cases as sc
        meta, arrays = sc.load_fixture()
    except (OSError, KeyError, ValueError):
        return None
    if case not in meta.get("cases", {}):
        return None
    worst, blocks_bad = 0.0, 0
    for name, v in (("ftle.0.bin", wT), ("ftle_noT.0.bin", wN)):
        ref = arrays[f"{case}:{name}:sub"]
        sub = v[::sc.STRIDE]
        if len(sub) != len(ref):
            return {"error": "size differs from ompVC's output"}
        worst = max(worst, float((np.abs(sub - ref) / np.maximum(np.abs(ref), 1e-13)).max()))
        nb = len(v) // sc.BLOCK
        blk = v[:nb * sc.BLOCK].reshape(nb, sc.BLOCK).sum(1)
        tol = 1e-12 * arrays[f"{case}:{name}:absblk"] + sc.BLOCK * 1e-13
        blocks_bad += int((np.abs(blk - arrays[f"{case}:{name}:blk"]) > tol).sum())
    return {"ftle_max_rel_strided": worst, "block_sums_outside_1e-12": blocks_bad,
            "time_stamp_matches": meta["cases"][case]["files"]["ftle.0.bin"]["time"] == time_stamp,
            "within_1e-12": worst <= 1e-12 and blocks_bad == 0}


# ------------------------------------------------------------------ double gyre

def dg_frames():
    """Config 1's frames in memory, exactly as synth.make_double_gyre_case
    writes them: nodes in (j, i) order with i fastest, w = 0."""
    import synth
    xs, ys = np.linspace(0.0, 2.0, DG_NX), np.linspace(0.0, 1.0, DG_NY)
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    out = []
    for n in range(DG_FRAMES):
        u, v = synth.double_gyre(X, Y, n * DG_DT)
        out.append(np.ascontiguousarray(np.stack([u, v, np.zeros_like(u)], -1).reshape(-1, 3)))
    return out


def bench_double_gyre(args, stream_of, barrier, fp64, rank):
    """Config 1 on the GPU: the double gyre's FTLE window (Cartesian 2D,
    FP64) timed with CUDA events over args.steps windows after one warm-up;
    one more window checked against the oracle and ompVC; the oracle on the
    same window on the host cores (rank 0)."""
    import torch

    import flow
    import fvc
    import synth
    frames = dg_frames()
    ax = flow.TimeAxis(0.0, DG_DT, DG_FRAMES, 0)
    ctx = fvc.Context(2, 0)
    ctx.set_cart_mesh(0.0, 2.0, DG_NX, 0.0, 1.0, DG_NY, 0.0, 0.0, 1)
    ctx.set_bounds([0.0, 2.0, 0.0, 1.0, 0.0, 0.0])
    ctx.set_integrator(1, DG_H, 0)
    flow.upload_frames(ctx, ax, frames)
    stream = stream_of(ctx)
    npts = DG_GRID[6] * DG_GRID[7]
    for _ in range(max(1, min(args.warmup, 3))):
        flow.run_ftle(ctx, ax, DG_GRID, DG_T)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps, stats = 0, []
    e0.record(stream)
    for _ in range(args.steps):
        wT, wN, st, js = flow.run_ftle(ctx, ax, DG_GRID, DG_T, fetch=False)
        steps += st
        stats.append(js)
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1)
    ms_main = sum(x["ms_main"] for x in stats)
    steps_main = sum(x["steps_main"] for x in stats)
    achieved = steps_main * DG_BYTES_PER_STEP / (ms_main / 1e3) / 1e9 if ms_main > 0 else 0.0
    peak, peak_kind = measured_peak()
    out = {"workload": f"double gyre, {DG_NX}x{DG_NY} nodes, {DG_FRAMES} frames dt={DG_DT}; FTLE "
                       f"{DG_GRID[6]}x{DG_GRID[7]} seeds over [0,2]x[0,1], T={DG_T}, RK4 h={DG_H}, f64",
           "value": steps / (ms / 1e3), "unit": "steps/s", "ms_per_step": ms / args.steps,
           "ftle_points_per_s": npts * args.steps / (ms / 1e3),
           "steps_per_window": steps / args.steps,
           "phases_ms_per_step": {k: sum(x[k] for x in stats) / args.steps
                                  for k in ("ms_setup", "ms_main", "ms_early", "ms_reduce")}}
    # the FP64 pipe bounds this kernel too (ops per step from the committed
    # ncu summary); the HBM figure beside it
    hbm = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "peak_source": peak_kind, "bytes_per_step": DG_BYTES_PER_STEP}
    _, prof = profiled_traffic()
    ops = (prof or {}).get("cart2_fp64_pipe_ops_per_step")
    if ops and fp64 and ms_main > 0:
        r = ops * steps_main / (ms_main / 1e3)
        out["roofline"] = {"bound": "fp64", "achieved": r / 1e9, "peak": fp64["fma_per_s"] / 1e9,
                           "unit": "G FP64-pipe instructions/s", "frac": r / fp64["fma_per_s"],
                           "peak_source": "measured in this run (tests/cuda/fp64_rate.cu, FP64 FMA rate)",
                           "ops_per_step": ops, "kernel": "k_ftle_pass1 (Cartesian 2D)", "hbm": hbm}
    else:
        out["roofline"] = dict(hbm, kernel="k_ftle_pass1 (Cartesian 2D)")
    if rank == 0 and not args.no_cpu:
        state = {}
        wT, wN, _, _ = flow.run_ftle(ctx, ax, DG_GRID, DG_T, state=state)
        with tempfile.TemporaryDirectory() as td:
            d = os.path.join(td, "dg")
            c = synth.make_double_gyre_case(d, nx=DG_NX, ny=DG_NY, nframes=DG_FRAMES, dt=DG_DT, prefix="dg")
            o, dump = os.path.join(td, "out"), os.path.join(td, "dump")
            os.makedirs(o)
            os.makedirs(dump)
            inp = os.path.join(td, "dg.in")
            synth.write_in_file(inp, **dict(c.params, Path_Output=o + "/", FTLE_Compute=1, FTLE_IntTLength=DG_T,
                                            Int_TimeStep=DG_H, **{
                                                "FTLE_MeshBounds.XMin": DG_GRID[0], "FTLE_MeshBounds.XMax": DG_GRID[1],
                                                "FTLE_MeshBounds.YMin": DG_GRID[2], "FTLE_MeshBounds.YMax": DG_GRID[3],
                                                "FTLE_MeshBounds.ZMin": 0.0, "FTLE_MeshBounds.ZMax": 0.0,
                                                "FTLE_MeshBounds.XRes": DG_GRID[6], "FTLE_MeshBounds.YRes": DG_GRID[7],
                                                "FTLE_MeshBounds.ZRes": 1}))
            import oracle_lib
            nthr = args.cpu_threads if args.cpu_threads > 0 else (os.cpu_count() or 1)
            os.environ["ORC_DUMP_STATE"] = dump
            try:
                rc, secs, csteps, err = oracle_lib.run(inp, nthr)
            finally:
                del os.environ["ORC_DUMP_STATE"]
            if rc:
                raise RuntimeError(f"oracle failed on the double gyre: {err}")
            out["cpu_baseline"] = {"value": csteps / secs, "unit": "steps/s", "cores": nthr, "kind": "port",
                                   "sample": f"the same window, {csteps} steps in {secs:.2f} s of advection"}
            out["parity"] = {"vs_oracle": parity_against_oracle(state, wT, wN, dump, o),
                             "vs_ompvc": parity_against_ompvc("dg_ftle", wT, wN, 0.0)}
    ctx.close()
    return out


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
                       "positions output every 10 steps (21 outputs, each copied to host memory by a writer "
                       "thread)"}
    finals = {}
    for prec in ("fp64", "bf16"):
        ctx = fvc.Context(3, 1)
        ctx.set_unstruct_mesh(xyz, conn, adj)
        ctx.set_bounds([0, 1, 0, 1, 0, 1])
        ctx.set_integrator(1, H, 0)
        ctx.set_precision(prec)
        flow.upload_frames(ctx, ax, frames)
        flow.run_tracers(ctx, ax, seeds[:4096], 0.0, 0.05, 21)          # warm-up
        flow.run_tracers(ctx, ax, seeds[:4096], 0.0, 0.05, 21, asynchronous=False)
        # one short release of the full size: the context's output ring is
        # sized to the largest release it has seen (allocated once)
        flow.run_tracers(ctx, ax, seeds, 0.0, 0.05, 2)
        # the blocking loop (each advance waits, each output is a blocking
        # compact-and-copy), for comparison
        t0 = time.perf_counter()
        outs_b, steps_b, _ = flow.run_tracers(ctx, ax, seeds, 0.0, 0.05, 21, asynchronous=False)
        wall_b = time.perf_counter() - t0
        # the release loop as it runs: advances queued, outputs through the
        # output ring to a writer thread that copies each into host memory
        t0 = time.perf_counter()
        phases = {}
        outs, steps, st = flow.run_tracers(ctx, ax, seeds, 0.0, 0.05, 21, timings=phases)
        wall = time.perf_counter() - t0
        # the final state for the error figures, from one more (untimed) run:
        # the release's own outputs are the 21 position files above
        fin = {}
        flow.run_tracers(ctx, ax, seeds, 0.0, 0.05, 21, state=fin)
        finals[prec] = fin
        same = len(outs) == len(outs_b) and all(np.array_equal(x, y) for x, y in zip(outs, outs_b))
        out[prec] = {"value": steps / wall, "unit": "steps/s", "steps": int(steps), "wall_s": wall,
                     "kernel_s": st["ms_main"] / 1e3,
                     "kernel_value": st["steps_main"] / (st["ms_main"] / 1e3) if st["ms_main"] > 0 else None,
                     "wall_over_kernel": wall / (st["ms_main"] / 1e3) if st["ms_main"] > 0 else None,
                     "blocking_wall_s": wall_b, "blocking_value": steps_b / wall_b,
                     "outputs_identical_to_blocking": bool(same and steps == steps_b),
                     "host_phases_s": phases, "seeding_ms_device": st["ms_setup"],
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
    out["speedup_vs_fp64"] = out["bf16"]["value"] / out["fp64"]["value"] if out["fp64"]["value"] else None
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
    out["speedup_vs_fp64"] = out["bf16"]["value"] / out["fp64"]["value"] if out["fp64"]["value"] else None
    import serve as _s
    out["bf16"]["errors_vs_fp64"] = _s.endpoint_errors(res["fp64"], res["bf16"])
    return out


def bench_served(args, tube, frames, cube_inputs):
    """The served workload: a Poisson request stream over both resident data
    sets for args.served_seconds at args.served_rate requests/s, 50% tracer
    releases on the tube (1e3-1e6 seeds, log-uniform), 40% FTLE grids on the
    cube (32^3-128^3), 10% residence-time releases on the tube (1e5 seeds, 3
    periods); admission by an HBM budget; latency from arrival to results on
    the host.  The same stream is served in the BF16 form and in the FP64
    form; a form that cannot keep up is stopped after the arrival window plus
    a grace period and reported as such (finished requests' latencies, the
    backlog).  args.served_sweep adds, per form, shorter streams at a range of
    rates and the highest rate that was sustained."""
    import serve
    xyz, conn, adj, cframes = cube_inputs
    frame_bytes = 32 * (len(tube.xyz) * serve.TUBE_FRAMES + len(xyz) * len(cframes))
    budget = max((SERVED_BUDGET - frame_bytes) // 2, 1)

    def run(prec, rate, duration, limit, seed=7):
        reqs = serve.poisson_requests(tube, rate=rate, duration=duration, seed=seed)
        sites = {"tube": serve.tube_site(prec, tube=tube, frames=frames, hbm_budget=budget),
                 "cube": serve.cube_site(prec, mesh=(xyz, conn, adj), frames=cframes, hbm_budget=budget)}
        serve.warm_pairs(sites["tube"])
        serve.run_batched(sites["cube"], [("ftle", (0, 1, 0, 1, 0, 1, 8, 8, 8), 0.0, 1.0)], graph=False, tune=False)
        r = serve.serve(sites, reqs, time_limit=limit, censor=True)
        r["offered_rate"] = rate
        r["sustained"] = serve.sustained(r, reqs, duration)
        for st in sites.values():
            st.close()
        return r

    out = {"workload": f"Poisson {args.served_rate:g} requests/s for {args.served_seconds:g} s: 50% tracer releases "
                       "(tube, 1e3-1e6 seeds log-uniform, 0.2-2 periods, +-direction), 40% FTLE grids (cube, "
                       "32^3-128^3, T=1), 10% residence time (tube, 1e5 seeds, 3 periods)",
           "hbm_budget_bytes": SERVED_BUDGET}
    limits = {"bf16": args.served_seconds + 240.0, "fp64": args.served_seconds + 30.0}
    forms = [f for f in ("bf16", "fp64") if f in args.served_forms.split(",")]
    for prec in forms:
        out[prec] = run(prec, args.served_rate, args.served_seconds, limits[prec])
        out["requests"] = out[prec].get("requests_total", out[prec]["requests"])
    if "bf16" in out and "fp64" in out:
        out["speedup_vs_fp64"] = (out["bf16"]["steps_per_s"] / out["fp64"]["steps_per_s"]
                                  if out["fp64"]["steps_per_s"] else None)
    if args.served_sweep:
        sweep = {}
        for prec, rates in (("bf16", (25, 50, 100, 125, 150, 175, 200)), ("fp64", (1, 2, 5, 10, 20))):
            rows = []
            for rate in rates:
                r = run(prec, rate, args.sweep_seconds, args.sweep_seconds + 20.0, seed=11)
                rows.append({k: r.get(k) for k in ("offered_rate", "requests", "requests_unfinished", "steps_per_s",
                                                  "p50_ms", "p95_ms", "p99_ms", "sustained")})
            ok = [x["offered_rate"] for x in rows if x["sustained"]]
            sweep[prec] = {"rows": rows, "max_sustained_rate": max(ok) if ok else None}
        out["rate_sweep"] = sweep
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


def ftle_error_by_time(ref_T, ref_N, got_T):
    """FTLE error (relative to the largest FP64 value) binned by each
    point's FTLE integration time |MinExitTime - StartTime| = FTLEwoT /
    FTLEwT of the FP64 window: early FTLE divides by that time, so short
    times amplify any change of the stretching."""
    scale = float(np.abs(ref_T).max()) or 1.0
    e = np.abs(got_T - ref_T) / scale
    with np.errstate(divide="ignore", invalid="ignore"):
        teff = np.where(ref_T != 0, np.abs(ref_N / ref_T), np.nan)
    out = []
    for lo, hi in ((0.0, 0.05), (0.05, 0.1), (0.1, 0.25), (0.25, 0.5), (0.5, 1.0 + 1e-9)):
        m = (teff >= lo) & (teff < hi)
        if m.any():
            out.append({"T_from": lo, "T_to": min(hi, 1.0), "points": int(m.sum()), "max": float(e[m].max()),
                        "rms": float(np.sqrt((e[m] ** 2).mean())), "p99": float(np.quantile(e[m], 0.99))})
    m = np.isnan(teff)
    if m.any():
        out.append({"T_from": None, "T_to": None, "points": int(m.sum()), "note": "FP64 FTLE is 0 (lambda <= 1)",
                    "max": float(e[m].max())})
    return out


def precision_forms(ctx, ax, grid, stream, barrier, args, fp64_value, ref, inputs):
    """BF16 and FP16 frames with FP32 stages (fvc_set_precision) on the same
    context and workload: one warm-up window, then args.steps timed windows
    with CUDA events; errors against ref = (FTLE field, FTLE-without-time
    field, final state) of an FP64 window.  The error is split by source:
    the FP64 form run on frames quantised and dequantised on the host
    (tests/quantise.py) carries the storage error alone; the mixed form
    against that run carries the FP32 arithmetic (and the mixed form's reuse
    of the main pass's record)."""
    import torch

    import flow
    import fvc
    import quantise
    ref_T, ref_N, ref_state = ref
    xyz, conn, adj, frames = inputs
    out = {}
    for name in ("bf16", "fp16"):
        ctx.set_precision(name)
        flow.run_ftle(ctx, ax, grid, T_WINDOW)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps, stats, st_last, T_last = 0, [], {}, None
        e0.record(stream)
        for k in range(args.steps):
            wT, wN, st, js = flow.run_ftle(ctx, ax, grid, T_WINDOW, fetch=False)
            steps += st
            stats.append(js)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        got_state = {}
        T_last = flow.run_ftle(ctx, ax, grid, T_WINDOW, state=got_state)[0]
        value = steps / (ms / 1000.0)
        # the storage error alone: the FP64 form on the 16-bit frames
        cq = fvc.Context(3, 1)
        cq.set_unstruct_mesh(xyz, conn, adj)
        cq.set_bounds([0, 1, 0, 1, 0, 1])
        cq.set_integrator(1, H, 0)
        flow.upload_frames(cq, ax, [quantise.dequantised(f, name) for f in frames])
        q_state = {}
        q_T = flow.run_ftle(cq, ax, grid, T_WINDOW, state=q_state)[0]
        cq.close()
        total = form_errors((ref_T, ref_state), (T_last, got_state))
        out[name] = {"value": value, "unit": "steps/s", "ms_per_step": ms / args.steps,
                     "ftle_points_per_s": args.grid ** 3 * args.steps / (ms / 1000.0),
                     "speedup_vs_fp64": value / fp64_value,
                     "steps_early_recorded_per_step": sum(x["steps_early_recorded"] for x in stats) / args.steps,
                     "phases_ms_per_step": {k: sum(s[k] for s in stats) / args.steps
                                            for k in ("ms_setup", "ms_main", "ms_early", "ms_reduce")},
                     "errors": total,
                     "ftle_max_rel_target": 1e-3,
                     "ftle_max_rel_to_max_achieved": total["ftle_max_rel_to_max"],
                     "errors_by_source": {
                         "storage": form_errors((ref_T, ref_state), (q_T, q_state)),
                         "arithmetic": form_errors((q_T, q_state), (T_last, got_state)),
                         "ftle_by_time_total": ftle_error_by_time(ref_T, ref_N, T_last),
                         "ftle_by_time_storage": ftle_error_by_time(ref_T, ref_N, q_T)}}
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

    fp64 = probe_fp64(local_rank)
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
            # the fields stay in HBM here; the end-to-end loop reads them back
            wT, wN, st, js = flow.run_ftle(ctx, ax, grid, T_WINDOW, fetch=False)
            steps_total += st
            stats.append(js)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    clocks = clk.summary()
    secs = ms / 1000.0
    secs_max, steps_all = reduce_over_ranks(secs, steps_total, world)
    steps_recorded = sum(s["steps_early_recorded"] for s in stats)
    steps_computed = steps_total - steps_recorded
    secs_c, steps_computed_all = reduce_over_ranks(secs, steps_computed, world)

    # roofline of the main advection kernel from its CUDA-event times: the
    # FP64 pipe (the bound that applies), and the HBM figure beside it
    ms_main = sum(s["ms_main"] for s in stats)
    steps_main = sum(s["steps_main"] for s in stats)
    launches_main = sum(s["intervals"] for s in stats)
    peak, peak_kind = measured_peak()
    achieved = (steps_main * BYTES_PER_STEP) / (ms_main / 1000.0) / 1e9 if ms_main > 0 else 0.0
    traffic_per_step, prof = profiled_traffic()
    traffic = traffic_per_step * steps_main / launches_main if traffic_per_step else None
    hbm = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "traffic": traffic, "peak_source": peak_kind, "bytes_per_step": BYTES_PER_STEP}
    ops_per_step = (prof or {}).get("fp64_pipe_ops_per_step")
    if ops_per_step and fp64 and ms_main > 0:
        ops = ops_per_step * steps_main / (ms_main / 1000.0)
        roofline = {"bound": "fp64", "achieved": ops / 1e9, "peak": fp64["fma_per_s"] / 1e9,
                    "unit": "G FP64-pipe instructions/s", "frac": ops / fp64["fma_per_s"], "traffic": traffic,
                    "peak_source": "measured in this run (tests/cuda/fp64_rate.cu, FP64 FMA rate)",
                    "ops_per_step": ops_per_step, "kernel": "k_ftle_pass1", "hbm": hbm}
    else:
        roofline = dict(hbm, kernel="k_ftle_pass1")
    gpu_launches = int(sum(s["launches"] for s in stats))

    # one more FP64 window, kept for the parity check and as the mixed forms'
    # reference
    ref_state = {}
    ref_T, ref_N, _, _ = flow.run_ftle(ctx, ax, grid, T_WINDOW, state=ref_state)

    # the mixed-precision forms on the same workload, against this FP64 window
    forms = None
    if not args.no_precision:
        forms = precision_forms(ctx, ax, grid, stream, barrier, args, steps_all / secs_max,
                                (ref_T, ref_N, ref_state), inputs)

    # end to end through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        pxyz, pconn, padj = pin(xyz), pin(conn), pin(adj)
        pframes = [pin(f) for f in frames]
        h2d = pxyz.nbytes + pconn.nbytes + padj.nbytes + sum(f.nbytes for f in pframes)
        d2h = 2 * 8 * npts
        # the context stays (as an application keeps it); every step sends
        # the mesh (validated, its records and bucket grid rebuilt on the
        # device) and all frames up again and reads both FTLE fields back
        # the fields come back into page-locked arrays the application keeps
        pin = (fvc.PinnedArray((args.grid ** 3,)), fvc.PinnedArray((args.grid ** 3,)))
        barrier()
        t0 = time.perf_counter()
        e2e_steps = 0
        for _ in range(args.steps):
            ctx.set_unstruct_mesh(pxyz, pconn, padj)
            flow.upload_frames(ctx, ax, pframes, asynchronous=True)
            wT, wN, st, _ = flow.run_ftle(ctx, ax, grid, T_WINDOW, out=(pin[0].a, pin[1].a))
            e2e_steps += st
        barrier()
        ctx.close()
        e2e_secs, e2e_all = reduce_over_ranks(time.perf_counter() - t0, e2e_steps, world)
        e2e = {"value": e2e_all / e2e_secs, "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
    else:
        ctx.close()

    dg = None
    if not args.no_dg:
        dg = bench_double_gyre(args, lambda c: torch.cuda.ExternalStream(c.stream()), barrier, fp64, rank)

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

    # the CPU oracle on the same window, and the parity of the FP64 window
    cpu = parity = None
    if rank == 0 and not args.no_cpu:
        with tempfile.TemporaryDirectory() as td:
            dump = os.path.join(td, "state")
            os.makedirs(dump)
            v, st, s2, nthr, out_dir = cpu_window(inputs, args.grid, args.cpu_threads, td, dump=dump)
            parity = {"vs_oracle": parity_against_oracle(ref_state, ref_T, ref_N, dump, out_dir)}
        cpu = {"value": v, "unit": "steps/s", "cores": nthr, "kind": "port",
               "sample": f"the whole window: FTLE {args.grid}^3 over T={T_WINDOW} (50 intervals), {st} steps in "
                         f"{s2:.2f} s of advection"}
    if rank == 0 and args.grid == 128 and args.cube == CUBE_N:
        parity = parity or {}
        parity["vs_ompvc"] = parity_against_ompvc("cube_ftle", ref_T, ref_N, 0.0)

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
            "steps_computed": int(steps_computed), "steps_computed_per_s": steps_computed_all / secs_c,
            "steps_main": int(steps_main), "steps_early": int(sum(s["steps_early"] for s in stats)),
            "steps_early_recorded": int(steps_recorded),
            "roofline": roofline,
            "gpu_launches": gpu_launches,
            "parity": parity,
            "precision_forms": forms,
            "double_gyre": dg,
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
        if parity and parity.get("vs_oracle"):
            line["parity"]["summary"] = "bitexact" if parity["vs_oracle"]["bitexact"] else "MISMATCH"
        print(json.dumps(line), flush=True)


def probe_advect(npts):
    """The step-level workload of --probe-advect; prints each call's steps."""
    import fvc
    import synth
    import build as fvc_build
    fvc_build.build()
    xyz, conn, adj = synth.kuhn_cube_mesh(32, jitter=0.2, seed=0)
    g = fvc.Context(3, 1)
    g.set_unstruct_mesh(xyz, conn, adj)
    g.set_bounds([0, 1, 0, 1, 0, 1])
    g.upload_frame(0, synth.abc_flow(xyz, 0.0))
    g.upload_frame(1, synth.abc_flow(xyz, 0.02))
    g.set_window(0, 1, 0.0, 0.02)
    g.set_integrator(1, H, 0)
    P = np.random.default_rng(0).uniform(0.05, 0.95, size=(npts, 3))
    eid = g.global_search(P)
    left = (eid < 0).astype(np.int32)
    for call in range(2):
        a = [P.copy(), np.zeros_like(P), eid.copy(), left.copy(), np.zeros(npts)]
        steps = g.advect(*a, 0.0, 0.02)
        print(json.dumps({"probe_advect_call": call, "steps": int(steps), "left": int(a[3].sum())}), flush=True)
    g.close()


def main():
    args = parse()
    if args.probe_advect:
        probe_advect(args.probe_advect)
        return
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
