"""Drivers of the batched and served forms (fvc_batch_* through fvc.Batch).

batched    a fixed set of jobs run to completion (optionally tuned and as one
           CUDA graph): the pulsatile bent-tube batch of tracer releases with
           uneven seed counts and windows.
served     a request stream: jobs arrive at Poisson times and are submitted
           when they arrive; each site's batch is ticked continuously, so
           requests join ticks already running, and a request's latency runs
           from its arrival to its results being on the host.

All computation happens in libfvc on the GPU; this module only generates
inputs, submits, ticks and reads results.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

import flow
import fvc
import synth

TUBE_PERIOD = 1.0
TUBE_FRAMES = 101          # 100 frames a period plus the closing frame (periodic data)


@dataclass
class Site:
    """One resident data set: context, time axis and its batch."""
    name: str
    ctx: fvc.Context
    ax: flow.TimeAxis
    batch: fvc.Batch = None
    tube: synth.Tube = None

    def close(self):
        if self.batch:
            self.batch.close()
        self.ctx.close()


def tube_site(prec="bf16", nc=40, nax=320, h=0.002, hbm_budget=0, tube=None, frames=None, resort_every=-1):
    """The bent tube (3,072,000 tets at nc = 40, nax = 320) with Womersley
    frames over one period, resident on a new context."""
    if tube is None:
        tube = synth.bent_tube_mesh(nc=nc, nax=nax)
    if frames is None:
        _, frames = synth.womersley_frames(tube, nframes=TUBE_FRAMES, period=TUBE_PERIOD)
    ctx = fvc.Context(3, 1)
    ctx.set_unstruct_mesh(tube.xyz, tube.conn, tube.adj)
    ctx.set_bounds(tube.bounds())
    ctx.set_integrator(1, h, 0)
    ctx.set_precision(prec)
    ax = flow.TimeAxis(0.0, TUBE_PERIOD / (TUBE_FRAMES - 1), TUBE_FRAMES, 1)
    flow.upload_frames(ctx, ax, frames)
    site = Site("tube", ctx, ax, tube=tube)
    site.batch = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, ax.periodic, hbm_budget=hbm_budget,
                           resort_every=resort_every)
    return site


def cube_site(prec="bf16", n=64, h=0.005, nframes=51, dt=0.02, hbm_budget=0, mesh=None, frames=None):
    """The jittered Kuhn cube with ABC frames (the FTLE workload's data)."""
    if mesh is None:
        mesh = synth.kuhn_cube_mesh(n, jitter=0.2, seed=0)
    xyz, conn, adj = mesh
    if frames is None:
        frames = [synth.abc_flow(xyz, k * dt) for k in range(nframes)]
    ctx = fvc.Context(3, 1)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, h, 0)
    ctx.set_precision(prec)
    ax = flow.TimeAxis(0.0, dt, nframes, 0)
    flow.upload_frames(ctx, ax, frames)
    site = Site("cube", ctx, ax)
    site.batch = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, ax.periodic, hbm_budget=hbm_budget)
    return site


def warm_pairs(site):
    """Two short releases covering the whole period forwards and backwards, so
    every frame pair's quantised records exist before anything is timed."""
    tube = site.tube
    s = 0.5 * tube.length
    jobs = [("tracers", synth.tube_cross_section_seeds(tube, 64, s, seed=1), 0.0, TUBE_PERIOD),
            ("tracers", synth.tube_cross_section_seeds(tube, 64, s, seed=2), TUBE_PERIOD, 0.0)]
    run_batched(site, jobs, graph=False, tune=False)


# ---------------------------------------------------------------- batched

def tube_batch_jobs(tube, njobs=64, nmin=1e3, nmax=1e6, seed=0):
    """The batch of tracer releases on the tube: seed counts log-uniform in
    [nmin, nmax] on random axial cross-sections, windows of U[0.2, 2]
    periods from a random start, forward or backward with probability 1/2."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(njobs):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        s = rng.uniform(0.05 * tube.length, 0.95 * tube.length)
        t0 = float(rng.uniform(0.0, TUBE_PERIOD))
        T = float(rng.uniform(0.2, 2.0)) * TUBE_PERIOD
        d = 1 if rng.uniform() < 0.5 else -1
        seeds = synth.tube_cross_section_seeds(tube, n, s, seed=seed * 1000 + k)
        jobs.append(("tracers", seeds, t0, t0 + d * T))
    return jobs


def submit(batch, job):
    kind, arg, t0, t1 = job
    if kind == "ftle":
        return batch.submit_ftle(arg, t0, t1)
    return batch.submit_tracers(arg, t0, t1, residence=kind == "residence")


def run_batched(site, jobs, graph=True, tune=True, results=False):
    """Runs the jobs as one batch; returns (steps, device seconds, wall
    seconds, batch stats, results or None)."""
    b = site.batch
    before = b.stats()
    t0 = time.perf_counter()
    ids = [submit(b, j) for j in jobs]
    if tune:
        b.autotune()
    b.run(graph=graph)
    wall = time.perf_counter() - t0
    st = b.stats()
    steps = 0
    for i in ids:
        js = b.job_stats(i)
        steps += js["steps_main"] + js["steps_early"]
    out = [b.tracer_result(i) for i in ids] if results else None
    for i in ids:
        b.release(i)
    secs = (st["ms_run"] - before["ms_run"]) / 1000.0
    return steps, secs, wall, st, out


def endpoint_errors(ref, got):
    """Endpoint error of the mixed form against the FP64 form over tracers
    whose exit status agrees; element-id and exit-status mismatch rates."""
    d, same_all, eid_bad, n_same = [], 0, 0, 0
    for r, g in zip(ref, got):
        same = r["left"] == g["left"]
        same_all += int(same.sum())
        if same.any():
            d.append(np.linalg.norm(g["X"][same] - r["X"][same], axis=1))
            eid_bad += int((g["eid"][same] != r["eid"][same]).sum())
            n_same += int(same.sum())
    d = np.concatenate(d) if d else np.zeros(1)
    ntot = sum(len(r["left"]) for r in ref)
    return {"endpoint_max": float(d.max()), "endpoint_rms": float(np.sqrt((d ** 2).mean())),
            "eid_mismatch_rate": eid_bad / max(n_same, 1), "left_mismatch_rate": 1.0 - same_all / max(ntot, 1)}


# ---------------------------------------------------------------- served

@dataclass
class Request:
    t_arrive: float
    site: str
    job: tuple
    kind: str
    npts: int
    t_done: float = None
    jid: int = None
    steps: int = 0
    result: object = None


def poisson_requests(tube, rate=200.0, duration=10.0, mix=(0.5, 0.4, 0.1), seed=0, tracer_range=(1e3, 1e5),
                     ftle_edges=(16, 48), rt_seeds=10_000, rt_periods=3.0, ftle_T=1.0):
    """Arrivals at Poisson times over `duration` seconds: tracer releases on the
    tube (seed counts log-uniform in tracer_range, windows as the batch's),
    FTLE grids on the cube (edge uniform in ftle_edges, forward over ftle_T)
    and residence-time releases on the tube (rt_seeds seeds, rt_periods
    periods), in the proportions of mix."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        u = rng.uniform()
        if u < mix[0]:
            n = int(round(math.exp(rng.uniform(math.log(tracer_range[0]), math.log(tracer_range[1])))))
            s = rng.uniform(0.05 * tube.length, 0.95 * tube.length)
            t0 = float(rng.uniform(0.0, TUBE_PERIOD))
            T = float(rng.uniform(0.2, 2.0)) * TUBE_PERIOD
            d = 1 if rng.uniform() < 0.5 else -1
            seeds = synth.tube_cross_section_seeds(tube, n, s, seed=int(rng.integers(1 << 30)))
            reqs.append(Request(t, "tube", ("tracers", seeds, t0, t0 + d * T), "tracers", n))
        elif u < mix[0] + mix[1]:
            e = int(rng.integers(ftle_edges[0], ftle_edges[1] + 1))
            reqs.append(Request(t, "cube", ("ftle", (0, 1, 0, 1, 0, 1, e, e, e), 0.0, ftle_T), "ftle", e ** 3))
        else:
            s = rng.uniform(0.05 * tube.length, 0.5 * tube.length)
            t0 = float(rng.uniform(0.0, TUBE_PERIOD))
            seeds = synth.tube_cross_section_seeds(tube, rt_seeds, s, seed=int(rng.integers(1 << 30)))
            reqs.append(Request(t, "tube", ("residence", seeds, t0, t0 + rt_periods * TUBE_PERIOD), "residence",
                                rt_seeds))
    return reqs


def serve(sites, requests, keep_results=False, time_limit=600.0):
    """Serves the requests in arrival order against the sites' batches.

    The loop submits every request whose arrival time has passed, ticks each
    site's batch (a tick enqueues one frame interval of every admitted job
    and returns; at most two are in flight per site, and the sites' streams
    run concurrently), and collects finished jobs: results copied to the
    host, the job released, its latency recorded.  Returns a summary dict."""
    pending = sorted(requests, key=lambda r: r.t_arrive)
    nxt = 0
    running = {name: {} for name in sites}
    done = []
    t0 = time.perf_counter()
    while len(done) < len(pending):
        now = time.perf_counter() - t0
        if now > time_limit:
            raise RuntimeError(f"serving did not finish within {time_limit} s")
        while nxt < len(pending) and pending[nxt].t_arrive <= now:
            r = pending[nxt]
            r.jid = submit(sites[r.site].batch, r.job)
            running[r.site][r.jid] = r
            nxt += 1
        busy = False
        for name, site in sites.items():
            if not running[name]:
                continue
            busy = True
            b = site.batch
            b.tick()
            for jid in list(running[name]):
                if b.poll(jid) == fvc.BATCH_DONE:
                    r = running[name].pop(jid)
                    if r.kind == "ftle":
                        res = b.ftle_result(jid)
                    elif r.kind == "residence":
                        res = b.residence_result(jid)
                    else:
                        res = b.tracer_result(jid)
                    js = b.job_stats(jid)
                    r.steps = js["steps_main"] + js["steps_early"]
                    r.t_done = time.perf_counter() - t0
                    if keep_results:
                        r.result = res
                    b.release(jid)
                    done.append(r)
        if not busy and nxt < len(pending):
            wait = pending[nxt].t_arrive - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.001))
    wall = time.perf_counter() - t0
    lat = np.array([r.t_done - r.t_arrive for r in done])
    steps = sum(r.steps for r in done)
    by_kind = {}
    for k in ("tracers", "ftle", "residence"):
        lk = np.array([r.t_done - r.t_arrive for r in done if r.kind == k])
        if len(lk):
            by_kind[k] = {"n": int(len(lk)), "p50_ms": 1e3 * float(np.percentile(lk, 50)),
                          "p99_ms": 1e3 * float(np.percentile(lk, 99))}
    return {"requests": len(done), "wall_s": wall, "steps": int(steps), "steps_per_s": steps / wall,
            "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p95_ms": 1e3 * float(np.percentile(lat, 95)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99)), "max_ms": 1e3 * float(lat.max()),
            "by_kind": by_kind}
