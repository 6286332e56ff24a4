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


# Releases advance ceil(intervals / TICK_INTERVALS) frame intervals per tick
# (fvc_batch_opts.tick_intervals), so a long release finishes in about as
# many ticks as a cube FTLE job of T = 1 (50 intervals) instead of holding
# its latency to one interval a tick.
TICK_INTERVALS = 48


def tube_site(prec="bf16", nc=40, nax=320, h=0.002, hbm_budget=0, tube=None, frames=None, resort_every=-1,
              tick_intervals=TICK_INTERVALS):
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
                           resort_every=resort_every, tick_intervals=tick_intervals)
    return site


def cube_site(prec="bf16", n=64, h=0.005, nframes=51, dt=0.02, hbm_budget=0, mesh=None, frames=None,
              tick_intervals=TICK_INTERVALS):
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
    site.batch = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, ax.periodic, hbm_budget=hbm_budget,
                           tick_intervals=tick_intervals)
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


class SectionSeeds:
    """n seeds on the tube's cross-section at axial position s, made when the
    request is submitted: a slice of one shared pool of points uniform in the
    disc of radius 1 - margin (tube_cross_section_seeds' distribution), mapped
    onto the section.  Keeps a stream of thousands of requests with up to a
    million seeds each from holding all their seeds in host memory at once."""
    _pool = None

    def __init__(self, tube, n, s, offset):
        self.tube, self.n, self.s, self.offset = tube, int(n), float(s), int(offset)

    @classmethod
    def pool(cls, size=1 << 20, margin=0.02, seed=12345):
        if cls._pool is None or len(cls._pool) < size:
            rng = np.random.default_rng(seed)
            rr = np.sqrt(rng.uniform(0.0, (1.0 - margin) ** 2, size))
            th = rng.uniform(0.0, 2 * math.pi, size)
            cls._pool = np.stack([rr * np.cos(th), rr * np.sin(th)], -1)
        return cls._pool

    def __call__(self):
        P = self.pool()
        idx = (self.offset + np.arange(self.n)) % len(P)
        C, T, N = synth.tube_centreline(np.array([self.s]), self.tube.length, self.tube.bend_radius)
        B = np.array([0.0, 1.0, 0.0])
        R = self.tube.radius
        return C[0] + R * (P[idx, 0:1] * N[0] + P[idx, 1:2] * B)


def submit(batch, job):
    kind, arg, t0, t1 = job
    if kind == "ftle":
        return batch.submit_ftle(arg, t0, t1)
    seeds = arg() if callable(arg) else arg
    return batch.submit_tracers(seeds, t0, t1, residence=kind == "residence")


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


def poisson_requests(tube, rate=200.0, duration=60.0, mix=(0.5, 0.4, 0.1), seed=0, tracer_range=(1e3, 1e6),
                     ftle_edges=(32, 128), rt_seeds=100_000, rt_periods=3.0, ftle_T=1.0):
    """Arrivals at Poisson times over `duration` seconds: tracer releases on the
    tube (seed counts log-uniform in tracer_range, windows as the batch's),
    FTLE grids on the cube (edge uniform in ftle_edges, forward over ftle_T)
    and residence-time releases on the tube (rt_seeds seeds, rt_periods
    periods), in the proportions of mix.  The defaults are the served
    workload's: 200 requests/s for 60 s, 1e3-1e6 tracer seeds, 32^3-128^3
    FTLE grids, 1e5-seed three-period residence-time releases.  Seeds are
    made at submission (SectionSeeds)."""
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
            seeds = SectionSeeds(tube, n, s, int(rng.integers(1 << 30)))
            reqs.append(Request(t, "tube", ("tracers", seeds, t0, t0 + d * T), "tracers", n))
        elif u < mix[0] + mix[1]:
            e = int(rng.integers(ftle_edges[0], ftle_edges[1] + 1))
            reqs.append(Request(t, "cube", ("ftle", (0, 1, 0, 1, 0, 1, e, e, e), 0.0, ftle_T), "ftle", e ** 3))
        else:
            s = rng.uniform(0.05 * tube.length, 0.5 * tube.length)
            t0 = float(rng.uniform(0.0, TUBE_PERIOD))
            seeds = SectionSeeds(tube, rt_seeds, s, int(rng.integers(1 << 30)))
            reqs.append(Request(t, "tube", ("residence", seeds, t0, t0 + rt_periods * TUBE_PERIOD), "residence",
                                rt_seeds))
    return reqs


class SeedPrefetch:
    """Makes the requests' seed arrays (SectionSeeds) on a thread of its own,
    in arrival order and at most `ahead` requests before the submission
    cursor, so that a request arrives with its seeds ready, as it would from
    a client, and their making does not hold up the serving loop."""

    def __init__(self, reqs, ahead=64):
        import threading
        self.reqs, self.ahead = reqs, ahead
        self.pos = 0
        self.cv = threading.Condition()
        self.ready = [threading.Event() for _ in reqs]
        self.stop = False
        self.th = threading.Thread(target=self._run, daemon=True)
        self.th.start()

    def _run(self):
        for i, r in enumerate(self.reqs):
            with self.cv:
                while i >= self.pos + self.ahead and not self.stop:
                    self.cv.wait()
                if self.stop:
                    return
            kind, arg, t0, t1 = r.job
            if callable(arg):
                r.job = (kind, arg(), t0, t1)
            self.ready[i].set()

    def take(self, i):
        with self.cv:
            self.pos = i + 1
            self.cv.notify()
        self.ready[i].wait()
        return self.reqs[i].job

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify()
        self.th.join()


def _result_copy(kind, res):
    """A request's results copied out of the batch's result block, in the
    blocking calls' shapes: (wT, wN), residence times, or the tracer state."""
    if kind == "ftle":
        return res["wT"].copy(), res["wN"].copy()
    if kind == "residence":
        return res["rt"].copy()
    return {k: res[k].copy() for k in ("X", "eid", "left", "ldt")}


def serve(sites, requests, keep_results=False, time_limit=600.0, censor=False):
    """Serves the requests in arrival order against the sites' batches.

    The loop submits every request whose arrival time has passed, ticks each
    site's batch (a tick enqueues one frame interval of every admitted job
    and returns; at most two are in flight per site, and the sites' streams
    run concurrently), and collects finished jobs: each job's results are
    queued to the host on the batch's result stream (fvc_batch_result_begin,
    at most fvc.BATCH_RESULT_SLOTS at a time per site) and, once there, the
    job is released and its latency recorded.  The loop never waits for a
    result's copy.  Returns a summary dict.

    time_limit: wall seconds.  Past it serving raises, or with censor=True
    stops: the summary then covers the requests that finished, counts the
    rest (arrived or not) and gives the unfinished requests' waiting time so
    far as a lower bound of their latency."""
    pending = sorted(requests, key=lambda r: r.t_arrive)
    nxt = 0
    running = {name: {} for name in sites}
    done = []
    host = {"submit": 0.0, "tick": 0.0, "poll": 0.0, "results": 0.0, "idle": 0.0}
    clock = time.perf_counter
    seeds = SeedPrefetch(pending)
    to_collect = {name: [] for name in sites}   # finished, results not yet queued
    collecting = {name: [] for name in sites}   # (jid, request, ticket)
    t0 = time.perf_counter()
    stopped = False
    while len(done) < len(pending):
        now = time.perf_counter() - t0
        if now > time_limit:
            if not censor:
                seeds.close()
                raise RuntimeError(f"serving did not finish within {time_limit} s")
            stopped = True
            break
        c0 = clock()
        while nxt < len(pending) and pending[nxt].t_arrive <= now:
            r = pending[nxt]
            r.jid = submit(sites[r.site].batch, seeds.take(nxt))
            running[r.site][r.jid] = r
            nxt += 1
        c1 = clock()
        host["submit"] += c1 - c0
        busy = False
        for name, site in sites.items():
            b = site.batch
            if running[name]:
                busy = True
                c0 = clock()
                b.tick()
                c1 = clock()
                host["tick"] += c1 - c0
                finished = [jid for jid in running[name] if b.poll(jid) == fvc.BATCH_DONE]
                host["poll"] += clock() - c1
                to_collect[name].extend((jid, running[name].pop(jid)) for jid in finished)
            if not (to_collect[name] or collecting[name]):
                continue
            busy = True
            c2 = clock()
            while to_collect[name] and len(collecting[name]) < fvc.BATCH_RESULT_SLOTS:
                jid, r = to_collect[name].pop(0)
                collecting[name].append((jid, r, b.result_begin(jid)))
            still = []
            for jid, r, ticket in collecting[name]:
                if not b.result_ready(ticket):
                    still.append((jid, r, ticket))
                    continue
                r.t_done = time.perf_counter() - t0
                if keep_results:
                    r.result = _result_copy(r.kind, b.result_get(ticket))
                js = b.job_stats(jid)
                r.steps = js["steps_main"] + js["steps_early"]
                b.result_release(ticket)
                b.release(jid)
                done.append(r)
            collecting[name] = still
            host["results"] += clock() - c2
        if not busy and nxt < len(pending):
            wait = pending[nxt].t_arrive - (time.perf_counter() - t0)
            if wait > 0:
                c0 = clock()
                time.sleep(min(wait, 0.001))
                host["idle"] += clock() - c0
    wall = time.perf_counter() - t0
    seeds.close()
    lat = np.array([r.t_done - r.t_arrive for r in done]) if done else np.zeros(1)
    steps = sum(r.steps for r in done)
    if stopped:
        # the jobs still running have advanced too: count their steps so far
        for name, site in sites.items():
            jids = list(running[name]) + [j for j, _ in to_collect[name]] + [j for j, _, _ in collecting[name]]
            for jid in jids:
                try:
                    js = site.batch.job_stats(jid)
                    steps += js["steps_main"] + js["steps_early"]
                except fvc.FvcError:
                    pass
    by_kind = {}
    for k in ("tracers", "ftle", "residence"):
        lk = np.array([r.t_done - r.t_arrive for r in done if r.kind == k])
        if len(lk):
            by_kind[k] = {"n": int(len(lk)), "p50_ms": 1e3 * float(np.percentile(lk, 50)),
                          "p99_ms": 1e3 * float(np.percentile(lk, 99))}
    out = {"requests": len(done), "wall_s": wall, "steps": int(steps), "steps_per_s": steps / wall,
           "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p95_ms": 1e3 * float(np.percentile(lat, 95)),
           "p99_ms": 1e3 * float(np.percentile(lat, 99)), "max_ms": 1e3 * float(lat.max()),
           "by_kind": by_kind, "host_s": {k: round(v, 3) for k, v in host.items()}}
    if stopped:
        waiting = np.array([wall - r.t_arrive for r in pending[:nxt] if r.t_done is None])
        out.update({"stopped_at_s": wall, "requests_total": len(pending), "requests_unfinished": len(pending) - len(done),
                    "requests_not_yet_arrived": len(pending) - nxt,
                    "unfinished_waited_p50_ms": 1e3 * float(np.percentile(waiting, 50)) if len(waiting) else None,
                    "note": "stopped at the time limit: latencies cover the finished requests only"})
    return out


def sustained(summary, reqs, duration, p99_limit_ms=1000.0):
    """Whether a served run kept up with its arrivals: every request finished
    within 5 s after the last arrival, p99 stayed under p99_limit_ms, and the
    requests arriving in the last third of the window waited (p99) no more
    than twice those of the first third, or under half the limit (a queue
    that grows fails these; at light load the thirds' p99s are a few dozen
    requests each and their ratio is noise)."""
    if summary.get("requests_unfinished"):
        return False
    if summary["wall_s"] > duration + 5.0 or summary["p99_ms"] > p99_limit_ms:
        return False
    early = [r.t_done - r.t_arrive for r in reqs if r.t_done is not None and r.t_arrive < duration / 3]
    late = [r.t_done - r.t_arrive for r in reqs if r.t_done is not None and r.t_arrive > 2 * duration / 3]
    if not early or not late:
        return True
    late99 = 1e3 * float(np.percentile(late, 99))
    return late99 <= max(2.0 * 1e3 * float(np.percentile(early, 99)), 0.5 * p99_limit_ms)
