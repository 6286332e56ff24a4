"""Frame-loop drivers over the C ABI for in-memory inputs.

These mirror the host loop of fvcflow (and of ompVC's main.c:170-227) for
callers that hold the mesh and frames in memory instead of in files: the
benchmark and the tests.  All arithmetic happens in libfvc on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

import fvc

TINY = 1.0e-10


@dataclass
class TimeAxis:
    """Data_TMin / Data_TDelta / Data_TRes / Data_TPeriodic of an input set."""
    tmin: float
    tdelta: float
    tres: int
    periodic: int = 0

    @property
    def tmax(self):
        return self.tmin + (self.tres - 1) * self.tdelta

    def frame_mod(self, frame):
        """File index of frame index `frame` (ompVC/velocity.c:174-177)."""
        m = int(math.fmod(frame, self.tres - 1))
        return m + self.tres - 1 if m < 0 else m

    def window(self, df, direction):
        """(frame_lo, tmin, tmax) of frame interval df (ompVC/main.c:188-195)."""
        lo = df if direction > 0 else df - 1
        tmin = self.tmin + lo * self.tdelta
        return lo, tmin, tmin + self.tdelta


def ftle_frame_range(ax: TimeAxis, t_start, T, direction):
    """Data_FirstFrame / Data_LastFrame for one FTLE slide (ompVC/parameters.c:322-333)."""
    t_end = t_start
    tminreq = min(t_start, t_end + direction * T)
    if tminreq < ax.tmin and not ax.periodic:
        tminreq = ax.tmin
    tmaxreq = max(t_start, t_end + direction * T)
    if tmaxreq > ax.tmax and not ax.periodic:
        tmaxreq = ax.tmax
    if direction > 0:
        return int(math.floor((tminreq - ax.tmin) / ax.tdelta)), int(math.ceil((tmaxreq - ax.tmin) / ax.tdelta))
    return int(math.ceil((tmaxreq - ax.tmin) / ax.tdelta)), int(math.floor((tminreq - ax.tmin) / ax.tdelta))


def upload_frames(ctx: fvc.Context, ax: TimeAxis, frames, asynchronous=False):
    """Upload every frame file once, under its file index.  asynchronous:
    through the frame pipeline (fvc_upload_frame_async; the arrays must be
    C-contiguous float64, page-locked for overlap, and stay alive and
    unchanged until the context has used them or frame_wait returned)."""
    for i, f in enumerate(frames):
        if asynchronous:
            ctx.upload_frame_async(i, f)
        else:
            ctx.upload_frame(i, f)


def run_ftle(ctx: fvc.Context, ax: TimeAxis, grid, T, direction=1, t_start=0.0, lsc=1, state=None, out=None,
             fetch=True, wait=False):
    """One FTLE slide over its whole integration window, frames resident.

    grid = (xmin, xmax, ymin, ymax, zmin, zmax, xres, yres, zres).  Returns
    (ftle_wT, ftle_woT, steps, job stats); a dict passed as state receives
    the slide's final point state (fvc_ftle_get_state).  out: host arrays
    for the two fields; fetch=False leaves them on the device (None).
    wait=True waits for every interval (the default queues them)."""
    if ax.periodic:
        stop = t_start + direction * T
    else:
        stop = max(min(t_start + direction * T, ax.tmax), ax.tmin)
    spec = fvc.FtleSpec(*grid[:6], *grid[6:9], lsc, t_start, stop, 1)
    job = fvc.FtleJob(ctx, spec)
    first, last = ftle_frame_range(ax, t_start, T, direction)
    steps, status = 0, 0
    res = None
    df = first
    while df != last:
        lo, tmin, tmax = ax.window(df, direction)
        ctx.set_window(ax.frame_mod(lo), ax.frame_mod(lo + 1), tmin, tmax)
        if status == 1 or (tmin - TINY <= t_start <= tmax + TINY):
            launch = status == 0
            t1 = t_start if launch else (tmin if direction > 0 else tmax)
            t2 = min(tmax, stop) if direction > 0 else max(tmin, stop)
            status = 1
            job.interval(launch, t1, t2, wait=wait)
            if ((stop - tmax) if direction > 0 else (tmin - stop)) < TINY:
                res = job.reduce(T, out=out, fetch=fetch)
                if state is not None:
                    state.update(job.get_state())
                break
        df += direction
    st = job.stats()
    steps = st["steps_main"] + st["steps_early"]
    job.close()
    if res is None:
        raise RuntimeError("FTLE window did not complete")
    return res[0], res[1], steps, st


class OutputWriter:
    """Takes a release's asynchronous outputs (fvc_tracer_output_wait) on a
    thread of its own, in ticket order, hands each to consume(index, array)
    and frees its slot, so the loop that advances the tracers never waits for
    the GPU.  consume runs on the writer thread and must copy what it keeps
    (the array is the library's page-locked slot).  At most `slots` outputs
    are outstanding: submit() blocks until one is freed."""

    def __init__(self, ctx: fvc.Context, consume, slots=fvc.TRACER_OUTPUT_SLOTS):
        import queue
        import threading
        self.ctx, self.consume = ctx, consume
        self.free = threading.Semaphore(slots)
        self.q = queue.Queue()
        self.err = None
        self.th = threading.Thread(target=self._run, daemon=True)
        self.th.start()

    def _run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            idx, ticket = item
            try:
                if self.err is None:
                    self.consume(idx, self.ctx.output_wait(ticket))
            except BaseException as e:  # reported by close()
                self.err = e
            finally:
                try:
                    self.ctx.output_release(ticket)
                except fvc.FvcError as e:
                    self.err = self.err or e
                self.free.release()

    def submit(self, idx, job: fvc.TracerJob, always=0):
        self.free.acquire()
        try:
            self.q.put((idx, job.output_begin(always)))
        except BaseException:
            self.free.release()
            raise

    def close(self):
        self.q.put(None)
        self.th.join()
        if self.err is not None:
            raise self.err


def run_tracers(ctx: fvc.Context, ax: TimeAxis, seeds, t_start, out_delta, out_res, direction=1, lsc=1,
                always=0, snapshots=True, state=None, asynchronous=True, consume=None, timings=None):
    """One tracer release from t_start with outputs every out_delta (ompVC's
    Compute_Tracer loop, ompVC/tracers.c:25-289).  Returns (list of output
    arrays, steps, job stats); a dict passed as state receives the release's
    final tracer state (fvc_tracer_get_state).

    asynchronous (default): advances are queued without waiting and every
    output goes through the output ring to an OutputWriter thread, which
    passes it to consume(index, array) (default: keep a copy in the list
    returned); otherwise each advance waits and each output is a blocking
    fvc_tracer_snapshot.  A dict passed as timings receives the host
    seconds of the release's phases (seeding, loop, draining the outputs,
    reading the final state)."""
    import time
    clock = time.perf_counter
    c0 = clock()
    t_end = t_start + (out_res - 1) * direction * out_delta
    first = int(math.floor((t_start - ax.tmin) / ax.tdelta)) if direction > 0 else int(math.ceil((t_start - ax.tmin) / ax.tdelta))
    last = int(math.ceil((t_end - ax.tmin) / ax.tdelta)) if direction > 0 else int(math.floor((t_end - ax.tmin) / ax.tdelta))
    job = fvc.TracerJob(ctx, seeds, lsc=lsc, chain=0)
    c1 = clock()
    stop = t_end
    outs = []
    writer = None
    if asynchronous and snapshots:
        def keep(idx, a):
            outs.append(np.array(a))
        writer = OutputWriter(ctx, consume or keep)
    nxt, frame_out, status, steps = t_start, 0, 0, 0
    df = first
    try:
        while df != last:
            lo, tmin, tmax = ax.window(df, direction)
            ctx.set_window(ax.frame_mod(lo), ax.frame_mod(lo + 1), tmin, tmax)
            t1 = tmin if direction > 0 else tmax
            while ((t1 - tmax) if direction > 0 else (tmin - t1)) < 0:
                t2 = min(nxt, tmax) if direction > 0 else max(tmin, nxt)
                if status != 2 and (status == 1 or (min(t1, t2) <= t_start <= max(t1, t2))):
                    if status == 0:
                        status = 1
                        t1 = t_start
                        job.launch(t_start)
                    if asynchronous:
                        job.advance(t1, t2, wait=False)
                    else:
                        steps += job.advance(t1, t2)
                    if abs(nxt - t2) < TINY and frame_out < out_res and snapshots:
                        if writer is not None:
                            writer.submit(frame_out, job, always)
                        else:
                            outs.append(job.snapshot(always))
                    elif abs(nxt - t2) < TINY and frame_out < out_res:
                        outs.append(None)
                if ((stop - t2) if direction > 0 else (t2 - stop)) < TINY:
                    status = 2
                if abs(t2 - nxt) < TINY:
                    nxt += direction * out_delta
                    frame_out += 1
                    if frame_out >= out_res:
                        break
                t1 = t2
            df += direction
    finally:
        c2 = clock()
        if writer is not None:
            writer.close()
    c3 = clock()
    st = job.stats()
    if asynchronous:
        steps = st["steps_main"]
    if state is not None:
        state.update(job.get_state())
    job.close()
    if timings is not None:
        timings.update({"seeding_s": c1 - c0, "loop_s": c2 - c1, "drain_s": c3 - c2, "finish_s": clock() - c3})
    return outs, steps, st
