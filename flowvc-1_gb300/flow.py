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


def run_ftle(ctx: fvc.Context, ax: TimeAxis, grid, T, direction=1, t_start=0.0, lsc=1, state=None):
    """One FTLE slide over its whole integration window, frames resident.

    grid = (xmin, xmax, ymin, ymax, zmin, zmax, xres, yres, zres).  Returns
    (ftle_wT, ftle_woT, steps, job stats); a dict passed as state receives
    the slide's final point state (fvc_ftle_get_state)."""
    if ax.periodic:
        stop = t_start + direction * T
    else:
        stop = max(min(t_start + direction * T, ax.tmax), ax.tmin)
    spec = fvc.FtleSpec(*grid[:6], *grid[6:9], lsc, t_start, stop, 1)
    job = fvc.FtleJob(ctx, spec)
    first, last = ftle_frame_range(ax, t_start, T, direction)
    steps, status = 0, 0
    out = None
    df = first
    while df != last:
        lo, tmin, tmax = ax.window(df, direction)
        ctx.set_window(ax.frame_mod(lo), ax.frame_mod(lo + 1), tmin, tmax)
        if status == 1 or (tmin - TINY <= t_start <= tmax + TINY):
            launch = status == 0
            t1 = t_start if launch else (tmin if direction > 0 else tmax)
            t2 = min(tmax, stop) if direction > 0 else max(tmin, stop)
            status = 1
            job.interval(launch, t1, t2, wait=False)
            if ((stop - tmax) if direction > 0 else (tmin - stop)) < TINY:
                out = job.reduce(T)
                if state is not None:
                    state.update(job.get_state())
                break
        df += direction
    st = job.stats()
    steps = st["steps_main"] + st["steps_early"]
    job.close()
    if out is None:
        raise RuntimeError("FTLE window did not complete")
    return out[0], out[1], steps, st


def run_tracers(ctx: fvc.Context, ax: TimeAxis, seeds, t_start, out_delta, out_res, direction=1, lsc=1,
                always=0, snapshots=True, state=None):
    """One tracer release from t_start with outputs every out_delta (ompVC's
    Compute_Tracer loop, ompVC/tracers.c:25-289).  Returns (list of output
    arrays, steps, job stats); a dict passed as state receives the release's
    final tracer state (fvc_tracer_get_state)."""
    t_end = t_start + (out_res - 1) * direction * out_delta
    first = int(math.floor((t_start - ax.tmin) / ax.tdelta)) if direction > 0 else int(math.ceil((t_start - ax.tmin) / ax.tdelta))
    last = int(math.ceil((t_end - ax.tmin) / ax.tdelta)) if direction > 0 else int(math.floor((t_end - ax.tmin) / ax.tdelta))
    job = fvc.TracerJob(ctx, seeds, lsc=lsc, chain=0)
    stop = t_end
    outs = []
    nxt, frame_out, status, steps = t_start, 0, 0, 0
    df = first
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
                steps += job.advance(t1, t2)
                if abs(nxt - t2) < TINY and frame_out < out_res:
                    outs.append(job.snapshot(always) if snapshots else None)
            if ((stop - t2) if direction > 0 else (t2 - stop)) < TINY:
                status = 2
            if abs(t2 - nxt) < TINY:
                nxt += direction * out_delta
                frame_out += 1
                if frame_out >= out_res:
                    break
            t1 = t2
        df += direction
    st = job.stats()
    if state is not None:
        state.update(job.get_state())
    job.close()
    return outs, steps, st
