"""The batched / served form (fvc_batch_*) against the single-job calls.

A job computed in a batch runs the same frame intervals, step sequences and
kernel arithmetic as the same job computed alone through fvc_tracer_* /
fvc_ftle_*, so every result must be bit-identical: alone, in a mix of
uneven jobs, under an HBM budget that forces admission in waves, with jobs
arriving while others run, and when the whole schedule is one CUDA graph.
Times are dyadic so every window end is exact."""
import math

import numpy as np
import pytest

import flow
import fvc
import synth

pytestmark = pytest.mark.gpu

TINY = 1.0e-10
DT = 0.03125
NFR = 17


@pytest.fixture(scope="module")
def case():
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=0)
    frames = [synth.abc_flow(xyz, k * DT) for k in range(NFR)]
    return xyz, conn, adj, frames


def make_ctx(case, prec, periodic=False):
    xyz, conn, adj, frames = case
    ctx = fvc.Context(3, 1)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, 0.01, 0)
    ctx.set_precision(prec)
    ax = flow.TimeAxis(0.0, DT, NFR, 1 if periodic else 0)
    flow.upload_frames(ctx, ax, frames)
    return ctx, ax


def single_tracers(ctx, ax, seeds, t0, t1, residence=False):
    """One release advanced interval by interval through fvc_tracer_*."""
    d = 1 if t1 > t0 else -1
    stop = t1 if ax.periodic else max(min(t1, ax.tmax), ax.tmin)
    job = fvc.TracerJob(ctx, seeds)
    x = (t0 - ax.tmin) / ax.tdelta
    df = math.floor(x) if d > 0 else math.ceil(x)
    launched = False
    while True:
        lo = df if d > 0 else df - 1
        tmin = ax.tmin + lo * ax.tdelta
        tmax = tmin + ax.tdelta
        ctx.set_window(ax.frame_mod(lo), ax.frame_mod(lo + 1), tmin, tmax)
        a = t0 if not launched else (tmin if d > 0 else tmax)
        if not launched:
            job.launch(t0)
            launched = True
        b = min(tmax, stop) if d > 0 else max(tmin, stop)
        job.advance(a, b)
        df += d
        if ((stop - tmax) if d > 0 else (tmin - stop)) < TINY:
            break
    st = job.get_state()
    rt = job.residence(t0, stop) if residence else None
    job.close()
    return st, rt


def jobs_spec():
    rng = np.random.default_rng(5)
    out = []
    for k, (n, t0, t1) in enumerate([(700, 0.0, 0.25), (40, 0.0625, 0.5), (3000, 0.5, 0.125),
                                      (1, 0.125, 0.1875), (1500, 0.25, 0.34375)]):
        out.append(("tracers", rng.uniform(-0.05, 1.05, (n, 3)), t0, t1))
    out.append(("residence", rng.uniform(0, 1, (900, 3)), 0.0625, 0.3125))
    out.append(("ftle", (0, 1, 0, 1, 0, 1, 9, 8, 7), 0.0, 0.25))
    out.append(("ftle", (0.1, 0.9, 0, 1, 0.05, 0.95, 6, 7, 8), 0.375, 0.125))
    return out


def single_results(ctx, ax, specs):
    res = []
    for kind, arg, t0, t1 in specs:
        if kind == "ftle":
            d = 1 if t1 > t0 else -1
            wT, wN, _, _ = flow.run_ftle(ctx, ax, arg, abs(t1 - t0), direction=d, t_start=t0)
            res.append((wT, wN))
        else:
            st, rt = single_tracers(ctx, ax, arg, t0, t1, residence=kind == "residence")
            res.append((st, rt))
    return res


def submit(b, spec):
    kind, arg, t0, t1 = spec
    if kind == "ftle":
        return b.submit_ftle(arg, t0, t1)
    return b.submit_tracers(arg, t0, t1, residence=kind == "residence")


def check(b, jid, spec, ref):
    kind = spec[0]
    assert b.poll(jid) == fvc.BATCH_DONE
    if kind == "ftle":
        wT, wN = b.ftle_result(jid)
        assert np.array_equal(wT, ref[0]) and np.array_equal(wN, ref[1]), "FTLE differs from the single job"
        return
    got = b.tracer_result(jid)
    for k in ("X", "eid", "left", "ldt"):
        assert np.array_equal(got[k], ref[0][k]), f"{kind} {k} differs from the single job"
    if kind == "residence":
        assert np.array_equal(b.residence_result(jid), ref[1])


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
@pytest.mark.parametrize("mode", ["eager", "graph", "budget", "served", "tuned", "resort", "resort_graph",
                                  "multi", "multi_graph", "multi_served"])
def test_batch_matches_single_jobs(case, prec, mode):
    ctx, ax = make_ctx(case, prec)
    specs = jobs_spec()
    ref = single_results(ctx, ax, specs)
    budget = 2_500_000 if mode == "budget" else 0
    resort = 1 if mode.startswith("resort") else (-1 if mode == "tuned" else 0)
    # multi: releases run several frame intervals a tick (tick_intervals 3:
    # 3 to 5 for these windows), FTLE jobs one
    ticks = 3 if mode.startswith("multi") else 0
    b = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0, hbm_budget=budget, resort_every=resort, tick_intervals=ticks)
    if mode in ("served", "multi_served"):
        # half the jobs first, the rest arriving while those run
        ids = [submit(b, s) for s in specs[::2]]
        for _ in range(3):
            b.tick()
        late = [submit(b, s) for s in specs[1::2]]
        while b.tick():
            pass
        order = list(range(0, len(specs), 2)) + list(range(1, len(specs), 2))
        ids = ids + late
    else:
        ids = [submit(b, s) for s in specs]
        order = list(range(len(specs)))
        if mode == "tuned":
            b.autotune()
        b.run(graph=mode in ("graph", "resort_graph", "multi_graph"))
    for jid, k in zip(ids, order):
        check(b, jid, specs[k], ref[k])
    st = b.stats()
    assert st["jobs_done"] == len(specs)
    if mode in ("graph", "resort_graph", "multi_graph"):
        assert st["graphs"] == 1
    if mode in ("multi", "multi_graph"):
        assert st["ticks"] < 13  # the longest release alone spans 13 intervals
    if mode == "tuned":
        assert st["tuned_threads"] in (64, 128, 256)
        assert st["tuned_resort"] in (0, 1)
    if mode.startswith("resort"):
        assert st["tuned_resort"] == 1
    b.close()
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "fp16"])
def test_batch_job_alone_equals_in_mix(case, prec):
    """Each job alone in its own batch gives the bytes it gives in the mix."""
    ctx, ax = make_ctx(case, prec)
    specs = jobs_spec()
    mix = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0)
    ids = [submit(mix, s) for s in specs]
    mix.run()
    for jid, s in zip(ids, specs):
        one = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0)
        j1 = submit(one, s)
        one.run()
        if s[0] == "ftle":
            a, b = one.ftle_result(j1), mix.ftle_result(jid)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        else:
            a, b = one.tracer_result(j1), mix.tracer_result(jid)
            for k in ("X", "eid", "left", "ldt"):
                assert np.array_equal(a[k], b[k])
        one.close()
    mix.close()
    ctx.close()


def test_batch_periodic_backward(case):
    """Periodic data: windows that wrap past the last frame, both directions."""
    ctx, ax = make_ctx(case, "fp64", periodic=True)
    rng = np.random.default_rng(9)
    specs = [("tracers", rng.uniform(0, 1, (500, 3)), 0.375, 0.75),
             ("tracers", rng.uniform(0, 1, (300, 3)), 0.125, -0.25),
             ("ftle", (0, 1, 0, 1, 0, 1, 6, 6, 6), 0.4375, 0.6875)]
    ref = single_results(ctx, ax, specs)
    b = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 1)
    ids = [submit(b, s) for s in specs]
    b.run()
    for jid, s, r in zip(ids, specs, ref):
        check(b, jid, s, r)
    b.close()
    ctx.close()


def test_batch_release_and_errors(case):
    ctx, ax = make_ctx(case, "fp64")
    b = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0)
    with pytest.raises(fvc.FvcError):
        b.submit_tracers(np.zeros((4, 3)) + 0.5, 0.25, 0.125, residence=True)  # residence time runs forward
    with pytest.raises(fvc.FvcError):
        b.submit_tracers(np.zeros((4, 3)) + 0.5, 0.25, 0.25)  # empty window
    jid = b.submit_tracers(np.full((8, 3), 0.5), 0.0, 0.0625)
    with pytest.raises(fvc.FvcError):
        b.release(jid)  # still queued
    b.run()
    b.release(jid)
    assert b.poll(jid) == fvc.BATCH_RELEASED
    with pytest.raises(fvc.FvcError):
        b.tracer_result(jid)
    b.close()
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
def test_batch_async_results(case, prec):
    """fvc_batch_result_*: the results a ticket points at equal the blocking
    calls' (tracer state in seed order through the device-side reordering,
    residence times, FTLE fields); at most FVC_BATCH_RESULT_SLOTS tickets are
    held; a job holding a ticket is not released; unknown tickets are refused."""
    ctx, ax = make_ctx(case, prec)
    specs = jobs_spec()
    b = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0)
    ids = [submit(b, s) for s in specs]
    b.run()
    tickets = [b.result_begin(j) for j in ids]
    assert len(tickets) == len(set(tickets)) == fvc.BATCH_RESULT_SLOTS
    with pytest.raises(fvc.FvcError) as e:
        b.result_begin(ids[0])  # every block is held
    assert e.value.status == fvc.FVC_ERR_STATE
    with pytest.raises(fvc.FvcError) as e:
        b.release(ids[0])  # its ticket is held
    assert e.value.status == fvc.FVC_ERR_STATE
    for jid, s, t in zip(ids, specs, tickets):
        got = b.result_get(t)
        assert b.result_ready(t)
        if s[0] == "ftle":
            wT, wN = b.ftle_result(jid)
            assert np.array_equal(got["wT"], wT) and np.array_equal(got["wN"], wN)
        else:
            ref = b.tracer_result(jid)
            for k in ("X", "eid", "left", "ldt"):
                assert np.array_equal(got[k], ref[k]), (s[0], k)
            if s[0] == "residence":
                assert np.array_equal(got["rt"], b.residence_result(jid))
        b.result_release(t)
        with pytest.raises(fvc.FvcError):
            b.result_get(t)  # released
        b.release(jid)
    with pytest.raises(fvc.FvcError):
        b.result_release(10 ** 6)
    b.close()
    ctx.close()
