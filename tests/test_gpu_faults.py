"""Failure detection without a GPU fault: failures are made on the host
(arguments, states, limits) and must come back as the documented statuses,
with the context still usable afterwards."""
import numpy as np
import pytest

import flow
import fvc
import synth

pytestmark = pytest.mark.gpu


def cube_ctx(max_hops=0, prec="fp64", n=6):
    xyz, conn, adj = synth.kuhn_cube_mesh(n, jitter=0.2, seed=0)
    ctx = fvc.Context(3, 1, max_hops=max_hops)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, 0.005, 0)
    ctx.set_precision(prec)
    frames = [synth.abc_flow(xyz, k * 0.02) for k in range(6)]
    ax = flow.TimeAxis(0.0, 0.02, 6, 0)
    flow.upload_frames(ctx, ax, frames)
    return ctx, ax


def advect_args(P, eid):
    return [P.copy(), np.zeros_like(P), eid.copy(), np.zeros(len(P), np.int32), np.zeros(len(P))]


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
def test_query_time_outside_the_window(prec):
    ctx, ax = cube_ctx(prec=prec)
    ctx.set_window(1, 2, 0.02, 0.04)
    P = synth.uniform_seeds(64, 3, seed=1)
    eid = ctx.global_search(P)
    with pytest.raises(fvc.FvcError) as e:
        ctx.advect(*advect_args(P, eid), 0.02, 0.07)  # ends past the window's 0.04
    assert e.value.status == fvc.FVC_ERR_TLOC
    # the context still works
    a = advect_args(P, eid)
    assert ctx.advect(*a, 0.02, 0.04) > 0
    ctx.close()


def test_walk_hop_cap():
    ctx, ax = cube_ctx(max_hops=1)
    ctx.set_window(0, 1, 0.0, 0.02)
    P = synth.uniform_seeds(256, 3, seed=2)
    eid = np.zeros(len(P), np.int32)  # every walk starts far away in element 0
    with pytest.raises(fvc.FvcError) as e:
        ctx.advect(*advect_args(P, eid), 0.0, 0.02)
    assert e.value.status == fvc.FVC_ERR_WALK
    ctx.close()


def test_ftle_fault_reported_by_the_call_that_waits():
    ctx, ax = cube_ctx()
    ctx.set_window(0, 1, 0.0, 0.02)
    spec = fvc.FtleSpec(0, 1, 0, 1, 0, 1, 6, 6, 6, 1, 0.0, 0.02, 1)
    job = fvc.FtleJob(ctx, spec)
    st = job.get_state()
    eid = st["eid"].copy()
    eid[7] = -1  # a live point without an element: "integrate point that already left"
    ctx.lib.fvc_ftle_set_state(job.h, None, fvc._i(eid), None, None, None, None, None)
    job.interval(0, 0.0, 0.02, wait=False)  # queued: no status yet
    with pytest.raises(fvc.FvcError) as e:
        job.reduce(0.02)
    assert e.value.status == fvc.FVC_ERR_STATE
    job.close()
    # a fresh job on the same context completes
    wT, wN, steps, _ = flow.run_ftle(ctx, ax, (0, 1, 0, 1, 0, 1, 5, 5, 5), 0.04)
    assert steps > 0 and np.isfinite(wT).all()
    ctx.close()


def test_batch_reports_failed_jobs_and_keeps_the_rest():
    """A hop cap of 1 lets no walk cross a face: a release that moves fails
    (at seed location or while advecting), a release of tracers outside the
    domain has nothing to walk and completes; one job's fault is its own."""
    ctx, ax = cube_ctx(max_hops=1)
    b = fvc.Batch(ctx, ax.tmin, ax.tdelta, ax.tres, 0)
    bad = b.submit_tracers(synth.uniform_seeds(500, 3, seed=5), 0.0, 0.06)
    good = b.submit_tracers(np.full((8, 3), 1.5), 0.0, 0.06)
    b.run()
    with pytest.raises(fvc.FvcError) as e:
        b.poll(bad)
    assert e.value.status in (fvc.FVC_ERR_WALK, fvc.FVC_ERR_CUDA, fvc.FVC_ERR_STATE)
    assert b.poll(good) == fvc.BATCH_DONE
    r = b.tracer_result(good)
    assert (r["left"] == 1).all()
    b.close()
    ctx.close()


@pytest.mark.parametrize("which", ["node", "neighbour"])
def test_bad_mesh_is_refused_and_the_old_mesh_stays(which):
    """An id out of range in the connectivity or adjacency is found on the
    device before the old mesh is released: FVC_ERR_ARG naming the lowest
    bad element, and the context keeps working on its old mesh."""
    ctx, ax = cube_ctx()
    ctx.cet_enable(3)  # exposure-time sums on the old mesh must survive the refusal
    xyz, conn, adj = synth.kuhn_cube_mesh(4, jitter=0.2, seed=1)
    conn, adj = conn.copy(), adj.copy()
    if which == "node":
        conn[9, 2] = len(xyz) + 7
        conn[30, 0] = -3
    else:
        adj[9, 1] = len(conn) + 1
    with pytest.raises(fvc.FvcError) as e:
        ctx.set_unstruct_mesh(xyz, conn, adj)
    assert e.value.status == fvc.FVC_ERR_ARG
    assert "element 9" in str(e.value)
    old_mesh_still_works(ctx)
    ctx.close()


def old_mesh_still_works(ctx):
    """The 6^3 cube of cube_ctx is still the context's mesh: global search,
    advection and the exposure-time sums (enabled by the caller) on it."""
    nelem = 6 * 6 ** 3
    cet, met, enc = ctx.cet_results(1, nelem)  # still enabled, still sized for the old mesh
    assert len(enc) == nelem and (enc == 0).all()
    ctx.set_window(0, 1, 0.0, 0.02)
    P = synth.uniform_seeds(64, 3, seed=1)
    eid = ctx.global_search(P)
    assert (eid >= 0).all()
    assert ctx.advect(*advect_args(P, eid), 0.0, 0.02) > 0


def test_bucket_grid_failure_keeps_the_old_mesh(monkeypatch):
    """A valid mesh whose bucket grid cannot be built (here: a cell cap far
    below what the mesh needs) is refused after its records were made; the
    context keeps its old mesh, grid and exposure-time sums, and a later mesh
    within the cap is accepted."""
    ctx, ax = cube_ctx()
    ctx.cet_enable(2)
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=1)
    monkeypatch.setenv("FVC_BUCKET_MAX_CELLS", "16")
    with pytest.raises(fvc.FvcError) as e:
        ctx.set_unstruct_mesh(xyz, conn, adj)
    assert e.value.status == fvc.FVC_ERR_ARG and "bucket grid" in str(e.value)
    old_mesh_still_works(ctx)
    monkeypatch.delenv("FVC_BUCKET_MAX_CELLS")
    ctx.set_unstruct_mesh(xyz, conn, adj)  # within the default cap: replaces the mesh
    with pytest.raises(fvc.FvcError) as e:
        ctx.cet_results(1, len(conn))  # the old mesh's sums went with it
    assert e.value.status == fvc.FVC_ERR_STATE
    P = synth.uniform_seeds(64, 3, seed=2)
    assert (ctx.global_search(P) >= 0).all()
    ctx.close()
