"""Asynchronous tracer outputs (fvc_tracer_output_begin / _wait / _release)
and queued advances (fvc_tracer_advance with steps == NULL).

The outputs a release loop takes through the output ring must be the bytes
the blocking path (a waiting advance, then fvc_tracer_snapshot) gives, in
both arithmetic forms; the ring refuses a fifth unreleased output and
unknown tickets; a fault of a queued advance comes back from the output
that follows it.  fvcflow's tracer files, which go through this path, are
compared with ompVC's in tests/test_gpu_golden.py and test_gpu_scale.py."""
import numpy as np
import pytest

import flow
import fvc
import synth

pytestmark = pytest.mark.gpu


def cube(prec="fp64", max_hops=0):
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=0)
    ctx = fvc.Context(3, 1, max_hops=max_hops)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, 0.005, 0)
    ctx.set_precision(prec)
    ax = flow.TimeAxis(0.0, 0.02, 16, 0)
    flow.upload_frames(ctx, ax, [synth.abc_flow(xyz, k * 0.02) for k in range(16)])
    return ctx, ax


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
@pytest.mark.parametrize("always", [0, 1])
def test_async_outputs_match_blocking_snapshots(engine, prec, always):
    ctx, ax = cube(prec)
    seeds = synth.uniform_seeds(20000, 3, seed=4, lo=-0.05, hi=1.05)
    a_state, b_state = {}, {}
    a, sa, _ = flow.run_tracers(ctx, ax, seeds, 0.0, 0.03, 9, always=always, state=a_state, asynchronous=False)
    b, sb, _ = flow.run_tracers(ctx, ax, seeds, 0.0, 0.03, 9, always=always, state=b_state, asynchronous=True)
    assert sa == sb > 0
    assert len(a) == len(b) == 9
    for k, (x, y) in enumerate(zip(a, b)):
        assert x.shape == y.shape and np.array_equal(x, y), f"output {k} differs"
    for key in ("X", "eid", "left", "ldt"):
        assert np.array_equal(a_state[key], b_state[key]), key
    assert len(a[-1]) < len(a[0]) or always  # tracers left, and outputs shrank
    ctx.close()


def test_ring_limits_and_tickets(engine):
    ctx, ax = cube()
    ctx.set_window(0, 1, 0.0, 0.02)
    job = fvc.TracerJob(ctx, synth.uniform_seeds(500, 3, seed=1))
    job.launch(0.0)
    job.advance(0.0, 0.01, wait=False)
    tickets = [job.output_begin() for _ in range(fvc.TRACER_OUTPUT_SLOTS)]
    with pytest.raises(fvc.FvcError) as e:
        job.output_begin()
    assert e.value.status == fvc.FVC_ERR_STATE
    first = np.array(ctx.output_wait(tickets[0]))
    ctx.output_release(tickets[0])
    with pytest.raises(fvc.FvcError) as e:
        ctx.output_wait(tickets[0])  # released
    assert e.value.status == fvc.FVC_ERR_STATE
    t5 = job.output_begin()  # a slot is free again
    for t in tickets[1:] + [t5]:
        assert np.array_equal(np.array(ctx.output_wait(t)), first)  # no advance in between
        ctx.output_release(t)
    with pytest.raises(fvc.FvcError):
        ctx.output_release(10 ** 6)
    assert np.array_equal(first, job.snapshot())
    job.close()
    ctx.close()


def test_queued_advance_fault_reported_by_the_output(engine):
    """A hop cap of 1: the queued advance's walks fail on the device; the
    call that returns is the output's wait, with FVC_ERR_WALK."""
    ctx, ax = cube(max_hops=1)
    ctx.set_window(0, 1, 0.0, 0.02)
    job = fvc.TracerJob(ctx, np.tile([0.51, 0.52, 0.53], (64, 1)))  # one point: seeds locate without hops
    job.launch(0.0)
    job.advance(0.0, 0.02, wait=False)
    t = job.output_begin()
    with pytest.raises(fvc.FvcError) as e:
        ctx.output_wait(t)
    assert e.value.status == fvc.FVC_ERR_WALK
    ctx.output_release(t)
    with pytest.raises(fvc.FvcError) as e:
        job.get_state()  # the job's next waiting call reports it too
    assert e.value.status == fvc.FVC_ERR_WALK
    job.close()
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
def test_waiting_calls_match_queued_ones(engine, prec):
    """A job's wait (an FTLE interval or a tracer advance that returns its
    steps) takes the accumulated counts without losing the live list the
    next call runs on: windows run with every call waiting give the bytes
    of the queued ones."""
    ctx, ax = cube(prec)
    grid = (0, 1, 0, 1, 0, 1, 12, 11, 10)
    sa, sb = {}, {}
    a = flow.run_ftle(ctx, ax, grid, 0.2, state=sa)
    b = flow.run_ftle(ctx, ax, grid, 0.2, state=sb, wait=True)
    assert a[2] == b[2] > 0
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for key in sa:
        assert np.array_equal(sa[key], sb[key]), key
    seeds = synth.uniform_seeds(5000, 3, seed=6, lo=-0.05, hi=1.05)
    ta, tb = {}, {}
    oa, stp_a, _ = flow.run_tracers(ctx, ax, seeds, 0.0, 0.03, 9, state=ta, asynchronous=True)
    ob, stp_b, _ = flow.run_tracers(ctx, ax, seeds, 0.0, 0.03, 9, state=tb, asynchronous=False)
    assert stp_a == stp_b > 0
    for x, y in zip(oa, ob):
        assert np.array_equal(x, y)
    for key in ("X", "eid", "left", "ldt"):
        assert np.array_equal(ta[key], tb[key]), key
    ctx.close()
