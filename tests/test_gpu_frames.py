"""The frame pipeline: frames uploaded asynchronously from page-locked
buffers (fvc_upload_frame_async) give results identical to blocking uploads,
including a resident frame replaced while earlier work that reads it is
still queued."""
import numpy as np
import pytest

import flow
import fvc
import synth

pytestmark = pytest.mark.gpu


def make(mesh, prec):
    xyz, conn, adj = mesh
    ctx = fvc.Context(3, 1)
    ctx.set_unstruct_mesh(xyz, conn, adj)
    ctx.set_bounds([0, 1, 0, 1, 0, 1])
    ctx.set_integrator(1, 0.005, 0)
    ctx.set_precision(prec)
    return ctx


@pytest.mark.parametrize("prec", ["fp64", "bf16"])
def test_async_frames_equal_blocking(prec):
    mesh = synth.kuhn_cube_mesh(10, jitter=0.2, seed=0)
    frames = [synth.abc_flow(mesh[0], k * 0.02) for k in range(11)]
    ax = flow.TimeAxis(0.0, 0.02, 11, 0)
    grid = (0, 1, 0, 1, 0, 1, 12, 11, 10)
    a = make(mesh, prec)
    flow.upload_frames(a, ax, frames)
    ref = flow.run_ftle(a, ax, grid, 0.2)
    b = make(mesh, prec)
    pins = []
    for k, f in enumerate(frames):
        p = fvc.PinnedArray(f.shape)
        p.a[...] = f
        pins.append(p)
        b.upload_frame_async(k, p.a)
    got = flow.run_ftle(b, ax, grid, 0.2)
    for k in range(len(frames)):
        b.frame_wait(k)
        assert b.frame_ready(k)
    assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
    # replace frame 3 with frame 7's values while a window over it is queued
    P = synth.uniform_seeds(500, 3, seed=2)
    b.set_window(3, 4, 0.06, 0.08)
    eid = b.global_search(P)
    X1, X2 = P.copy(), P.copy()
    args = lambda X: [X, np.zeros_like(X), eid.copy(), np.zeros(len(X), np.int32), np.zeros(len(X))]  # noqa: E731
    s1 = args(X1)
    b.advect(*s1, 0.06, 0.08)
    pins[3].a[...] = frames[7]
    b.upload_frame_async(3, pins[3].a)
    b.set_window(3, 4, 0.06, 0.08)
    s2 = args(X2)
    b.advect(*s2, 0.06, 0.08)
    a.upload_frame(3, frames[7])
    a.set_window(3, 4, 0.06, 0.08)
    s3 = args(P.copy())
    a.advect(*s3, 0.06, 0.08)
    for x, y in zip(s2, s3):
        assert np.array_equal(x, y)
    assert not np.array_equal(s1[0], s2[0])
    a.close()
    b.close()
