"""fvc_advect_noalloc: advection without device allocation.

Some callers cannot allocate GPU memory while they advect: an application
whose own pool allocator has taken the rest of the device, or a code path in
which the device synchronisation of a cudaMalloc is not allowed.  For them the
library has fvc_advect_noalloc, which keeps its scratch in one fixed array per
GPU.  These tests call it through the C ABI and require the same results as
fvc_advect, bit for bit (the tolerance of every advection test here), on two
calls in a row: the second call finds the first call's bytes in the shared
array and must not be affected by them.  The file is named to be collected
last; it needs nothing from the other test files and runs alone as well.
"""
import os
import re

import numpy as np
import pytest

import fvc
import synth
from conftest import ROOT

pytestmark = pytest.mark.gpu


def header_limit():
    src = open(os.path.join(ROOT, "include", "fvc.h")).read()
    return int(re.search(r"#define FVC_NOALLOC_MAX_POINTS (\d+)", src).group(1))


def tet_context(int_type, extrap):
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=3)
    g = fvc.Context(3, 1)
    g.set_unstruct_mesh(xyz, conn, adj)
    g.set_bounds([0, 1, 0, 1, 0, 1])
    g.upload_frame(0, synth.abc_flow(xyz, 0.3) * 0.3)
    g.upload_frame(1, synth.abc_flow(xyz, 0.4) * 0.3)
    g.set_window(0, 1, 0.3, 0.4)
    g.set_integrator(int_type, 0.0071, extrap)
    return g


def cart2_context(int_type):
    nx, ny = 41, 21
    xs, ys = np.linspace(0, 2, nx), np.linspace(0, 1, ny)
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    g = fvc.Context(2, 0)
    g.set_cart_mesh(0.0, 2.0, nx, 0.0, 1.0, ny, 0.0, 0.0, 1)
    g.set_bounds([0, 2, 0, 1, -1, 1])
    for k, t in enumerate((0.3, 0.4)):
        u, v = synth.double_gyre(X, Y, t)
        g.upload_frame(k, np.stack([u, v, np.zeros_like(u)], -1).reshape(-1, 3))
    g.set_window(0, 1, 0.3, 0.4)
    g.set_integrator(int_type, 0.0071, 0)
    return g


def points(g, n, rng, dims):
    lo, hi = np.zeros(3), np.array([1.0, 1.0, 1.0] if dims == 3 else [2.0, 1.0, 0.0])
    P = rng.uniform(lo - 0.02 * hi, hi * 1.02, size=(n, 3))
    if dims == 2:
        P[:, 2] = 0.0
        eid = np.full(n, -1, np.int32)
        left = ((P[:, :2] < 0) | (P[:, :2] > hi[:2])).any(1).astype(np.int32)
    else:
        eid = g.global_search(P)
        left = (eid < 0).astype(np.int32)
    V = rng.normal(size=(n, 3)) * 0.1
    return [P, V, eid, left, np.zeros(n)]


def both(g, state, t0, t1):
    """The same advection through fvc_advect and fvc_advect_noalloc."""
    a = [x.copy() for x in state]
    b = [x.copy() for x in state]
    sa = g.advect(*a, t0, t1)
    sb = g.advect_noalloc(*b, t0, t1)
    for nm, x, y in zip(["X", "V", "eid", "left", "ldt"], a, b):
        assert np.array_equal(x, y), f"{nm} differs from fvc_advect"
    assert sa == sb > 0
    return b


@pytest.mark.parametrize("int_type,extrap", [(1, 0), (0, 1), (3, 0)])
def test_noalloc_tet_matches_advect_twice(engine, int_type, extrap):
    g = tet_context(int_type, extrap)
    rng = np.random.default_rng(100 + int_type)
    # first call: many points forward; second call: fewer, different points
    # backward, so the array still holds the first call's larger arrays
    both(g, points(g, 20000, rng, 3), 0.3, 0.3877)
    both(g, points(g, 3001, rng, 3), 0.4, 0.3123)
    g.close()


def test_noalloc_cart2_matches_advect_twice(engine):
    g = cart2_context(1)
    rng = np.random.default_rng(7)
    s = both(g, points(g, 5000, rng, 2), 0.3, 0.35)
    both(g, s, 0.35, 0.4)  # continue from the first call's results
    g.close()


def test_noalloc_allocates_no_device_memory(engine):
    """The entry point's own claim: calls of different sizes leave the
    device's free memory unchanged, on a context that has never run
    fvc_advect (so no pool or scratch of the context exists to reuse).  One
    warm-up call comes first: the driver may load the kernels' code on their
    first launch, which is not an allocation of this library."""
    torch = pytest.importorskip("torch")
    g = tet_context(1, 0)
    rng = np.random.default_rng(11)
    calls = [points(g, n, rng, 3) for n in (64, 17, 5000, header_limit())]
    g.advect_noalloc(*[x.copy() for x in calls[0]], 0.3, 0.33)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for st in calls[1:]:
        assert g.advect_noalloc(*[x.copy() for x in st], 0.3, 0.35) > 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0, "fvc_advect_noalloc changed the device's free memory"
    g.close()


def test_noalloc_at_its_limit_and_beyond(engine):
    limit = header_limit()
    g = tet_context(1, 0)
    rng = np.random.default_rng(5)
    both(g, points(g, limit, rng, 3), 0.3, 0.33)
    both(g, points(g, 17, rng, 3), 0.33, 0.36)
    over = points(g, limit + 1, rng, 3)
    with pytest.raises(fvc.FvcError) as e:
        g.advect_noalloc(*over, 0.3, 0.33)
    assert e.value.status == fvc.FVC_ERR_ARG and str(limit) in str(e.value)
    g.close()
