"""The mixed-precision form (BF16 / FP16 frames with per-frame, per-component
FP32 scales, FP32 location / interpolation / RK4 stages, Kahan-compensated
FP32 positions, FP64 near-face containment) against the FP64 form, which the
other GPU tests pin bit for bit to the CPU oracle and ompVC.

The tolerances are stated per test: they follow from the 16-bit storage
(BF16 keeps 8 significant bits, FP16 11) and FP32 arithmetic, not from any
bit-level agreement."""
import numpy as np
import pytest

import fvc
import flow
import synth

pytestmark = pytest.mark.gpu

# largest relative rounding error of one stored component, relative to the
# frame's max |component| (the scale)
QERR = {"bf16": 2.0 ** -9, "fp16": 2.0 ** -11}


def tet_field(n=8, seed=0):
    xyz, conn, adj = synth.kuhn_cube_mesh(n, jitter=0.2, seed=seed)
    frames = [synth.abc_flow(xyz, t) * 0.3 for t in (0.3, 0.4)]
    return xyz, conn, adj, frames


def make_ctx(F, prec, int_type=1, h=0.0071):
    xyz, conn, adj, frames = F
    g = fvc.Context(3, 1)
    g.set_unstruct_mesh(xyz, conn, adj)
    g.set_bounds([0, 1, 0, 1, 0, 1])
    g.upload_frame(7, frames[0])
    g.upload_frame(8, frames[1])
    g.set_window(7, 8, 0.3, 0.4)
    g.set_integrator(int_type, h, 0)
    g.set_precision(prec)
    return g


def seeds(g, n, rng, lo=0.05, hi=0.95):
    P = rng.uniform(lo, hi, size=(n, 3))
    eid = g.global_search(P)
    return P, eid, (eid < 0).astype(np.int32)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_velocity_within_quantisation(engine, prec):
    F = tet_field()
    g64, gm = make_ctx(F, "fp64"), make_ctx(F, prec)
    P, eid, left = seeds(g64, 4000, np.random.default_rng(1))
    u64 = g64.velocity(P, eid.copy(), left.copy(), 0.337)
    um = gm.velocity(P, eid.copy(), left.copy(), 0.337)
    # per component: two frames' rounding (each <= QERR * scale) plus FP32
    scale = np.maximum(np.abs(F[3][0]).max(0), np.abs(F[3][1]).max(0))
    err = np.abs(um - u64)
    assert (err <= QERR[prec] * scale * 1.05 + 1e-6).all(), (err / scale).max()
    g64.close()
    gm.close()


@pytest.mark.parametrize("prec,tol", [("bf16", 2e-3), ("fp16", 3e-4)])
def test_rk4_endpoints_close(engine, prec, tol):
    F = tet_field()
    g64, gm = make_ctx(F, "fp64"), make_ctx(F, prec)
    P, eid, left = seeds(g64, 5000, np.random.default_rng(2))
    a = [P.copy(), np.zeros_like(P), eid.copy(), left.copy(), np.zeros(len(P))]
    b = [P.copy(), np.zeros_like(P), eid.copy(), left.copy(), np.zeros(len(P))]
    s64 = g64.advect(*a, 0.3, 0.4)
    sm = gm.advect(*b, 0.3, 0.4)
    both = (a[3] == 0) & (b[3] == 0)
    assert both.mean() > 0.9
    err = np.abs(a[0][both] - b[0][both]).max()
    # 14 RK4 steps of h = 0.0071 through a field with |u| <= 1.1: the
    # endpoint error is the velocity error times the time, amplified by the
    # flow's stretching over 0.1 time units
    assert err < tol, err
    assert abs(sm - s64) <= 0.02 * s64
    # element ids agree wherever both runs still have the point
    assert (a[2][both] != b[2][both]).mean() < 0.01
    g64.close()
    gm.close()


def test_kahan_keeps_fp64_accuracy(engine):
    """Euler in a uniform flow whose velocity and step are exact in BF16 and
    FP32: the only error left is the accumulation of 1,000 increments, which
    Kahan compensation keeps near FP64 level (a plain FP32 sum would err by
    about 1e-5)."""
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=0)
    u = np.array([2.0 ** -6, 2.0 ** -7, -(2.0 ** -8)])
    frame = np.tile(u, (len(xyz), 1))
    N, h = 1000, 2.0 ** -8
    g = fvc.Context(3, 1)
    g.set_unstruct_mesh(xyz, conn, adj)
    g.set_bounds([0, 1, 0, 1, 0, 1])
    g.upload_frame(0, frame)
    g.upload_frame(1, frame)
    g.set_window(0, 1, 0.0, N * h)
    g.set_integrator(0, h, 0)
    g.set_precision("bf16")
    rng = np.random.default_rng(3)
    P, eid, left = seeds(g, 2000, rng, 0.3, 0.7)
    X = P.copy()
    steps = g.advect(X, None, eid, left, np.zeros(len(P)), 0.0, N * h)
    assert steps == N * len(P) and left.sum() == 0
    exact = P + N * h * u
    assert np.abs(X - exact).max() < 1e-9
    g.close()


# Measured on a GB300 (error / largest FP64 FTLE value): BF16 total max
# 0.0852 rms 0.0116, FP16 max 0.0101 rms 0.00135, all but ~4e-6 of it the
# 16-bit storage; the FP32 arithmetic against the FP64 form on the same
# 16-bit frames: max 4.2e-6 / 3.8e-6, rms 4.8e-7 / 4.9e-7.  The bounds sit
# 1.4-2.5x above those figures.
@pytest.mark.parametrize("prec,tol_max,tol_rms", [("bf16", 0.12, 0.016), ("fp16", 0.015, 0.002)])
def test_ftle_errors_bounded(engine, prec, tol_max, tol_rms):
    """FTLE on a 24^3 grid over T = 0.4 (20 frame intervals): max and RMS
    error relative to the largest FP64 FTLE value.  The error is also split
    by source: the FP64 form on the frames quantised and dequantised on the
    host carries the 16-bit storage error alone, and the mixed form against
    that run carries the FP32 arithmetic, bounded on its own."""
    import quantise
    xyz, conn, adj = synth.kuhn_cube_mesh(8, jitter=0.2, seed=0)
    frames = [synth.abc_flow(xyz, t) for t in np.arange(21) * 0.02]
    ax = flow.TimeAxis(0.0, 0.02, 21, 0)
    grid = (0, 1, 0, 1, 0, 1, 24, 24, 24)
    out = {}
    for p, fr in (("fp64", frames), (prec, frames), ("storage", [quantise.dequantised(f, prec) for f in frames])):
        g = fvc.Context(3, 1)
        g.set_unstruct_mesh(xyz, conn, adj)
        g.set_bounds([0, 1, 0, 1, 0, 1])
        g.set_integrator(1, 0.005, 0)
        g.set_precision(p if p != "storage" else "fp64")
        flow.upload_frames(g, ax, fr)
        wT, wN, steps, st = flow.run_ftle(g, ax, grid, 0.4)
        out[p] = wT
        g.close()
    ref, got = out["fp64"], out[prec]
    scale = np.abs(ref).max()
    err = np.abs(got - ref) / scale
    storage = np.abs(out["storage"] - ref) / scale
    arith = np.abs(got - out["storage"]) / scale
    print(prec, "FTLE error / largest value: total max %.3g rms %.3g; storage max %.3g rms %.3g; "
          "arithmetic max %.3g rms %.3g" % (err.max(), np.sqrt((err ** 2).mean()), storage.max(),
                                            np.sqrt((storage ** 2).mean()), arith.max(),
                                            np.sqrt((arith ** 2).mean())))
    assert err.max() < tol_max, err.max()
    assert np.sqrt((err ** 2).mean()) < tol_rms
    assert arith.max() < 1e-5, arith.max()
    assert np.sqrt((arith ** 2).mean()) < 1.2e-6


def test_mixed_refusals(engine):
    F = tet_field()
    g = make_ctx(F, "fp64", int_type=3)
    g.set_precision("bf16")
    P, eid, left = seeds(g, 10, np.random.default_rng(4))
    with pytest.raises(fvc.FvcError) as e:
        g.advect(P, None, eid, left, np.zeros(10), 0.3, 0.4)
    assert e.value.status == fvc.FVC_ERR_ARG
    g.set_integrator(1, 0.01, 0)
    with pytest.raises(fvc.FvcError) as e:
        g.advect_noalloc(P, None, eid, left, np.zeros(10), 0.3, 0.4)
    assert e.value.status == fvc.FVC_ERR_ARG
    g.close()
    c = fvc.Context(2, 0)
    with pytest.raises(fvc.FvcError) as e:
        c.set_precision("fp16")
    assert e.value.status == fvc.FVC_ERR_ARG
    c.close()


def test_state_roundtrip_in_mixed_form(engine):
    """A job's positions go in as FP64 and come back as FP64 through the
    (X, c) pairs: equal to 2^-48 relative."""
    F = tet_field()
    g = make_ctx(F, "bf16")
    spec = fvc.FtleSpec(0, 1, 0, 1, 0, 1, 6, 5, 4, 1, 0.3, 0.4, 0)
    job = fvc.FtleJob(g, spec)
    X = np.random.default_rng(5).uniform(0.1, 0.9, size=(120, 3))
    state = job.get_state()
    state["X"] = X
    job.set_state(state)
    back = job.get_state()["X"]
    assert np.abs(back - X).max() <= 2.0 ** -48
    job.close()
    g.close()


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_fvcflow_precision_option(engine, tmp_path, prec):
    """fvcflow --precision runs the golden cube FTLE case in a mixed form:
    the same output files as the FP64 form, finite, within the mixed form's
    error of the reference's FTLE (short window, smooth flow)."""
    import os
    from conftest import GOLDEN, run_golden
    got, _ = run_golden(engine.FVCFLOW, "cube", "ftle_fwd", tmp_path, extra_args=("--precision", prec))
    exp = os.path.join(GOLDEN, "cube", "expected", "ftle_fwd")
    assert sorted(os.listdir(got)) == sorted(os.listdir(exp))
    for f in sorted(os.listdir(exp)):
        if not f.endswith(".bin") or "Cartesian" in f:
            continue
        A = np.fromfile(os.path.join(exp, f), np.float64)[1:]
        B = np.fromfile(os.path.join(got, f), np.float64)[1:]
        assert A.shape == B.shape and np.isfinite(B).all(), f
        assert np.abs(B - A).max() <= 0.05 * max(np.abs(A).max(), 1e-12), f
