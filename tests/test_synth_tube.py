"""Host-side generators of the batched / served workloads (no GPU): the
bent-tube mesh, its Womersley frames, the tube batch and the request stream."""
import math

import numpy as np

import serve
import synth


def test_tube_mesh_is_a_valid_positive_tet_mesh():
    t = synth.bent_tube_mesh(nc=6, nax=12)
    assert t.conn.shape == (6 * 6 * 12 * 6, 4)
    assert t.xyz.shape == (7 * 7 * 13, 3)
    vol = synth._tet_volume(t.xyz, t.conn.astype(np.int64))
    assert (vol > 0).all()
    # every interior face is shared by exactly two tets, and adjacency is mutual
    E = len(t.conn)
    for e in range(0, E, 7):
        for slot in range(4):
            nb = t.adj[e, slot]
            if nb >= 0:
                assert e in t.adj[nb]
    # boundary faces: the wall (4 sides x 6 x 12 quads) and the two ends, 2 triangles per quad
    assert int((t.adj < 0).sum()) == 2 * (4 * 6 * 12 + 2 * 36)
    # the wall nodes lie on the unit circle around the centre line
    wall = np.isclose(t.r, 1.0)
    C, T, N = synth.tube_centreline(t.s[wall], t.length, t.bend_radius)
    assert np.allclose(np.linalg.norm(t.xyz[wall] - C, axis=1), t.radius)


def test_womersley_frames_no_slip_periodic_and_scaled():
    t = synth.bent_tube_mesh(nc=6, nax=12)
    times, frames = synth.womersley_frames(t, nframes=21, peak=1.0, amp=0.5, alpha=4.0)
    assert len(frames) == 21 and math.isclose(times[-1], 1.0)
    assert np.array_equal(frames[0], frames[-1])           # closing frame repeats the first
    wall = np.isclose(t.r, 1.0)
    for f in frames:
        assert np.abs(f[wall]).max() < 1e-12                # no slip
    centre = np.argmin(t.r)
    speeds = [float(np.dot(f[centre], t.tangent[centre])) for f in frames[:-1]]
    assert math.isclose(max(speeds) - 1.0, 0.5, rel_tol=0.05)  # Poiseuille peak plus the harmonic
    # the velocity follows the axis
    k = 5
    along = np.einsum("ij,ij->i", frames[k], t.tangent)
    assert np.allclose(np.linalg.norm(frames[k], axis=1), np.abs(along))


def test_tube_batch_and_requests_are_seeded_and_shaped():
    t = synth.bent_tube_mesh(nc=6, nax=12)
    a = serve.tube_batch_jobs(t, njobs=16, nmin=10, nmax=1000, seed=3)
    b = serve.tube_batch_jobs(t, njobs=16, nmin=10, nmax=1000, seed=3)
    assert all(np.array_equal(x[1], y[1]) and x[2:] == y[2:] for x, y in zip(a, b))
    for kind, seeds, t0, t1 in a:
        assert kind == "tracers" and 10 <= len(seeds) <= 1000
        assert 0.2 - 1e-12 <= abs(t1 - t0) <= 2.0 + 1e-12
        # seeds inside the tube
        d = np.linalg.norm(seeds - synth.tube_centreline(
            np.full(len(seeds), 0.0), t.length, t.bend_radius)[0], axis=1)
        assert np.isfinite(d).all()
    reqs = serve.poisson_requests(t, rate=400.0, duration=5.0, seed=1, tracer_range=(10, 100),
                                  ftle_edges=(4, 6), rt_seeds=20)
    n = len(reqs)
    assert 1600 < n < 2400                                   # Poisson(2000)
    frac = {k: sum(r.kind == k for r in reqs) / n for k in ("tracers", "ftle", "residence")}
    assert abs(frac["tracers"] - 0.5) < 0.05 and abs(frac["ftle"] - 0.4) < 0.05
    assert abs(frac["residence"] - 0.1) < 0.03
    assert all(r2.t_arrive >= r1.t_arrive for r1, r2 in zip(reqs, reqs[1:]))
    for r in reqs:
        if r.kind == "ftle":
            assert r.site == "cube" and 4 ** 3 <= r.npts <= 6 ** 3
        else:
            assert r.site == "tube"
        if r.kind == "residence":
            assert r.job[3] > r.job[2]


def test_section_seeds_lie_on_their_cross_section():
    """Seeds made at submission (serve.SectionSeeds): deterministic, inside
    the disc of radius (1 - margin) R around the centreline point, in the
    plane normal to the axis there."""
    import serve
    t = synth.bent_tube_mesh(nc=6, nax=12)
    for s in (0.3, 0.5 * t.length, 0.97 * t.length):
        a = serve.SectionSeeds(t, 5000, s, 123)()
        b = serve.SectionSeeds(t, 5000, s, 123)()
        assert a.shape == (5000, 3) and np.array_equal(a, b)
        C, T, N = synth.tube_centreline(np.array([s]), t.length, t.bend_radius)
        d = a - C[0]
        assert np.abs(d @ T[0]).max() < 1e-12
        assert np.linalg.norm(d, axis=1).max() <= 0.98 * t.radius + 1e-12
