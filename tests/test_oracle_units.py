"""Unit checks of the CPU oracle's building blocks and the input generators."""
import math
import os

import numpy as np
import pytest

import oracle_lib
import synth


def test_max_eig_matches_numpy():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        D = rng.normal(size=(3, 3)) * rng.choice([1e-3, 1.0, 30.0])
        C = D.T @ D
        lam = oracle_lib.max_eig(C)
        ref = np.linalg.eigvalsh(C)[-1]
        assert abs(lam - ref) <= 1e-13 * max(abs(ref), 1e-300) + 1e-300


def test_max_eig_degenerate_and_diagonal():
    assert oracle_lib.max_eig(np.eye(3)) == 1.0
    assert oracle_lib.max_eig(np.diag([2.0, 5.0, 3.0])) == 5.0
    assert oracle_lib.max_eig(np.zeros((3, 3))) == 0.0
    a = np.full((3, 3), 1.0)
    assert abs(oracle_lib.max_eig(a) - 3.0) < 1e-14


def _cube_oracle(n=6):
    xyz, conn, adj = synth.kuhn_cube_mesh(n, jitter=0.2, seed=0)
    o = oracle_lib.Oracle(3, 1)
    o.set_unstruct(xyz, conn, adj)
    o.set_bounds([0, 1, 0, 1, 0, 1])
    return o, xyz, conn, adj


def test_kuhn_mesh_is_conforming():
    xyz, conn, adj = synth.kuhn_cube_mesh(5, jitter=0.2, seed=0)
    E = conn.shape[0]
    assert E == 6 * 125 and xyz.shape[0] == 216
    # every interior face is shared by exactly two elements, symmetric
    for s in range(4):
        nb = adj[:, s]
        m = nb >= 0
        assert (adj[nb[m]] == np.arange(E)[m][:, None]).any(1).all()
    assert (adj < 0).sum() == 6 * 25 * 2


def test_global_search_is_lowest_id_containing():
    o, xyz, conn, adj = _cube_oracle()
    pts = synth.uniform_seeds(300, 3, seed=5)
    got = o.global_search(pts)
    assert (got >= 0).all()
    # walking from any element finds an element containing the point too
    again = o.local_search(pts, np.zeros(len(pts), np.int32))
    assert (again >= 0).all()


def test_ab2_is_second_order():
    """AB2 has no reference implementation; pin it by its convergence order on
    a steady solid-body rotation sampled on a Cartesian grid (exact solution a
    circle)."""
    n = 81
    g = np.linspace(-1.0, 1.0, n)
    Y, X = np.meshgrid(g, g, indexing="ij")
    uvw = np.stack([-Y, X, np.zeros_like(X)], -1).reshape(-1, 3)
    errs = []
    for h in (0.02, 0.01, 0.005):
        o = oracle_lib.Oracle(2, 0)
        o.set_cart(-1.0, 1.0, n, -1.0, 1.0, n, 0.0, 0.0, 1)
        o.set_bounds([-1, 1, -1, 1, 0, 0])
        o.set_frames(uvw, uvw, 0.0, 1.0)
        o.set_integrator(3, h, 0)
        P = np.array([[0.5, 0.0, 0.0]])
        V = np.zeros((1, 3))
        eid = np.zeros(1, np.int32)
        left = np.zeros(1, np.int32)
        ldt = np.zeros(1)
        o.advect(P, V, eid, left, ldt, 0.0, 1.0)
        exact = np.array([0.5 * math.cos(1.0), 0.5 * math.sin(1.0)])
        errs.append(np.linalg.norm(P[0, :2] - exact))
    r1 = errs[0] / errs[1]
    r2 = errs[1] / errs[2]
    assert 3.0 < r1 < 5.0 and 3.0 < r2 < 5.0, errs


def test_rk4_error_fourth_order_in_time():
    """Sanity: RK4 on a linear-in-space field is exact up to time-stepping."""
    n = 41
    g = np.linspace(-1.0, 1.0, n)
    Y, X = np.meshgrid(g, g, indexing="ij")
    uvw = np.stack([-Y, X, np.zeros_like(X)], -1).reshape(-1, 3)
    errs = []
    for h in (0.1, 0.05):
        o = oracle_lib.Oracle(2, 0)
        o.set_cart(-1.0, 1.0, n, -1.0, 1.0, n, 0.0, 0.0, 1)
        o.set_bounds([-1, 1, -1, 1, 0, 0])
        o.set_frames(uvw, uvw, 0.0, 1.0)
        o.set_integrator(1, h, 0)
        P = np.array([[0.5, 0.0, 0.0]])
        o.advect(P, np.zeros((1, 3)), np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1), 0.0, 1.0)
        errs.append(np.linalg.norm(P[0, :2] - [0.5 * math.cos(1.0), 0.5 * math.sin(1.0)]))
    assert 12 < errs[0] / errs[1] < 20, errs
