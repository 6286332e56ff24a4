"""A fixed step-level advection workload for profilers.

Runs fvc_advect (RK4, h = 0.005) twice over one frame interval [0, 0.02]
for a seeded set of points in [0.05, 0.95]^3 on a jittered Kuhn-cube mesh
with ABC frames, and prints the accepted steps of each call.  The second
k_advect launch is the one to capture, e.g.

  ncu --metrics <list> --clock-control none -k regex:k_advect -s 1 -c 1 \\
      python flowvc-1_gb300/advect_probe.py 32 262144

and per-step figures are the captured totals divided by the printed steps.
Arguments: mesh cells per edge (default 32), points (default 262144).
"""
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import numpy as np  # noqa: E402

import fvc  # noqa: E402
import synth  # noqa: E402


def main():
    n_cells = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    npts = int(sys.argv[2]) if len(sys.argv) > 2 else 262144
    xyz, conn, adj = synth.kuhn_cube_mesh(n_cells, jitter=0.2, seed=0)
    g = fvc.Context(3, 1)
    g.set_unstruct_mesh(xyz, conn, adj)
    g.set_bounds([0, 1, 0, 1, 0, 1])
    g.upload_frame(0, synth.abc_flow(xyz, 0.0))
    g.upload_frame(1, synth.abc_flow(xyz, 0.02))
    g.set_window(0, 1, 0.0, 0.02)
    g.set_integrator(1, 0.005, 0)
    P = np.random.default_rng(0).uniform(0.05, 0.95, size=(npts, 3))
    eid = g.global_search(P)
    left = (eid < 0).astype(np.int32)
    V, ldt = np.zeros_like(P), np.zeros(npts)
    for call in range(2):
        a = [P.copy(), V.copy(), eid.copy(), left.copy(), ldt.copy()]
        t = time.perf_counter()
        steps = g.advect(*a, 0.0, 0.02)
        print(f"call {call}: steps {steps} seconds {time.perf_counter() - t:.6f} left {int(a[3].sum())}")
    g.close()


if __name__ == "__main__":
    main()
