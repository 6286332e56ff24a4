"""Times the unmodified ompVC beside the oracle port on the benchmark's FTLE
workload, so that the port's speed as the timed CPU baseline is on record.

Workload: the 128^3 FTLE grid on the 1,572,864-tet jittered cube, ABC
frames, RK4 h = 0.005, forward over T = 1 (tests/scale_cases.py,
"cube_ftle"), generated here.  Runs, on this machine's cores:

  ompVC, Output_TRes = 1       one output slide: UPPERLOOP (forced by
                               Int_Extrapolate = 0, ompVC/parameters.c:
                               395-421) parallelises over slides, so one core
  ompVC, Output_TRes = nproc   nproc slides 0.02 apart, one per core
  port, 1 thread / nproc threads, on both inputs

Each time is the whole program's wall time (ompVC reports no advection-only
time: its FTLE loop also writes and reads the grid to a temporary file every
frame interval); the port also reports its advection phase.  Results go to
cpu_calibration.json beside this script.

Usage:  python tests/golden/scale/calibrate_cpu.py   (needs oracle/_ref/ompflowVC)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.join(ROOT, "flowvc-1_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import scale_cases as sc  # noqa: E402
import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ompflowVC")
PORT = os.path.join(ROOT, "oracle", "build", "orcflow")


def timed(cmd):
    t0 = time.time()
    r = subprocess.run(cmd, capture_output=True, text=True)
    wall = time.time() - t0
    if r.returncode:
        sys.exit(f"{cmd[0]} failed:\n{r.stdout[-1500:]}\n{r.stderr[-1500:]}")
    return wall, r.stdout


def main():
    nproc = os.cpu_count() or 1
    rows = []
    with tempfile.TemporaryDirectory() as td:
        data = sc.make_inputs("cube", td)
        # frames past t = 1 for the later slides (the ABC flow is analytic)
        xyz, _, _ = synth.kuhn_cube_mesh(64, jitter=0.2, seed=0)
        for f in range(sc.CUBE_FRAMES, sc.CUBE_FRAMES + nproc):
            synth.write_frame(os.path.join(data, f"cube_vel.{f}.bin"), f * sc.CUBE_DT,
                              synth.abc_flow(xyz, f * sc.CUBE_DT))
        for slides in (1, nproc):
            over = dict(Output_TRes=slides, Output_TDelta=sc.CUBE_DT, Num_threads=nproc,
                        Data_TRes=sc.CUBE_FRAMES + nproc)
            inp = sc.write_in("cube_ftle", data, os.path.join(td, f"omp{slides}"),
                              os.path.join(td, f"omp{slides}.in"), **over)
            wall, _ = timed([REF, inp])
            rows.append({"program": "ompVC", "slides": slides, "threads": nproc,
                         "cores_used": min(slides, nproc), "wall_s": round(wall, 2)})
            print(rows[-1], flush=True)
            for thr in (1, nproc):
                inp = sc.write_in("cube_ftle", data, os.path.join(td, f"orc{slides}_{thr}"),
                                  os.path.join(td, f"orc{slides}_{thr}.in"), **over)
                wall, out = timed([PORT, inp, str(thr)])
                d = json.loads(out.strip().splitlines()[-1])
                rows.append({"program": "port", "slides": slides, "threads": thr, "cores_used": thr,
                             "wall_s": round(wall, 2), "advect_s": round(d["advect_seconds"], 2),
                             "steps": d["steps"]})
                print(rows[-1], flush=True)
    res = {"workload": "FTLE 128^3 on the 1,572,864-tet jittered cube, ABC frames, RK4 h=0.005, T=1 per slide; "
                       "slides 0.02 apart",
           "host": {"nproc": nproc, "machine": os.uname().machine}, "rows": rows}
    with open(os.path.join(HERE, "cpu_calibration.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
