"""Generate the golden fixtures under tests/golden/ by running the reference.

For every case below this script writes small synthetic inputs in ompVC's
file formats (flowvc-1_gb300/synth.py), runs the unmodified ompVC program
built from the reference sources (oracle/Makefile.ref -> oracle/_ref/ompflowVC)
on each parameter set, and stores the inputs, the parameters and ompVC's
output files.  The tests compare the CPU oracle and the GPU engine against
these files; the inputs are committed (not regenerated) so that both machines
read identical bytes.

Usage:  python tests/golden/make_golden.py   (needs oracle/_ref/ompflowVC)
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "flowvc-1_gb300"))
import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ompflowVC")


def fb(x0, x1, y0, y1, z0, z1, nx, ny, nz):
    return {"FTLE_MeshBounds.XMin": x0, "FTLE_MeshBounds.XMax": x1, "FTLE_MeshBounds.YMin": y0,
            "FTLE_MeshBounds.YMax": y1, "FTLE_MeshBounds.ZMin": z0, "FTLE_MeshBounds.ZMax": z1,
            "FTLE_MeshBounds.XRes": nx, "FTLE_MeshBounds.YRes": ny, "FTLE_MeshBounds.ZRes": nz}


def tb(x0, x1, y0, y1, z0, z1, nx, ny, nz):
    return {"Trace_MeshBounds.XMin": x0, "Trace_MeshBounds.XMax": x1, "Trace_MeshBounds.YMin": y0,
            "Trace_MeshBounds.YMax": y1, "Trace_MeshBounds.ZMin": z0, "Trace_MeshBounds.ZMax": z1,
            "Trace_MeshBounds.XRes": nx, "Trace_MeshBounds.YRes": ny, "Trace_MeshBounds.ZRes": nz}


FTLE = {"FTLE_Compute": 1}
TRACE = {"Trace_Compute": 1}


def cases():
    """(name, builder(dir) -> synth.Case, {run: .in overrides})"""
    out = []

    # ompVC's GenerateTracerMesh leaves LeftDomainTime uninitialised on
    # Cartesian grids (ompVC/tracers.c:1345-1357 set it only for unstructured
    # meshes), so its output there depends on heap contents; the Cartesian
    # tracer fixtures use seed lists, for which ompVC is well defined.
    def dg(d):
        c = synth.make_double_gyre_case(d, nx=33, ny=17, nframes=11, dt=0.1, prefix="dg")
        g = np.stack(np.meshgrid(np.linspace(0.1, 1.9, 20), np.linspace(0.1, 0.9, 10), indexing="xy"), -1).reshape(-1, 2)
        pts = np.concatenate([g, [[2.5, 0.5], [-0.2, 0.3]]])
        synth.write_seed_list(os.path.join(d, "seeds2d.bin"), np.c_[pts, np.zeros(len(pts))], 2)
        return c
    out.append(("dg", dg, {
        "ftle_fwd": dict(FTLE, FTLE_IntTLength=0.8, Int_TimeStep=0.01, **fb(0, 2, 0, 1, 0, 0, 41, 21, 1)),
        "ftle_bwd": dict(FTLE, FTLE_IntTLength=0.7, Int_TimeStep=0.015, Int_TimeDirection=-1, Output_TStart=1.0,
                         **fb(0.05, 1.95, 0.02, 0.98, 0, 0, 30, 16, 1)),
        "ftle_slides": dict(FTLE, FTLE_IntTLength=0.5, Int_TimeStep=0.02, Output_TRes=3, Output_TDelta=0.2,
                            **fb(-0.1, 2.1, 0, 1, 0, 0, 24, 12, 1)),
        "ftle_euler": dict(FTLE, FTLE_IntTLength=0.6, Int_TimeStep=0.01, Int_Type=0, **fb(0, 2, 0, 1, 0, 0, 25, 13, 1)),
        "tracer_list": dict(TRACE, Trace_InFile="seeds2d.bin", Trace_InFileFormat=4, Output_TRes=6, Output_TDelta=0.15,
                            Trace_IntTLength=0.8, Int_TimeStep=0.01),
        "ftle_rkf": dict(FTLE, FTLE_IntTLength=0.8, Int_Type=2, Int_Accuracy=1e-6, Int_MinTimeStep=1e-4,
                         Int_MaxTimeStep=0.05, **fb(0, 2, 0, 1, 0, 0, 25, 13, 1)),
        "tracer_rkf": dict(TRACE, Trace_InFile="seeds2d.bin", Trace_InFileFormat=4, Output_TRes=6, Output_TDelta=0.15,
                           Trace_IntTLength=0.8, Int_Type=2, Int_Accuracy=1e-7, Int_MinTimeStep=1e-4,
                           Int_MaxTimeStep=0.04),
    }))

    def dgp(d):  # one full period of the double gyre (period 10): periodic data
        return synth.make_double_gyre_case(d, nx=21, ny=11, nframes=11, dt=1.0, prefix="dgp")
    out.append(("dg_periodic", dgp, {
        "ftle_wrap": dict(FTLE, Data_TPeriodic=1, FTLE_IntTLength=13.0, Int_TimeStep=0.1, Output_TStart=4.0,
                          **fb(0, 2, 0, 1, 0, 0, 21, 11, 1)),
    }))

    def tri(d):
        return synth.make_tri_case(d, n=8, nframes=11, dt=0.1, prefix="tri")
    out.append(("tri", tri, {
        "ftle_fwd": dict(FTLE, FTLE_IntTLength=0.8, Int_TimeStep=0.01, **fb(0, 2, 0, 1, 0, 0, 33, 17, 1)),
        "ftle_bwd": dict(FTLE, FTLE_IntTLength=0.5, Int_TimeStep=0.02, Int_TimeDirection=-1, Output_TStart=1.0,
                         **fb(0.1, 1.9, 0.05, 0.95, 0, 0, 19, 10, 1)),
        "tracer_grid": dict(TRACE, Trace_GenerateMesh=1, Output_TRes=5, Output_TDelta=0.2, Trace_IntTLength=0.8,
                            Int_TimeStep=0.01, **tb(0.05, 1.95, 0.05, 0.95, 0, 0, 15, 8, 1)),
        "tracer_rt": dict(TRACE, Trace_GenerateMesh=1, Output_TRes=5, Output_TDelta=0.2, Trace_IntTLength=0.8,
                          Int_TimeStep=0.01, Trace_ComputeRT=1, Trace_NumLaunchTimes=2, Trace_LaunchTimeSpacing=0.2,
                          **tb(0.0, 2.0, 0.05, 0.95, 0, 0, 12, 6, 1)),
        "tracer_cet": dict(TRACE, Trace_GenerateMesh=1, Output_TRes=5, Output_TDelta=0.2, Trace_IntTLength=0.8,
                           Int_TimeStep=0.01, Trace_ComputeCET=1, Trace_CETSubsteps=6, Num_threads=1,
                           **tb(0.05, 1.95, 0.05, 0.95, 0, 0, 15, 8, 1)),
    }))

    def cube(d):
        c = synth.make_abc_cube_case(d, n=6, nframes=11, dt=0.02, prefix="cube")
        synth.write_seed_list(os.path.join(d, "seeds.bin"), synth.uniform_seeds(600, 3, seed=3), 3)
        pts = synth.uniform_seeds(120, 3, seed=4, lo=-0.1, hi=1.1)
        with open(os.path.join(d, "seeds.txt"), "w") as f:
            f.write(f"{len(pts)}\n")
            for p in pts:
                f.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
        return c
    out.append(("cube", cube, {
        "ftle_fwd": dict(FTLE, FTLE_IntTLength=0.2, Int_TimeStep=0.005, **fb(0, 1, 0, 1, 0, 1, 10, 9, 8)),
        "ftle_bwd": dict(FTLE, FTLE_IntTLength=0.15, Int_TimeStep=0.004, Int_TimeDirection=-1, Output_TStart=0.2,
                         **fb(0, 1, 0, 1, 0, 1, 9, 9, 9)),
        "ftle_nolsc": dict(FTLE, FTLE_IntTLength=0.1, Int_TimeStep=0.006, LocalSearchChecking=0,
                           **fb(-0.05, 1.05, 0, 1, 0.1, 0.9, 8, 7, 6)),
        "ftle_slides": dict(FTLE, FTLE_IntTLength=0.1, Int_TimeStep=0.005, Output_TRes=2, Output_TDelta=0.05,
                            **fb(0, 1, 0, 1, 0, 1, 7, 7, 7)),
        "tracer_list": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=6, Output_TDelta=0.03,
                            Trace_IntTLength=0.2, Int_TimeStep=0.005),
        "tracer_ascii": dict(TRACE, Trace_InFile="seeds.txt", Trace_InFileFormat=1, Output_TRes=4, Output_TDelta=0.05,
                             Trace_IntTLength=0.2, Int_TimeStep=0.004, Int_Type=0),
        "tracer_grid": dict(TRACE, Trace_GenerateMesh=1, Output_TRes=8, Output_TDelta=0.02, Trace_IntTLength=0.12,
                            Int_TimeStep=0.004, Trace_NumLaunchTimes=3, Trace_LaunchTimeSpacing=0.02,
                            **tb(0.0, 1.0, 0.05, 0.95, 0.1, 0.9, 6, 5, 4)),
        "tracer_always": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=4, Output_TDelta=0.06,
                              Trace_IntTLength=0.2, Int_TimeStep=0.005, Trace_AlwaysOutput=1),
        "tracer_rkf": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=6, Output_TDelta=0.03,
                           Trace_IntTLength=0.2, Int_Type=2, Int_Accuracy=1e-7, Int_MinTimeStep=1e-4,
                           Int_MaxTimeStep=0.01),
        "ftle_rkf": dict(FTLE, FTLE_IntTLength=0.12, Int_Type=2, Int_Accuracy=1e-6, Int_MinTimeStep=1e-4,
                         Int_MaxTimeStep=0.01, **fb(0, 1, 0, 1, 0, 1, 8, 7, 6)),
        # residence time (OutputRT): seed list with points outside the mesh,
        # two releases; and a generated seed grid
        "tracer_rt": dict(TRACE, Trace_InFile="seeds.txt", Trace_InFileFormat=1, Output_TRes=5, Output_TDelta=0.04,
                          Trace_IntTLength=0.12, Int_TimeStep=0.005, Trace_NumLaunchTimes=2,
                          Trace_LaunchTimeSpacing=0.04, Trace_ComputeRT=1),
        "tracer_rt_grid": dict(TRACE, Trace_GenerateMesh=1, Output_TRes=4, Output_TDelta=0.05, Trace_IntTLength=0.15,
                               Int_TimeStep=0.005, Trace_ComputeRT=1, **tb(0.0, 1.0, 0.05, 0.95, 0.1, 0.9, 6, 5, 4)),
        # exposure time (ComputeExposureTime / OutputCET) with RK4, Euler and
        # RKF; one thread, because ompVC's OpenMP loop adds the sums without
        # synchronisation
        "tracer_cet": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=4, Output_TDelta=0.05,
                           Trace_IntTLength=0.15, Int_TimeStep=0.005, Trace_ComputeCET=1, Trace_CETSubsteps=5,
                           Num_threads=1),
        "tracer_cet_euler": dict(TRACE, Trace_InFile="seeds.txt", Trace_InFileFormat=1, Output_TRes=4,
                                 Output_TDelta=0.05, Trace_IntTLength=0.15, Int_TimeStep=0.004, Int_Type=0,
                                 Trace_NumLaunchTimes=2, Trace_LaunchTimeSpacing=0.05, Trace_ComputeCET=1,
                                 Trace_CETSubsteps=3, Num_threads=1),
        "tracer_cet_rkf": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=4, Output_TDelta=0.05,
                               Trace_IntTLength=0.15, Int_Type=2, Int_Accuracy=1e-7, Int_MinTimeStep=1e-4,
                               Int_MaxTimeStep=0.01, Trace_ComputeCET=1, Trace_CETSubsteps=4, Num_threads=1),
    }))

    def c3(d):
        c = synth.make_cart3d_case(d, n=9, nframes=11, dt=0.05, prefix="c3")
        synth.write_seed_list(os.path.join(d, "seeds.bin"), synth.uniform_seeds(300, 3, seed=6, lo=-0.05, hi=1.05), 3)
        return c
    out.append(("cart3d", c3, {
        "ftle_fwd": dict(FTLE, FTLE_IntTLength=0.3, Int_TimeStep=0.01, **fb(0, 1, 0, 1, 0, 1, 9, 10, 11)),
        "tracer_list": dict(TRACE, Trace_InFile="seeds.bin", Trace_InFileFormat=4, Output_TRes=5, Output_TDelta=0.1,
                            Trace_IntTLength=0.4, Int_TimeStep=0.01),
    }))
    return out


def run_ref(case_dir, name, params):
    od = os.path.join(case_dir, "expected", name)
    shutil.rmtree(od, ignore_errors=True)
    os.makedirs(od)
    inp = os.path.join(case_dir, f"_{name}.in")
    synth.write_in_file(inp, **dict(params, Path_Data=os.path.join(case_dir, "inputs") + "/", Path_Output=od + "/"))
    r = subprocess.run([REF, inp], capture_output=True, text=True)
    os.remove(inp)
    if r.returncode:
        raise RuntimeError(f"ompVC failed on {case_dir}/{name}:\n{r.stderr[-2000:]}")
    # intermediate files ompVC leaves beside the inputs are not fixtures
    for f in os.listdir(os.path.join(case_dir, "inputs")):
        if f.endswith((".IC", "_ic.bin")) or "_slide" in f:
            os.remove(os.path.join(case_dir, "inputs", f))


def main():
    """All cases (inputs regenerated), or with arguments CASE/RUN ... only those
    runs, on the committed inputs."""
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -f oracle/Makefile.ref")
    only = [a.split("/") for a in sys.argv[1:]]
    if only:
        table = {name: runs for name, _, runs in cases()}
        for name, rn in only:
            cd = os.path.join(HERE, name)
            with open(os.path.join(cd, "params.json")) as f:
                params = json.load(f)
            params["runs"][rn] = table[name][rn]
            with open(os.path.join(cd, "params.json"), "w") as f:
                json.dump(params, f, indent=1, sort_keys=True)
            run_ref(cd, rn, dict(params["base"], **params["runs"][rn]))
            print(name, rn)
        return
    for name, build, runs in cases():
        cd = os.path.join(HERE, name)
        shutil.rmtree(cd, ignore_errors=True)
        c = build(os.path.join(cd, "inputs"))
        base = {k: v for k, v in c.params.items() if k not in ("Path_Data", "Path_Output")}
        params = {"base": base, "runs": runs}
        with open(os.path.join(cd, "params.json"), "w") as f:
            json.dump(params, f, indent=1, sort_keys=True)
        for rn, over in runs.items():
            run_ref(cd, rn, dict(base, **over))
        print(name, sorted(runs))


if __name__ == "__main__":
    main()
