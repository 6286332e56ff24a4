"""The workloads of the benchmark configurations at full size, as ompVC input
sets: the parity cases that run at the sizes the engine is measured on.

  cube_ftle_5   1,572,864-tet jittered cube (64^3 cells x 6, seed 0), ABC
                frames dt = 0.02; FTLE on a 128^3 seed grid, RK4 h = 0.005,
                LocalSearchChecking = 1, forward over the first 5 frame
                intervals (T = 0.1)
  cube_ftle     the same over the whole window, T = 1 (50 intervals)
  cube_tracers  1,000,000 tracers uniform in the cube (seed 0) released at
                t = 0, RK4 h = 0.005 over T = 1, positions written every
                0.05 (21 output times; every tracer has left by t = 0.5,
                and ompVC writes no file once none is left: 10 files)
  dg_ftle       double gyre on 257 x 129 nodes, 101 frames dt = 0.1; FTLE
                on a 512 x 256 seed grid over [0,2] x [0,1], RK4 h = 0.01,
                forward over T = 10

Inputs are generated with fixed seeds and the portable sine of synth.py, so
every machine writes the same bytes (input_digests checks that).  Used by the
fixture script tests/golden/scale/make_scale_golden.py (which runs ompVC on
them), by the CPU tests of the oracle against ompVC's outputs and by the GPU
tests of the engine against the oracle.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

import synth

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scale")

CUBE_FRAMES, CUBE_DT = 51, 0.02
DG_FRAMES, DG_DT = 101, 0.1
CUBE_BOUNDS = {"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0, "Data_MeshBounds.YMin": 0.0,
               "Data_MeshBounds.YMax": 1.0, "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0}


def _ftle_grid(x0, x1, y0, y1, z0, z1, nx, ny, nz):
    return {"FTLE_MeshBounds.XMin": x0, "FTLE_MeshBounds.XMax": x1, "FTLE_MeshBounds.YMin": y0,
            "FTLE_MeshBounds.YMax": y1, "FTLE_MeshBounds.ZMin": z0, "FTLE_MeshBounds.ZMax": z1,
            "FTLE_MeshBounds.XRes": nx, "FTLE_MeshBounds.YRes": ny, "FTLE_MeshBounds.ZRes": nz}


CUBE_BASE = dict(Dimensions=3, Data_MeshType=1, Data_InFilePrefix="cube", Data_SuffixTMin=0, Data_SuffixTDelta=1,
                 Data_TRes=CUBE_FRAMES, Data_TDelta=CUBE_DT, Data_TMin=0.0, Data_TPeriodic=0, Int_Type=1,
                 Int_TimeStep=0.005, LocalSearchChecking=1, **CUBE_BOUNDS)

CASES = {
    "cube_ftle_5": ("cube", dict(CUBE_BASE, FTLE_Compute=1, FTLE_IntTLength=0.1,
                                 **_ftle_grid(0, 1, 0, 1, 0, 1, 128, 128, 128))),
    "cube_ftle": ("cube", dict(CUBE_BASE, FTLE_Compute=1, FTLE_IntTLength=1.0,
                               **_ftle_grid(0, 1, 0, 1, 0, 1, 128, 128, 128))),
    "cube_tracers": ("cube", dict(CUBE_BASE, Trace_Compute=1, Trace_InFile="seeds1m.bin", Trace_InFileFormat=4,
                                  Output_TRes=21, Output_TDelta=0.05, Trace_IntTLength=1.0)),
    "dg_ftle": ("dg", dict(Dimensions=2, Data_MeshType=0, Data_InFilePrefix="dg", Data_SuffixTMin=0,
                           Data_SuffixTDelta=1, Data_TRes=DG_FRAMES, Data_TDelta=DG_DT, Data_TMin=0.0,
                           Data_TPeriodic=0, Int_Type=1, Int_TimeStep=0.01, FTLE_Compute=1, FTLE_IntTLength=10.0,
                           **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 2.0,
                              "Data_MeshBounds.YMin": 0.0, "Data_MeshBounds.YMax": 1.0,
                              "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 0.0},
                           **_ftle_grid(0, 2, 0, 1, 0, 0, 512, 256, 1))),
}

# FTLE fields are summarised for the committed fixture: every STRIDE-th
# value in output order, and the sums of consecutive blocks of BLOCK values
FTLE_FILES = ("ftle.0.bin", "ftle_noT.0.bin")
STRIDE = 509
BLOCK = 4096


def make_inputs(kind, root):
    """Write the input set `kind` ("cube" or "dg") under root/kind (once);
    returns that directory."""
    d = os.path.join(root, kind)
    done = os.path.join(d, ".complete")
    if os.path.exists(done):
        return d
    os.makedirs(d, exist_ok=True)
    if kind == "cube":
        xyz, conn, adj = synth.kuhn_cube_mesh(64, jitter=0.2, seed=0)
        synth.write_unstructured_mesh(os.path.join(d, "cube"), xyz, conn, adj)
        for f in range(CUBE_FRAMES):
            synth.write_frame(os.path.join(d, f"cube_vel.{f}.bin"), f * CUBE_DT, synth.abc_flow(xyz, f * CUBE_DT))
        synth.write_seed_list(os.path.join(d, "seeds1m.bin"), synth.uniform_seeds(1_000_000, 3, seed=0), 3)
    else:
        synth.make_double_gyre_case(d, nx=257, ny=129, nframes=DG_FRAMES, dt=DG_DT, prefix="dg")
    open(done, "w").close()
    return d


def write_in(case, data_dir, out_dir, path, **over):
    kind, params = CASES[case]
    os.makedirs(out_dir, exist_ok=True)
    synth.write_in_file(path, **dict(params, Path_Data=data_dir + "/", Path_Output=out_dir + "/", **over))
    return path


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 22), b""):
            h.update(chunk)
    return h.hexdigest()


def input_digests(data_dir):
    """SHA-256 of the generated input files (mesh, frames, seeds); files the
    programs write next to them (ompVC's ftle_ic.bin) are not inputs."""
    kind = os.path.basename(os.path.normpath(data_dir))
    return {f: sha256(os.path.join(data_dir, f)) for f in sorted(os.listdir(data_dir))
            if f.endswith(".bin") and (f.startswith(kind + "_") or f.startswith("seeds"))}


def summarise(out_dir):
    """Digests of every output file; for the FTLE fields also the time stamp,
    the strided values and the block sums (float64 arrays)."""
    files, arrays = {}, {}
    for f in sorted(os.listdir(out_dir)):
        p = os.path.join(out_dir, f)
        files[f] = {"sha256": sha256(p), "bytes": os.path.getsize(p)}
        if f in FTLE_FILES:
            a = np.fromfile(p, "<f8")
            files[f]["time"] = float(a[0])
            v = a[1:]
            arrays[f + ":sub"] = v[::STRIDE].copy()
            nb = len(v) // BLOCK
            arrays[f + ":blk"] = v[:nb * BLOCK].reshape(nb, BLOCK).sum(1)
            arrays[f + ":absblk"] = np.abs(v[:nb * BLOCK]).reshape(nb, BLOCK).sum(1)
    return files, arrays


def ic_arrays(path):
    """Element ids and left flags of an FTLE_ICFile (the located seed grid
    ompVC writes at initialisation, ompVC/ftle.c:383-628): three int32
    resolutions, then one 104-byte FTLEPoint record a seed with the element
    id at byte 48 and LeftDomain at byte 56 (ompVC/structs.h layout on
    x86-64 and aarch64)."""
    raw = np.fromfile(path, np.uint8)
    res = raw[:12].view(np.int32)
    n = int(res[0]) * int(res[1]) * int(res[2])
    rec = raw[12:12 + 104 * n].reshape(n, 104)
    eid = rec[:, 48:52].copy().view(np.int32).ravel()
    left = rec[:, 56:60].copy().view(np.int32).ravel()
    return eid, left


def ic_digests(path):
    """Digests of the IC file's element ids and left flags; eid_inside_sha256
    covers the ids of the points inside only (ompVC leaves the id of a point
    it marks outside unset: whatever its heap held)."""
    eid, left = ic_arrays(path)
    inside = np.where(left != 0, -1, eid).astype(np.int32)
    return {"n": int(len(eid)), "eid_sha256": hashlib.sha256(eid.tobytes()).hexdigest(),
            "eid_inside_sha256": hashlib.sha256(inside.tobytes()).hexdigest(),
            "left_sha256": hashlib.sha256(left.tobytes()).hexdigest()}


def check_ic_against_fixture(case, ic_path, meta):
    """The located seed grid (element ids, left flags) of an FTLE run on the
    cube against ompVC's; every cube FTLE case shares cube_ftle_5's grid."""
    if not case.startswith("cube_ftle"):
        return False
    exp = meta["cases"]["cube_ftle_5"]["ic"]
    got = ic_digests(ic_path)
    assert got["n"] == exp["n"], f"{case}: {got['n']} seeds in the IC file, ompVC wrote {exp['n']}"
    assert got["left_sha256"] == exp["left_sha256"], f"{case}: seed left flags differ from ompVC's"
    assert got["eid_sha256"] == exp["eid_sha256"], f"{case}: seed element ids differ from ompVC's"
    return True


def load_fixture():
    with open(os.path.join(FIXTURE, "expected.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(FIXTURE, "ftle_summaries.npz")))
    return meta, arrays


def check_ftle_against_fixture(case, out_dir, meta, arrays, rtol=1e-12, atol=1e-13):
    """FTLE fields of a run against ompVC's, through the committed summaries:
    each strided value within rtol / atol, each block sum within rtol of the
    block's sum of magnitudes plus BLOCK * atol.  Returns the largest
    relative difference of the strided values."""
    worst = 0.0
    for f in FTLE_FILES:
        a = np.fromfile(os.path.join(out_dir, f), "<f8")
        exp = meta["cases"][case]["files"][f]
        assert a.nbytes == exp["bytes"], f"{case} {f}: {a.nbytes} bytes, ompVC wrote {exp['bytes']}"
        assert a[0] == exp["time"], f"{case} {f}: time stamp"
        v = a[1:]
        sub, ref = v[::STRIDE], arrays[f"{case}:{f}:sub"]
        np.testing.assert_allclose(sub, ref, rtol=rtol, atol=atol, err_msg=f"{case} {f} strided values")
        nb = len(v) // BLOCK
        blk = v[:nb * BLOCK].reshape(nb, BLOCK).sum(1)
        tol = rtol * arrays[f"{case}:{f}:absblk"] + BLOCK * atol
        bad = np.abs(blk - arrays[f"{case}:{f}:blk"]) > tol
        assert not bad.any(), f"{case} {f}: {int(bad.sum())} block sums differ from ompVC's"
        worst = max(worst, float((np.abs(sub - ref) / np.maximum(np.abs(ref), 1e-300)).max()))
    return worst


def check_exact_files(case, out_dir, meta, names=None):
    """Files that must be byte-identical to ompVC's (tracer outputs, the
    FTLE .info and _Cartesian files), by digest."""
    exp = meta["cases"][case]["files"]
    got = sorted(os.listdir(out_dir))
    assert got == sorted(exp), f"{case}: output files {got}, ompVC wrote {sorted(exp)}"
    for f in names if names is not None else [f for f in exp if f not in FTLE_FILES]:
        assert sha256(os.path.join(out_dir, f)) == exp[f]["sha256"], f"{case} {f}: bytes differ from ompVC's"
