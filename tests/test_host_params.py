"""fvcflow's .in handling: ompVC's positional format, refused options."""
import os
import subprocess

import pytest

import synth


def _run(engine, path):
    return subprocess.run([engine.FVCFLOW, path], capture_output=True, text=True)


@pytest.mark.parametrize("over,msg", [
    (dict(Int_Type=2, Int_Accuracy=0.0), "RKF integration parameters must be positive"),
    (dict(Particle_Radius=0.1), "inertial"),
    (dict(Trace_Compute=1, FTLE_Compute=1), "concurrently"),
    (dict(Int_TimeDirection=2), "Int_TimeDirection"),
    (dict(Data_TRes=1), "Data_TRes"),
    (dict(FTLE_Compute=0), "nothing to compute"),
])
def test_refused_before_any_gpu_work(engine, tmp_path, over, msg):
    p = str(tmp_path / "x.in")
    base = dict(Path_Data=str(tmp_path), Path_Output=str(tmp_path), Dimensions=3, Data_MeshType=1,
                Data_InFilePrefix="none", Data_TRes=11, Data_TDelta=0.1, FTLE_Compute=1,
                **{"Data_MeshBounds.XMin": 0.0, "Data_MeshBounds.XMax": 1.0, "Data_MeshBounds.YMin": 0.0,
                   "Data_MeshBounds.YMax": 1.0, "Data_MeshBounds.ZMin": 0.0, "Data_MeshBounds.ZMax": 1.0,
                   "FTLE_MeshBounds.ZMax": 1.0, "FTLE_MeshBounds.ZRes": 2})
    base.update(over)
    synth.write_in_file(p, **base)
    r = _run(engine, p)
    assert r.returncode != 0
    assert msg in r.stderr


def test_truncated_in_file(engine, tmp_path):
    p = str(tmp_path / "t.in")
    with open(p, "w") as f:
        f.write("# comment only\nPath_Data = pwd\nPath_Output = pwd\n")
    r = _run(engine, p)
    assert r.returncode != 0 and "could not read parameter" in r.stderr


def test_missing_in_file(engine, tmp_path):
    r = _run(engine, str(tmp_path / "nope.in"))
    assert r.returncode != 0 and "Could not open input file" in r.stderr


def test_unknown_precision_refused(engine, tmp_path):
    r = subprocess.run([engine.FVCFLOW, str(tmp_path / "x.in"), "--precision", "fp8"], capture_output=True, text=True)
    assert r.returncode != 0 and "unknown precision 'fp8'" in r.stderr
