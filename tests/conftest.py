"""Shared fixtures: build the oracle (CPU, test infrastructure) and the engine,
and run golden cases through either program."""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "flowvc-1_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA engine)")


@pytest.fixture(scope="session")
def oracle_bin():
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return os.path.join(ROOT, "oracle", "build", "orcflow")


@pytest.fixture(scope="session")
def engine():
    import build as fvc_build
    fvc_build.build()
    return fvc_build


def undefined_files(case, run):
    return {f for c, r, f in REFERENCE_UNDEFINED if (c, r) == (case, run)}


def golden_cases():
    out = []
    for name in sorted(os.listdir(GOLDEN)):
        pj = os.path.join(GOLDEN, name, "params.json")
        if os.path.exists(pj):
            with open(pj) as f:
                P = json.load(f)
            for run in sorted(P["runs"]):
                out.append((name, run))
    return out


def run_golden(exe, case, run, tmp_path, extra_args=()):
    """Run `exe` on golden case/run with inputs copied under tmp_path; returns the output dir."""
    import synth
    with open(os.path.join(GOLDEN, case, "params.json")) as f:
        P = json.load(f)
    data = os.path.join(str(tmp_path), case + "_in")
    if not os.path.exists(data):
        shutil.copytree(os.path.join(GOLDEN, case, "inputs"), data)
    out = os.path.join(str(tmp_path), case + "_" + run + "_" + os.path.basename(exe))
    os.makedirs(out, exist_ok=True)
    inp = os.path.join(str(tmp_path), f"{case}_{run}.in")
    synth.write_in_file(inp, **dict(P["base"], **P["runs"][run], Path_Data=data + "/", Path_Output=out + "/"))
    r = subprocess.run([exe, inp, *extra_args], capture_output=True, text=True)
    assert r.returncode == 0, f"{exe} failed:\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}"
    return out, r.stdout


def check_ic(case, run, tmp_path, who):
    """The located seed grid a run wrote (its FTLE_ICFile in the case's copied
    inputs: left flags, and element ids of the seeds inside -- ompVC leaves
    the others unset) against ompVC's for the same run
    (tests/golden/<case>/ic.json, made by tests/golden/make_ic_digests.py).
    Returns False when the run has no recorded grid."""
    import scale_cases as sc
    pj = os.path.join(GOLDEN, case, "ic.json")
    if not os.path.exists(pj):
        return False
    with open(pj) as f:
        exp = json.load(f).get(run)
    if exp is None:
        return False
    got = sc.ic_digests(os.path.join(str(tmp_path), case + "_in", "ftle_ic.bin"))
    assert got["n"] == exp["n"], f"{who} {case} {run}: {got['n']} seeds in the IC file, ompVC wrote {exp['n']}"
    assert got["left_sha256"] == exp["left_sha256"], f"{who} {case} {run}: seed left flags differ from ompVC's"
    assert got["eid_inside_sha256"] == exp["eid_inside_sha256"], \
        f"{who} {case} {run}: element ids of seeds inside differ from ompVC's"
    return True


# FTLE fields: the engine computes the Cauchy-Green eigenvalue with its own
# solvers (the trigonometric closed form on C - I, Jacobi where that is
# ill-conditioned; the reference uses Householder + QL on C), so FTLE values
# agree to a few ulps of lambda; log(lambda) amplifies the reference's
# rounding near lambda = 1.  Positions and tracer outputs are compared bit
# for bit.
FTLE_RTOL = 1e-12
FTLE_ATOL = 1e-13


# Exposure-time sums (<RT>_CET / _MET files): the GPU adds each element's
# contributions with atomics, in an order of its own, so sums of many terms
# can differ from ompVC's serial order in their last bits.
CET_RTOL = 1e-12

# Files whose content in ompVC depends on undefined behaviour.  OutputRT
# (ompVC/residencetime.c:154) discards the buffer ReadInTraceLaunch returns
# and reads through the pointer that WriteOutTraceLaunch freed
# (ompVC/tracers.c:1649-1656, 1689-1695): with glibc's reuse of freed blocks
# release 0 comes out right and every later release repeats release 0's
# tracer states.  The engine writes each release's own residence times; these
# files are compared with the oracle only.
REFERENCE_UNDEFINED = {("cube", "tracer_rt", "rt.1.bin"), ("tri", "tracer_rt", "rt.1.bin")}


def compare_outputs(expected_dir, got_dir, ftle_rtol=FTLE_RTOL, ftle_atol=FTLE_ATOL, skip=(), cet_rtol=0.0):
    exp = sorted(os.listdir(expected_dir))
    got = sorted(f for f in os.listdir(got_dir))
    assert exp == got, f"output files differ: expected {exp}, got {got}"
    for f in exp:
        if f in skip:
            continue
        a = open(os.path.join(expected_dir, f), "rb").read()
        b = open(os.path.join(got_dir, f), "rb").read()
        if (f.endswith((".info", "_Cartesian.bin", "_coordinates.bin", "_ENC.0.bin")) or f.startswith("tracer")
                or f.startswith("rt.")):
            assert a == b, f"{f}: bytes differ"
            continue
        if f.endswith(("_CET.0.bin", "_MET.0.bin")):
            A, B = np.frombuffer(a, "<f8"), np.frombuffer(b, "<f8")
            assert len(A) == len(B) and A[0] == B[0], f"{f}: length or time stamp"
            if cet_rtol == 0.0:
                assert a == b, f"{f}: bytes differ"
            else:
                np.testing.assert_allclose(B[1:], A[1:], rtol=cet_rtol, atol=0, err_msg=f)
            continue
        assert len(a) == len(b), f"{f}: length {len(a)} != {len(b)}"
        A = np.frombuffer(a, "<f8")
        B = np.frombuffer(b, "<f8")
        assert A[0] == B[0], f"{f}: time stamp"
        np.testing.assert_allclose(B[1:], A[1:], rtol=ftle_rtol, atol=ftle_atol, err_msg=f)


def compare_state_dumps(dump_expected, dump_got):
    """FTLE grid states written by `--dump-state` (fvcflow) and ORC_DUMP_STATE
    (the oracle): int32 n, n x 3 positions, then element ids, left flags and
    have-FTLE flags (n int32 each).  Positions, left flags and have flags
    must be identical, element ids wherever the point is still inside."""
    files = sorted(os.listdir(dump_expected))
    assert files == sorted(os.listdir(dump_got)), "state dumps differ in number"
    for f in files:
        a = np.fromfile(os.path.join(dump_expected, f), np.uint8)
        b = np.fromfile(os.path.join(dump_got, f), np.uint8)
        assert a.size == b.size, f"{f}: sizes differ"
        n = int(a[:4].view(np.int32)[0])
        Xa = a[4:4 + 24 * n].view(np.float64)
        Xb = b[4:4 + 24 * n].view(np.float64)
        ia = a[4 + 24 * n:].view(np.int32).reshape(3, n)
        ib = b[4 + 24 * n:].view(np.int32).reshape(3, n)
        live = ia[1] == 0
        assert np.array_equal(Xa, Xb), f"{f}: positions differ at {int((Xa != Xb).sum())} coordinates"
        assert np.array_equal(ia[1], ib[1]), f"{f}: left flags differ"
        assert np.array_equal(ia[2] != 0, ib[2] != 0), f"{f}: have flags differ"
        assert np.array_equal(ia[0][live], ib[0][live]), f"{f}: element ids differ"
    return len(files)
