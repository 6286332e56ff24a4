"""The CPU oracle against ompVC at the benchmark configurations' full sizes.

ompVC itself ran once on these inputs (tests/golden/scale/make_scale_golden.py)
and its outputs are committed as digests and FTLE summaries.  Here the oracle
runs on the same inputs, regenerated byte for byte (their digests are checked
first), and must reproduce them: tracer files, FTLE .info and _Cartesian files
byte-identical, FTLE fields within the tolerance of conftest (the oracle's
eigen-solver is its own) through every 509th value and block sums.  The
oracle is the checker of the GPU engine (tests/test_gpu_scale.py), so this
pins it where the engine is measured, not only on the small golden cases.
"""
import os
import subprocess

import pytest

import scale_cases as sc
from conftest import FTLE_ATOL, FTLE_RTOL


@pytest.fixture(scope="module")
def scale_data(tmp_path_factory):
    meta, arrays = sc.load_fixture()
    root = str(tmp_path_factory.mktemp("scale"))
    return root, meta, arrays


def run_oracle(oracle_bin, case, root, meta):
    kind, _ = sc.CASES[case]
    data = sc.make_inputs(kind, root)
    assert sc.input_digests(data) == meta["inputs"][kind], \
        "generated inputs differ from the ones ompVC ran on: regenerate the fixture"
    out = os.path.join(root, "orc_" + case)
    inp = sc.write_in(case, data, out, os.path.join(root, case + ".in"))
    r = subprocess.run([oracle_bin, inp, str(os.cpu_count() or 1)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


@pytest.mark.parametrize("case", ["cube_ftle_5", "cube_ftle", "dg_ftle"])
def test_oracle_ftle_matches_ompvc_at_scale(oracle_bin, scale_data, case):
    root, meta, arrays = scale_data
    out = run_oracle(oracle_bin, case, root, meta)
    sc.check_exact_files(case, out, meta)
    sc.check_ic_against_fixture(case, os.path.join(root, sc.CASES[case][0], "ftle_ic.bin"), meta)
    worst = sc.check_ftle_against_fixture(case, out, meta, arrays, rtol=FTLE_RTOL, atol=FTLE_ATOL)
    print(case, "largest relative FTLE difference from ompVC (strided values):", worst)


def test_oracle_tracers_match_ompvc_at_scale(oracle_bin, scale_data):
    root, meta, arrays = scale_data
    out = run_oracle(oracle_bin, "cube_tracers", root, meta)
    sc.check_exact_files("cube_tracers", out, meta)
