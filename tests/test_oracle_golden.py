"""The CPU oracle against ompVC's own outputs (the golden fixtures).

Tracer, residence-time and exposure-time files must be byte-identical (the
oracle adds exposure times in ompVC's serial order); FTLE fields agree within
the tolerance in conftest (only the eigen-solver differs from the
reference's), and the located seed grid of every FTLE run on an
unstructured mesh (element ids, left flags) is ompVC's byte for byte.  Files
that depend on undefined behaviour in ompVC are listed in
conftest.REFERENCE_UNDEFINED."""
import os

import pytest

from conftest import GOLDEN, check_ic, compare_outputs, golden_cases, run_golden, undefined_files


@pytest.mark.parametrize("case,run", golden_cases())
def test_oracle_matches_reference(oracle_bin, tmp_path, case, run):
    out, _ = run_golden(oracle_bin, case, run, tmp_path)
    compare_outputs(os.path.join(GOLDEN, case, "expected", run), out, skip=undefined_files(case, run))
    check_ic(case, run, tmp_path, "oracle")  # the located seed grid, byte for byte
