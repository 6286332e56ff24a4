"""The CPU oracle against ompVC's own outputs (the golden fixtures).

Tracer files must be byte-identical; FTLE fields agree within the tolerance
in conftest (only the eigen-solver differs from the reference's)."""
import os

import pytest

from conftest import GOLDEN, compare_outputs, golden_cases, run_golden


@pytest.mark.parametrize("case,run", golden_cases())
def test_oracle_matches_reference(oracle_bin, tmp_path, case, run):
    out, _ = run_golden(oracle_bin, case, run, tmp_path)
    compare_outputs(os.path.join(GOLDEN, case, "expected", run), out)
