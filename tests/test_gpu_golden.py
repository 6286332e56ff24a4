"""The GPU engine (fvcflow over libfvc) against ompVC's outputs and the oracle.

Tracer files and FTLE grid states (positions, element ids, exit flags) must
be bit-identical to the oracle; tracer files byte-identical to ompVC's; FTLE
fields within the tolerance in conftest."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, compare_outputs, golden_cases, run_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,run", golden_cases())
def test_engine_matches_reference(engine, oracle_bin, tmp_path, case, run):
    dump_g = tmp_path / "dump_gpu"
    dump_o = tmp_path / "dump_orc"
    dump_g.mkdir()
    dump_o.mkdir()
    got, _ = run_golden(engine.FVCFLOW, case, run, tmp_path, extra_args=("--dump-state", str(dump_g)))
    compare_outputs(os.path.join(GOLDEN, case, "expected", run), got)
    os.environ["ORC_DUMP_STATE"] = str(dump_o)
    try:
        orc, _ = run_golden(oracle_bin, case, run, tmp_path)
    finally:
        del os.environ["ORC_DUMP_STATE"]
    # against the oracle: FTLE to a few ulps (CUDA's log vs glibc's), the rest exact
    compare_outputs(orc, got, ftle_rtol=1e-14, ftle_atol=1e-15)
    for f in sorted(os.listdir(dump_o)):
        a = np.fromfile(dump_o / f, np.uint8)
        b = np.fromfile(dump_g / f, np.uint8)
        n = int(a[:4].view(np.int32)[0])
        Xa = a[4:4 + 24 * n].view(np.float64)
        Xb = b[4:4 + 24 * n].view(np.float64)
        ia = a[4 + 24 * n:].view(np.int32).reshape(3, n)
        ib = b[4 + 24 * n:].view(np.int32).reshape(3, n)
        live = ia[1] == 0
        assert np.array_equal(Xa, Xb), f"{f}: positions differ"
        assert np.array_equal(ia[1], ib[1]), f"{f}: left flags differ"
        assert np.array_equal(ia[2] != 0, ib[2] != 0), f"{f}: have flags differ"
        assert np.array_equal(ia[0][live], ib[0][live]), f"{f}: element ids differ"
