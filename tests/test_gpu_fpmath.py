"""The FP64-pipe savers (flowvc-1_gb300/csrc/fvc_fpmath.cuh) against CUDA's
IEEE operations on the GPU: the Markstein division must return exactly the
IEEE quotient and the integer FP32 truncation exactly __double2float_rz, on
2^28 seeded operands each (wide exponents, element-volume scales, exact
quotients, near-midpoint quotients, division by 6 and the fallback edges)."""
import json
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_div_rn_and_f32_trunc_match_ieee(tmp_path):
    exe = os.path.join(str(tmp_path), "fpmath_check")
    src = os.path.join(ROOT, "tests", "cuda", "fpmath_check.cu")
    inc = os.path.join(ROOT, "flowvc-1_gb300", "csrc")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-I", inc,
                    "-o", exe, src], check=True, capture_output=True)
    r = subprocess.run([exe, str(1 << 26), "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["n_div"] == 1 << 28
    assert out["bad_div"] == 0, out
    assert out["bad_cvt"] == 0, out
