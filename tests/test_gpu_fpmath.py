"""The helpers of flowvc-1_gb300/csrc/fvc_fpmath.cuh on the GPU: the
Markstein division must return exactly CUDA's IEEE quotient and the integer
FP32 truncation exactly __double2float_rz, on 2^28 seeded operands each
(wide exponents, element-volume scales, exact quotients, near-midpoint
quotients, division by 6 and the fallback edges); rn_root4 must be the
correctly rounded fourth root on seeded inputs; the comparisons and
conversions done on bit patterns must match the FP64 operations."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_div_rn_and_f32_trunc_match_ieee(tmp_path):
    exe = os.path.join(str(tmp_path), "fpmath_check")
    src = os.path.join(ROOT, "tests", "cuda", "fpmath_check.cu")
    inc = os.path.join(ROOT, "flowvc-1_gb300", "csrc")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-I", inc,
                    "-o", exe, src], check=True, capture_output=True)
    roots = os.path.join(str(tmp_path), "root4.bin")
    r = subprocess.run([exe, str(1 << 26), "4", roots], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["n_div"] == 1 << 28
    assert out["bad_div"] == 0, out
    assert out["bad_cvt"] == 0, out
    assert out["n_tiny"] == 1 << 26 and out["bad_tiny"] == 0, out
    assert out["n_bits"] == 1 << 26, out
    assert out["bad_lt"] == out["bad_floor"] == out["bad_i2d"] == out["bad_zero"] == 0, out
    # rn_root4: correctly rounded, checked exactly on the host with rationals
    # ((c -/+ half an ulp)^4 must bracket x).  The host libm's pow(x, 0.25),
    # which the reference's RKF calls, is not always correctly rounded: how
    # often it differs is printed, not asserted.
    xy = np.fromfile(roots, np.float64).reshape(-1, 2)
    assert len(xy) == 1 << 18
    for x, c in xy[:8192]:
        assert brackets(float(x), float(c)), (x, c)
    print("libm pow(x, 0.25) differs from the correctly rounded root in",
          int((xy[:, 1] != np.power(xy[:, 0], 0.25)).sum()), "of", len(xy))


def brackets(x, c):
    """True when c = RN(x^(1/4)): (c - u/2)^4 < x < (c + u/2)^4, u the
    spacing below / above c, in exact integer arithmetic."""
    from fractions import Fraction
    X = Fraction(x)
    lo = (Fraction(c) + Fraction(np.nextafter(c, 0.0))) / 2
    hi = (Fraction(c) + Fraction(np.nextafter(c, np.inf))) / 2
    return lo ** 4 < X < hi ** 4
