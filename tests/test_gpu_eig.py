"""The FTLE eigenvalue on the GPU (flowvc-1_gb300/csrc/fvc_ftle_math.cuh):
the closed form on C - I must agree with LAPACK's symmetric solver on
seeded Cauchy-Green tensors from the identity to strongly stretching ones,
hand the ill-conditioned ones (two largest eigenvalues nearly equal) to
the Jacobi solver, and the Jacobi solver must agree as well.  Compared as
FTLE values, 0.5 log1p(lambda - 1), within the golden tests' 1e-12
relative / 1e-13 absolute."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def tensors(rng, n):
    """C - I for F = Q1 diag(s) Q2 in five families: log-normal stretches,
    near-rigid motions (deviations 1e-6 .. 1e-1), two largest stretches
    nearly equal, two smallest nearly equal, mild stretches; plus exact
    cases (identity, diagonal)."""
    out, fam = [], []
    for it in range(n):
        kind = it % 5
        q1, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        q2, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        if kind == 0:
            s = np.exp(rng.normal(0, 2, 3))
        elif kind == 1:
            s = 1 + rng.normal(0, 10 ** rng.uniform(-6, -1), 3)
        elif kind == 2:
            x = np.exp(rng.uniform(0, 4))
            s = np.array([x, x * (1 + rng.normal(0, 10 ** rng.uniform(-6, -1))), 1 / x ** 2])
        elif kind == 3:
            x = np.exp(rng.uniform(0, 4))
            s = np.array([x * x, (1 + rng.normal(0, 1e-3)) / x, 1 / x])
        else:
            s = np.exp(rng.normal(0, 0.5, 3))
        F = q1 @ np.diag(s) @ q2
        out.append(F.T @ F - np.eye(3))
        fam.append(kind)
    out.append(np.zeros((3, 3)))
    fam.append(5)
    out.append(np.diag([0.5, -0.25, 3.0]))
    fam.append(5)
    return np.array(out), np.array(fam)


def test_closed_form_and_jacobi_agree_with_lapack(tmp_path):
    exe = os.path.join(str(tmp_path), "eig_check")
    src = os.path.join(ROOT, "tests", "cuda", "eig_check.cu")
    inc = os.path.join(ROOT, "flowvc-1_gb300", "csrc")
    inc2 = os.path.join(ROOT, "include")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I", inc, "-I", inc2, "-o", exe, src], check=True, capture_output=True)
    rng = np.random.default_rng(7)
    A, fam = tensors(rng, 20000)
    fin = os.path.join(str(tmp_path), "C.bin")
    fout = os.path.join(str(tmp_path), "out.bin")
    A.astype(np.float64).tofile(fin)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(fout, np.float64).reshape(-1, 3)
    closed, ok, jac = out[:, 0], out[:, 1] > 0.5, out[:, 2]
    ref = np.linalg.eigvalsh(A)[:, -1]
    keep = ref > -1.0 + 1e-3  # lambda well above 0, so log1p is defined

    def ftle(lm1):
        return 0.5 * np.log1p(lm1)

    tol = lambda f: 1e-12 * np.abs(f) + 1e-13  # noqa: E731
    f_ref = ftle(ref[keep])
    # the closed form where it accepts the matrix
    sel = keep & ok
    assert np.all(np.abs(ftle(closed[sel]) - ftle(ref[sel])) <= tol(ftle(ref[sel])))
    # the Jacobi solver on every matrix
    assert np.all(np.abs(ftle(jac[keep]) - f_ref) <= tol(f_ref))
    # what the closed form leaves: mostly the nearly equal largest pairs, few others
    assert ok[fam == 3].all() and ok[fam == 5].all()
    assert (~ok[fam == 2]).mean() > 0.5
    assert (~ok[(fam == 0) | (fam == 4)]).mean() < 0.05
