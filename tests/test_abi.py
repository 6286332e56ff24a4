"""The C-ABI library: it loads, and exports exactly what include/fvc.h declares."""
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared():
    src = open(os.path.join(ROOT, "include", "fvc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fvc_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("fvc_create", "fvc_advect", "fvc_ftle_interval", "fvc_ftle_reduce", "fvc_tracer_advance"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    import ctypes
    lib = ctypes.CDLL(engine.LIB)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(engine):
    import fvc
    assert sorted(fvc.SIGNATURES) == declared()
    lib = fvc.load()
    assert lib.fvc_abi_version() == 3


def test_create_without_gpu_fails_cleanly(engine):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import fvc
    with pytest.raises(fvc.FvcError):
        fvc.Context(3, 1)
