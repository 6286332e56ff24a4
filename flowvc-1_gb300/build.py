"""Build recipe for the engine: libfvc.so (CUDA, sm_103a) and the fvcflow host.

Everything is compiled in-tree into flowvc-1_gb300/build/ with explicit nvcc
and gcc commands (no cmake), translation units in parallel.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "build")
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libfvc.so")
FVCFLOW = os.path.join(BUILD, "fvcflow")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: the FP64 path reproduces ompVC's separately rounded multiply
# and add; -lineinfo keeps source correlation for ncu.
NVFLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["fvc_kernels.cu", "fvc_api.cu", "fvc_variant_c2.cu", "fvc_variant_c3.cu",
              "fvc_variant_u2.cu", "fvc_variant_u3.cu", "fvc_variant_u2m.cu", "fvc_variant_u3m.cu",
              "fvc_mixed_kernels.cu", "fvc_cet.cu", "fvc_batch.cu"]
# resident 128-thread blocks per SM the integrator kernels are compiled for
# (register budget 65536 / (128 * n)); FVC_MINBLOCKS overrides it for sweeps
MINBLOCKS = os.environ.get("FVC_MINBLOCKS", "4")
MX_MINBLOCKS = os.environ.get("FVC_MX_MINBLOCKS", "4")
TASK_MINBLOCKS = os.environ.get("FVC_TASK_MINBLOCKS", "3")
# batch ticks queued on the GPU at once (FVC_BATCH_INFLIGHT overrides it)
BATCH_INFLIGHT = os.environ.get("FVC_BATCH_INFLIGHT", "2")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    out = [os.path.abspath(__file__)]
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def build_lib(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _newer(obj, deps):
            jobs.append([NVCC, *ARCH, *NVFLAGS, "-DFVC_MINBLOCKS=" + MINBLOCKS, "-DFVC_MX_MINBLOCKS=" + MX_MINBLOCKS,
                         "-DFVC_TASK_MINBLOCKS=" + TASK_MINBLOCKS, "-DFVC_BATCH_INFLIGHT=" + BATCH_INFLIGHT,
                         "-c", os.path.join(CSRC, src),
                         "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    if force or jobs or _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


def build_host(force=False):
    srcs = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".c")] if os.path.isdir(HOST) else []
    if not srcs:
        return None
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    if force or _newer(FVCFLOW, srcs + hdrs + [LIB, os.path.join(INCLUDE, "fvc.h")]):
        _run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-Wall", "-Wno-format-truncation", "-I" + INCLUDE, *srcs,
              "-L" + BUILD, "-lfvc", "-Wl,-rpath,$ORIGIN", "-lm", "-pthread", "-o", FVCFLOW])
    return FVCFLOW


def build(force=False, verbose=False):
    build_lib(force=force, verbose=verbose)
    build_host(force=force)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
