"""Record, for every FTLE run of the golden cases on unstructured meshes,
the located seed grid ompVC writes at initialisation (its FTLE_ICFile:
element ids and left flags, as SHA-256 digests) in
tests/golden/<case>/ic.json.

The runs use the committed inputs and parameters (the same .in files the
tests write), so only the digests are new; the other fixture files are not
touched.  Needs the reference program built from its sources
(oracle/Makefile.ref -> oracle/_ref/ompflowVC).

Usage:  python tests/golden/make_ic_digests.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "flowvc-1_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import scale_cases as sc  # noqa: E402
import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ompflowVC")


def main():
    if not os.path.exists(REF):
        sys.exit(f"{REF} is missing: build it with make -f oracle/Makefile.ref")
    for case in sorted(os.listdir(HERE)):
        pj = os.path.join(HERE, case, "params.json")
        if not os.path.exists(pj):
            continue
        P = json.load(open(pj))
        if P["base"].get("Data_MeshType") != 1:
            continue
        digests = {}
        for run in sorted(P["runs"]):
            params = dict(P["base"], **P["runs"][run])
            if not params.get("FTLE_Compute"):
                continue
            with tempfile.TemporaryDirectory() as td:
                data = os.path.join(td, "in")
                shutil.copytree(os.path.join(HERE, case, "inputs"), data)
                out = os.path.join(td, "out")
                os.makedirs(out)
                inp = os.path.join(td, "run.in")
                synth.write_in_file(inp, **dict(params, Path_Data=data + "/", Path_Output=out + "/"))
                r = subprocess.run([REF, inp], capture_output=True, text=True)
                if r.returncode:
                    sys.exit(f"ompVC failed on {case} {run}:\n{r.stdout[-2000:]}")
                digests[run] = sc.ic_digests(os.path.join(data, params.get("FTLE_ICFile", "ftle_ic.bin")))
            print(case, run, digests[run]["n"], "seeds", flush=True)
        if digests:
            with open(os.path.join(HERE, case, "ic.json"), "w") as f:
                json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
