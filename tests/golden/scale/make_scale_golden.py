"""Generate the full-size fixtures under tests/golden/scale/ by running the
reference.

For every case of tests/scale_cases.py this script writes the inputs,
runs the unmodified ompVC program built from the reference sources
(oracle/Makefile.ref -> oracle/_ref/ompflowVC) and stores, instead of the
outputs themselves (tens of MB each), their summaries:

  expected.json        SHA-256 and size of every output file, the FTLE time
                       stamps, the SHA-256 of every input file, of the
                       located seed grid's element ids and left flags
                       (ompVC's FTLE_ICFile), and the wall time and
                       settings of each ompVC run
  ftle_summaries.npz   per FTLE field every 509th value and the sums of
                       blocks of 4096 values (with the sums of magnitudes)

ompVC runs as its input files ask: FTLE with one output slide runs on one
core (UPPERLOOP), tracers on Num_threads cores (TRACER_LOWERLOOP).  The
whole script takes about ten minutes on one x86-64 core for the FTLE
cases.

Usage:  python tests/golden/scale/make_scale_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.join(ROOT, "flowvc-1_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import scale_cases as sc  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ompflowVC")


def main(names):
    if not os.path.exists(REF):
        sys.exit(f"{REF} is missing: build it with make -f oracle/Makefile.ref")
    jpath = os.path.join(HERE, "expected.json")
    npath = os.path.join(HERE, "ftle_summaries.npz")
    meta = json.load(open(jpath)) if os.path.exists(jpath) else {"inputs": {}, "cases": {}}
    arrays = dict(np.load(npath)) if os.path.exists(npath) else {}
    nthreads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as td:
        for case in names:
            kind, _ = sc.CASES[case]
            data = sc.make_inputs(kind, td)
            meta["inputs"][kind] = sc.input_digests(data)
            out = os.path.join(td, "out_" + case)
            inp = sc.write_in(case, data, out, os.path.join(td, case + ".in"), Num_threads=nthreads)
            t0 = time.time()
            r = subprocess.run([REF, inp], capture_output=True, text=True)
            wall = time.time() - t0
            if r.returncode:
                sys.exit(f"ompVC failed on {case}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
            files, arr = sc.summarise(out)
            meta["cases"][case] = {"files": files, "ompvc_wall_s": round(wall, 2), "host_threads": nthreads}
            ic = os.path.join(data, "ftle_ic.bin")
            if sc.CASES[case][1].get("FTLE_Compute") and kind == "cube" and os.path.exists(ic):
                # the located seed grid: element ids and left flags
                meta["cases"][case]["ic"] = sc.ic_digests(ic)
                os.remove(ic)
            for k in [k for k in arrays if k.startswith(case + ":")]:
                del arrays[k]
            arrays.update({f"{case}:{k}": v for k, v in arr.items()})
            print(f"{case}: ompVC {wall:.1f} s, {len(files)} files", flush=True)
    with open(jpath, "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    np.savez_compressed(npath, **arrays)


if __name__ == "__main__":
    main(sys.argv[1:] or list(sc.CASES))
