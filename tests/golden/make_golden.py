"""Regenerate the golden fixtures in this directory from the reference's own CPU library.

Usage (needs the reference tree and g++; single-threaded so the reference's per-thread rounding
mode is the same for every facet):

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py

It builds oracle/_ref (oracle/build_ref.sh), creates each seeded problem of cases.CASES, runs the
reference library through the pipeliner's ABI sequence (bullseye_gb300.imaging.run_imaging) and
stores inputs and outputs in <case>_<precision>.npz.
"""
import os
import sys

os.environ.setdefault("OMP_NUM_THREADS", "1")
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from bullseye_gb300 import synth  # noqa: E402
from bullseye_gb300.imaging import run_imaging  # noqa: E402
from cases import CASES, PRECISIONS, case_path, cpu_conv, problem_to_arrays  # noqa: E402
from oracle.harness import build_reference, load_reference  # noqa: E402


def main():
    if not build_reference():
        raise SystemExit("reference sources not available")
    for prec in PRECISIONS:
        lib = load_reference(prec)
        for name, (call, pkw, rkw) in CASES.items():
            p = synth.small_problem(prec, **pkw)
            res = run_imaging(lib, p.with_conv(cpu_conv(p)), call, keep_raw=True, **rkw)
            out = problem_to_arrays(p)
            out["out_raw_grid"] = res.raw_grid
            out["out_grid"] = res.grid
            out["out_normalization"] = res.normalization
            for k in ("sampling", "image", "psf"):
                v = getattr(res, k)
                if v is not None:
                    out["out_" + k] = v
            out["call"] = np.asarray(call)
            np.savez_compressed(case_path(name, prec), **out)
            print("wrote", case_path(name, prec))


if __name__ == "__main__":
    main()
