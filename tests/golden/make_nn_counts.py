"""Generate tests/golden/nn_counts_<precision>.npz with the reference's own nearest-neighbour policy.

Runs the reference CPU gridder instantiated with convolution_NN on the sampling function
(oracle/ref_nn_harness.cpp, compiled from the reference's headers by oracle/build_ref.sh) on the
inputs of nn_cases.make_inputs, in grid and facet mode, and stores the integer counts (the real
parts of the sampling-function grid).

Usage: python tests/golden/make_nn_counts.py
"""
from __future__ import annotations

import ctypes
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from bullseye_gb300.abi import complex_dtype  # noqa: E402
from nn_cases import FACETS, NX, NY, SF_CH, host_ptr, make_inputs, make_struct  # noqa: E402
from oracle.harness import REF, build_reference  # noqa: E402


def main():
    build_reference()
    for prec, suffix in (("single", "32"), ("double", "64")):
        lib = ctypes.CDLL(os.path.join(REF, f"libref_nn{suffix}.so"))
        lib.ref_sampling_counts_nn.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_sampling_counts_nn.restype = None
        d = make_inputs(prec)
        out = {f"in_{k}": v for k, v in d.items()}
        for faceting in (0, 1):
            F = FACETS if faceting else 1
            buf = np.zeros((F, SF_CH, NY, NX), complex_dtype(prec))
            st = make_struct(prec, d, bool(faceting), host_ptr, host_ptr(buf))
            lib.ref_sampling_counts_nn(ctypes.byref(st), faceting)
            assert np.all(buf.imag == 0) and np.all(buf.real == np.round(buf.real))
            out[f"counts_{'facet' if faceting else 'grid'}"] = buf.real.astype(np.uint32)
        path = os.path.join(HERE, f"nn_counts_{prec}.npz")
        np.savez_compressed(path, **out)
        print("wrote", path, {k: int(v.sum()) for k, v in out.items() if k.startswith("counts")})


if __name__ == "__main__":
    main()
