"""Loaders for the oracle libraries.  TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and the CPU-baseline leg of bench.py import this module.  It builds
and loads:

* ``oracle/_build/liboracle_cpu{32,64}.so`` -- the C restatement of the reference CPU imaging
  library (oracle/bullseye_oracle.c), compiled here and on any machine with gcc;
* ``oracle/_ref/libcpu_imaging{32,64}.so`` -- the reference's own CPU library compiled from its
  sources by oracle/build_ref.sh (only where the reference tree is present).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from bullseye_gb300.abi import bind_exports  # noqa: E402

BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
_SUFFIX = {"single": "32", "double": "64"}


def build_oracle(force: bool = False) -> None:
    """Compile the C restatement in both precisions (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    src = [os.path.join(HERE, "bullseye_oracle.c"), os.path.join(HERE, "fftw_shim.c")]
    newest = max(os.path.getmtime(s) for s in src + [os.path.join(HERE, "shim", "fftw3.h")])
    procs = []
    for prec, macro in (("single", "ORACLE_SINGLE"), ("double", "ORACLE_DOUBLE")):
        out = os.path.join(BUILD, f"liboracle_cpu{_SUFFIX[prec]}.so")
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["gcc", f"-D{macro}", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-I" + HERE, *src, "-o", out, "-lm"]
        procs.append(subprocess.Popen(cmd))
    for pr in procs:
        if pr.wait() != 0:
            raise RuntimeError("oracle build failed")


def build_reference() -> bool:
    """Build oracle/_ref from the reference sources when they are present; True if available."""
    script = os.path.join(HERE, "build_ref.sh")
    have = all(os.path.exists(os.path.join(REF, f"libcpu_imaging{s}.so")) for s in ("32", "64"))
    if not have:
        subprocess.run(["bash", script], check=True)
    return all(os.path.exists(os.path.join(REF, f"libcpu_imaging{s}.so")) for s in ("32", "64"))


def _load(path: str):
    lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0)
    return bind_exports(lib)


def load_oracle(precision: str):
    build_oracle()
    lib = _load(os.path.join(BUILD, f"liboracle_cpu{_SUFFIX[precision]}.so"))
    lib.oracle_last_error.restype = ctypes.c_int
    lib.oracle_last_error.argtypes = []
    lib.oracle_sampling_counts_nn.restype = None
    lib.oracle_sampling_counts_nn.argtypes = [ctypes.c_void_p, ctypes.c_int]
    return lib


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REF, f"libcpu_imaging{s}.so")) for s in ("32", "64"))


def load_reference(precision: str):
    """The reference's own CPU library (x86-64 build here).  Raises if it is not built."""
    path = os.path.join(REF, f"libcpu_imaging{_SUFFIX[precision]}.so")
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    return _load(path)
