"""Build the GB300 imaging libraries in-tree with nvcc (sm_103a only).

Produces ``bullseye_gb300/lib/libgpu_imaging32.so`` and ``libgpu_imaging64.so`` from
the ``.cu`` files under ``bullseye_gb300/csrc``, compiled once per precision (``-DBULLSEYE_SINGLE`` /
``-DBULLSEYE_DOUBLE``), the two compiles running in parallel.  Nothing is installed outside the
repository.  The build is incremental: a library is rebuilt when any source under ``csrc`` is
newer than it.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def library_path(precision: str) -> str:
    return os.path.join(LIBDIR, "libgpu_imaging%s.so" % ("32" if precision == "single" else "64"))


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(CSRC, "*.h")) + [os.path.abspath(__file__)])


def _cmd(precision: str, out: str, verbose_ptxas: bool = False):
    ch = cuda_home()
    macro = "-DBULLSEYE_SINGLE" if precision == "single" else "-DBULLSEYE_DOUBLE"
    cmd = [os.path.join(ch, "bin", "nvcc"), *ARCH, "-O3", "-lineinfo", "-std=c++17", macro, "--threads", "4",
           "-Xcompiler", "-fPIC", "-shared", "--expt-relaxed-constexpr",
           os.path.join(CSRC, "imaging_lib.cu"), os.path.join(CSRC, "noalloc.cu"),
           os.path.join(CSRC, "batched.cu"), os.path.join(CSRC, "adjoint.cu"),
           os.path.join(CSRC, "sampling_nn.cu"), os.path.join(CSRC, "rows.cu"), "-o", out,
           "-L" + os.path.join(ch, "lib64"), "-lcufft",
           "-Xlinker", "-rpath," + os.path.join(ch, "lib64")]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    return cmd


def build(force: bool = False, verbose_ptxas: bool = False) -> list[str]:
    """Compile both precisions if out of date; returns the library paths."""
    os.makedirs(LIBDIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in _sources())
    procs = []
    outs = []
    for prec in ("single", "double"):
        out = library_path(prec)
        outs.append(out)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        tmp = out + ".tmp"
        procs.append((subprocess.Popen(_cmd(prec, tmp, verbose_ptxas), stdout=subprocess.PIPE,
                                       stderr=subprocess.STDOUT, text=True), tmp, out))
    errors = []
    for pr, tmp, out in procs:
        log, _ = pr.communicate()
        if pr.returncode != 0:
            errors.append(log)
        else:
            if verbose_ptxas and log:
                print(log)
            os.replace(tmp, out)
    if errors:
        raise RuntimeError("nvcc build failed:\n" + "\n".join(errors))
    return outs


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
