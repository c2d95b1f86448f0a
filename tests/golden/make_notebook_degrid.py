"""Generate tests/golden/notebook_degrid.npz by running the reference's prototype degridder.

Runs cells 16 (filter) and 17 (degridder) of the reference's
writing_and_wiki/notebooks/Resampling.ipynb as written, on a seeded random model grid and seeded
uv points, and stores inputs and outputs.  The notebook is Python 2 era code; three stand-ins let
the two cells run unchanged: ``np.complex`` (removed from numpy) is the builtin complex, the
filter array truncates float indices (as numpy of that time did), and ``plt`` is a no-op.

The uv points keep clear of decision boundaries so that single-precision coordinates select the
same cells and taps: |frac(u) - 1/2| > 1e-3 (the rounding of the centre cell) and the
fractional part of the filter offset (1 - u + round(u)) * OVERSAMPLE is in (1e-3, 1 - 1e-3).
Most points lie where both the notebook and the imaging library accept them; the last rows sit
at the grid edge, where the notebook skips them or reads wrapped cells.

Usage: python tests/golden/make_notebook_degrid.py [path to the reference checkout]
"""
from __future__ import annotations

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
N = 64
ROWS = 400
EDGE_ROWS = 8
SEED = 1717


class _TruncIndex:
    """The notebook's filter array: float indices truncate."""

    def __init__(self, a):
        self.a = a

    def __getitem__(self, i):
        return self.a[int(i)]


class _NoPlot:
    def __getattr__(self, name):
        return lambda *a, **k: None


def _cells(ref_root):
    path = os.path.join(ref_root, "writing_and_wiki", "notebooks", "Resampling.ipynb")
    nb = json.load(open(path))
    cells = nb["worksheets"][0]["cells"] if "worksheets" in nb else nb["cells"]
    code = [c for c in cells if c["cell_type"] == "code"]
    src = lambda c: "".join(c.get("input", c.get("source", "")))  # noqa: E731
    filt = next(src(c) for c in code if "AA = np.sinc" in src(c))
    degrid = next(src(c) for c in code if "interpolated_value / norm_value" in src(c))
    return filt, degrid


def _points(rng, n, lo, hi, os_):
    out = []
    while len(out) < n:
        u = rng.uniform(lo, hi)
        f = u - np.floor(u)
        off = (1 - u + round(u)) * os_
        if abs(f - 0.5) > 1e-3 and 1e-3 < off - np.floor(off) < 1 - 1e-3:
            out.append(u)
    return np.array(out)


def main(ref_root):
    filt_src, degrid_src = _cells(ref_root)
    npx = types.ModuleType("numpy_notebook")
    npx.__dict__.update(np.__dict__)
    npx.complex = complex
    ns = {"np": npx, "plt": _NoPlot()}
    exec(filt_src, ns)
    support, os_ = ns["SUPPORT"], ns["OVERSAMPLE"]
    full = ns["FULL_SUPPORT"]
    aa = np.array(ns["AA"], dtype=np.float64)
    rng = np.random.default_rng(SEED)
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    # interior points: accepted by the notebook and by the library's footprint test
    lo, hi = support + 1.0, N - full - 3.0
    uv = np.stack([_points(rng, ROWS - EDGE_ROWS, lo, hi, os_), _points(rng, ROWS - EDGE_ROWS, lo, hi, os_)], 1)
    edge = np.stack([_points(rng, EDGE_ROWS, N - full - 1.0, N - 1.0, os_), _points(rng, EDGE_ROWS, lo, hi, os_)], 1)
    scaled_uv = np.concatenate([uv, edge])
    ns.update(ROW_COUNT=ROWS, scaled_uv=scaled_uv, model_regular=model, Nx=N, Ny=N, AA=_TruncIndex(aa))
    exec(degrid_src, ns)
    vis = np.asarray(ns["vis"], dtype=np.complex128)
    out = os.path.join(HERE, "notebook_degrid.npz")
    np.savez_compressed(out, model=model, scaled_uv=scaled_uv, aa=aa, vis=vis, support=support, oversample=os_,
                        interior_rows=ROWS - EDGE_ROWS)
    print("wrote", out, "rows", ROWS, "nonzero", int(np.count_nonzero(vis)))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BULLSEYE_REFERENCE")
    if not root:
        raise SystemExit(f"usage: {sys.argv[0]} <reference root> (or set BULLSEYE_REFERENCE)")
    main(root)
