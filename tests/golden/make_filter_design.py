"""Generate tests/golden/filter_design.npz by running the reference's filter-design study.

Runs the code cells of the reference's writing_and_wiki/notebooks/Filter design.ipynb that build
the three windowed-sinc filters and their aliasing-energy figures (cells 4, 5, 6, 8, 10, 12 and
13), and stores the filters, their responses and the figures.  The notebook is Python 2 code; the
stand-ins that let it run under Python 3 are: integer division where Python 2 divided integers
(``full_support/2`` and ``full_support*oversample/2``), ``np.trapz`` (renamed
``np.trapezoid`` in numpy 2), a no-op ``plt``, and cell 13's print statements dropped (its three
figures are read from the namespace).

Usage: python tests/golden/make_filter_design.py [path to the reference checkout]
"""
from __future__ import annotations

import json
import os
import sys
import types

import numpy as np
from scipy import signal as sg
from scipy import special as sp

HERE = os.path.dirname(os.path.abspath(__file__))


class _NoPlot:
    def __getattr__(self, name):
        return lambda *a, **k: None


def _py2(src: str) -> str:
    return src.replace("full_support*oversample/2", "full_support*oversample//2").replace(
        "full_support/2", "full_support//2")


def main(ref_root):
    path = os.path.join(ref_root, "writing_and_wiki", "notebooks", "Filter design.ipynb")
    nb = json.load(open(path))
    cells = nb["worksheets"][0]["cells"] if "worksheets" in nb else nb["cells"]
    code = ["".join(c.get("input", c.get("source", ""))) for c in cells if c["cell_type"] == "code"]
    npx = types.ModuleType("numpy_notebook")
    npx.__dict__.update(np.__dict__)
    npx.trapz = np.trapezoid
    ns = {"np": npx, "plt": _NoPlot(), "sp": sp, "sg": sg}
    # code[0] is the import cell; code[1..6] are cells 4, 5, 6, 8, 10, 12; code[7] is cell 13
    for src in code[1:7]:
        exec(_py2(src), ns)
    exec("\n".join(line for line in code[7].splitlines() if not line.lstrip().startswith("print")), ns)
    out = os.path.join(HERE, "filter_design.npz")
    np.savez_compressed(out, full_support=ns["full_support"], oversample=ns["oversample"], beta=ns["beta"], x=ns["x"],
                        sinc=ns["sinc"], sinc_hamming=ns["sinc_hamming"], kb=ns["kb"], fft_sinc=ns["fft_sinc"],
                        fft_sinc_hamming=ns["fft_sinc_hamming"], fft_kb=ns["fft_kb"],
                        aliasing=np.array([ns["aSinc"], ns["aHammingSinc"], ns["aKBSinc"]]))
    print("wrote", out, "aliasing % (sinc, hamming, kb):", ns["aSinc"], ns["aHammingSinc"], ns["aKBSinc"])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BULLSEYE_REFERENCE")
    if not root:
        raise SystemExit(f"usage: {sys.argv[0]} <reference root> (or set BULLSEYE_REFERENCE)")
    main(root)
