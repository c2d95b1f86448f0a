"""Pin the restated prototype degridder to the output of the reference notebook itself.

tests/golden/notebook_degrid.npz holds what cells 16 and 17 of the reference's
writing_and_wiki/notebooks/Resampling.ipynb compute, run as written on seeded inputs
(tests/golden/make_notebook_degrid.py).  The restatement in oracle/notebook_degridder.py must
reproduce the filter exactly and the degridded values to FP64 rounding; the GPU adjoint is then
checked against the same fixture (tests/test_gpu_adjoint.py).
"""
import os

import numpy as np

from oracle.notebook_degridder import notebook_degrid, notebook_filter

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    return np.load(os.path.join(HERE, "golden", "notebook_degrid.npz"))


def test_filter_matches_notebook():
    d = _fixture()
    aa = notebook_filter(int(d["support"]), int(d["oversample"]))
    assert aa.shape == d["aa"].shape
    assert np.array_equal(aa, d["aa"])


def test_degridder_matches_notebook():
    d = _fixture()
    vis, norms = notebook_degrid(d["model"], d["scaled_uv"], d["aa"], int(d["support"]), int(d["oversample"]))
    ref = d["vis"]
    assert np.max(np.abs(vis - ref)) <= 1e-13 * np.max(np.abs(ref))
    # the edge rows are skipped by the notebook's acceptance test
    n_in = int(d["interior_rows"])
    assert np.all(ref[n_in:] == 0) and np.all(norms[n_in:] == 0)
    assert np.all(norms[:n_in] > 0)
