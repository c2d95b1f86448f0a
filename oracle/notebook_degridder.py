"""Restatement of the reference's prototype degridder.  TEST INFRASTRUCTURE ONLY.

The reference ships one degridder: the prototype in writing_and_wiki/notebooks/Resampling.ipynb.
Cell 16 builds its anti-aliasing filter, cell 17 degrids a regular (model) uv grid onto the
measured uv points.  Only tests import this module; it is pinned against
tests/golden/notebook_degrid.npz, which tests/golden/make_notebook_degrid.py generated by running
those two notebook cells themselves.

Conventions of the notebook (kept here):

* ``scaled_uv`` is in pixels with the grid centre at N/2 (cell 13);
* the footprint's centre cell is ``round(u)``, its first cell ``round(u) - SUPPORT``;
* the filter index is ``conv * OVERSAMPLE + (1 - u + round(u)) * OVERSAMPLE`` truncated (a
  float index, which the numpy of the notebook's time truncated);
* a point is skipped (value 0) when ``round(u) + FULL_SUPPORT >= N`` or ``round(u) < 0``;
* the grid is indexed ``model[u_cell, v_cell]``;
* the value is the tap-weighted sum divided by the sum of the taps.
"""
from __future__ import annotations

import numpy as np


def notebook_filter(support: int, oversample: int) -> np.ndarray:
    """Cell 16: sinc(x / OVERSAMPLE) sampled on the padded, oversampled support."""
    full = 2 * support + 1
    padded = full + 2
    size = padded + (padded - 1) * (oversample - 1)
    centre = size // 2
    x = np.arange(-centre, centre + 1)
    return np.sinc(x / float(oversample))


def notebook_degrid(model: np.ndarray, scaled_uv: np.ndarray, aa: np.ndarray, support: int, oversample: int):
    """Cell 17: (values, tap sums) of the degridded points; skipped points give (0, 0)."""
    nx, ny = model.shape
    full = 2 * support + 1
    rows = scaled_uv.shape[0]
    vis = np.zeros(rows, np.complex128)
    norms = np.zeros(rows)
    for r in range(rows):
        u, v = float(scaled_uv[r, 0]), float(scaled_uv[r, 1])
        du, dv = int(round(u)), int(round(v))
        fu = (1 - u + du) * oversample
        fv = (1 - v + dv) * oversample
        if dv + full >= ny or du + full >= nx or dv < 0 or du < 0:
            continue
        tu = aa[(np.arange(full) * oversample + fu).astype(np.int64)]
        tv = aa[(np.arange(full) * oversample + fv).astype(np.int64)]
        w = np.outer(tu, tv)  # [conv_u, conv_v]
        cu = du - support + np.arange(full)
        cv = dv - support + np.arange(full)
        block = model[np.ix_(cu, cv)]  # negative cells wrap, as numpy indexing does in the notebook
        vis[r] = np.sum(block * w) / np.sum(w)
        norms[r] = np.sum(w)
    return vis, norms
